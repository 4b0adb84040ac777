// Drop-in GridCount2d (reference: include/gridCount2d.h:23-48).
//
// update() sorts the points into cells (Morton-ordered cells, points inside a
// cell by their previous index) and permutes the caller's arrays in place, as
// the reference does; d_ind is the permutation.  apply_f_frnn<Functor> stays a
// header template (a functor cannot cross a C ABI): it launches the caller's
// functor as f(i, j, pos[j] - pos[i], sqrt(r2)) for every sorted pair with
// r2 = dot(d, d) <= rad^2, including i == j like the reference.  Compile the
// calling translation unit with nvcc.
#pragma once

#include "../mcl_gb300.h"
#include "Host_Triangulation.h"

#ifdef __CUDACC__
namespace mcleap_detail {
__device__ inline unsigned spread16(unsigned w) {
  w &= 0xffff;
  w = (w | (w << 8)) & 0x00FF00FFu;
  w = (w | (w << 4)) & 0x0F0F0F0Fu;
  w = (w | (w << 2)) & 0x33333333u;
  w = (w | (w << 1)) & 0x55555555u;
  return w;
}
__device__ inline int cell_coord(float p, float mn, float c, int n, int periodic) {
  float kf = floorf(__fdiv_rn(__fsub_rn(p, mn), c));
  kf = fminf(fmaxf(kf, -1.0e9f), 1.0e9f);
  int k = (int)kf;
  if (periodic) {
    k %= n;
    if (k < 0) k += n;
  } else {
    k = k < 0 ? 0 : (k >= n ? n - 1 : k);
  }
  return k;
}
template <class Functor>
__global__ void apply_f_frnn_kernel(Functor f, int n, const glm::vec2* pos, mcl_grid_desc g, float rad2, int w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const glm::vec2 pi = pos[i];
  const int x0 = cell_coord(pi.x, g.min_x, g.cell_x, g.cells_x, g.periodic);
  const int y0 = cell_coord(pi.y, g.min_y, g.cell_y, g.cells_y, g.periodic);
  for (int oy = -w; oy <= w; ++oy) {
    int y = y0 + oy;
    if (g.periodic) { y %= g.cells_y; if (y < 0) y += g.cells_y; }
    else if (y < 0 || y >= g.cells_y) continue;
    for (int ox = -w; ox <= w; ++ox) {
      int x = x0 + ox;
      if (g.periodic) { x %= g.cells_x; if (x < 0) x += g.cells_x; }
      else if (x < 0 || x >= g.cells_x) continue;
      const int c = g.morton ? (int)(spread16((unsigned)x) | (spread16((unsigned)y) << 1)) : y * g.cells_x + x;
      const int b = g.cell_start_dev[c], k = g.cell_count_dev[c];
      for (int j = b; j < b + k; ++j) {
        const glm::vec2 d = pos[j] - pi;
        const float r2 = __fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y));
        if (r2 <= rad2) f(i, j, d, sqrt((double)r2));
      }
    }
  }
}
}  // namespace mcleap_detail
#endif

struct GridCount2d {
  int numP;
  int blocksize = 64;
  mcl_grid* grid = nullptr;
  const int* d_ind = nullptr;

  GridCount2d(int numP_, glm::vec2 min, glm::vec2 cell_size, glm::ivec2 num_cells) : numP(numP_) {
    mcleap_detail::check(mcl_grid_create(numP, min.x, min.y, cell_size.x, cell_size.y, num_cells.x, num_cells.y, 0,
                                         &grid));
    refresh();
  }
  ~GridCount2d() { mcl_grid_destroy(grid); }
  GridCount2d(const GridCount2d&) = delete;
  GridCount2d& operator=(const GridCount2d&) = delete;

  void update(glm::vec2* pos) { update(pos, nullptr); }
  void update(glm::vec2* pos, glm::vec2* vel) {
    mcleap_detail::check(
        mcl_grid_update(grid, reinterpret_cast<mcl_float2*>(pos), reinterpret_cast<mcl_float2*>(vel), nullptr));
    refresh();
  }

#ifdef __CUDACC__
  template <class Functor>
  void apply_f_frnn(Functor& f, glm::vec2* pos, const float rad) {
    mcl_grid_desc g;
    mcleap_detail::check(mcl_grid_describe(grid, &g));
    const float w1 = rad / g.cell_x, w2 = rad / g.cell_y;
    int w = (int)ceilf(w1 > w2 ? w1 : w2);
    if (w < 1) w = 1;
    mcleap_detail::apply_f_frnn_kernel<Functor><<<(numP + 127) / 128, 128>>>(f, numP, pos, g, rad * rad, w);
  }
#endif

  float mean_num_particle_in_cell() {
    float m = 0.f;
    mcleap_detail::check(mcl_grid_mean_occupancy(grid, &m));
    return m;
  }

 private:
  void refresh() {
    const int32_t* perm = nullptr;
    mcl_grid_tables(grid, &perm, nullptr, nullptr, nullptr, nullptr);
    d_ind = perm;
  }
};
