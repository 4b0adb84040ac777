// Neighbourhood queries on the device mesh and the uniform grid, plus the
// predicate diagnostics entry points.
//
//   one-ring      DeviceTriangulation::oneRing / oneRing2   (include/kernels.cuh:54-121)
//   closest       DeviceTriangulation::closestNeighbors[2]  (include/kernels.cuh:129-165)
//   mesh FRNN     DeviceTriangulation::getFRNN / getFRNN2   (include/kernels.cuh:169-272)
//   grid          GridCount2d (include/gridCount2d.h): counting sort of points
//                 into row-major cells, stable inside a cell,
//                 then fixed-radius queries over the (2w+1)^2 cell stencil.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.cuh"

using namespace mcl;

namespace {

int qfail(int code, const std::string& msg) {
  mcl_set_last_error(msg);
  return code;
}

#define QCK(call)                                                                       \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess) return qfail(MCL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Reference squared distance, include/kernels.cuh:125-127: no FMA contraction.
__device__ __forceinline__ float sqdist(float2 a, float2 b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y);
  return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

struct MeshView {
  const int4* ev;
  const int4* en;
  const int* vhe;
  const float2* pos;
  int V, E;
};

__device__ __forceinline__ int mv_origin(const MeshView& M, int h) {
  return __ldg(reinterpret_cast<const int*>(M.ev) + 4 * (h >> 1) + (h & 1));
}
__device__ __forceinline__ int mv_next(const MeshView& M, int h) {
  return __ldg(reinterpret_cast<const int*>(M.en) + 4 * (h >> 1) + 2 * (h & 1));
}
// The reference's PREV_OUTGOING(h) = next(twin(h)): the next outgoing half-edge
// clockwise around the origin (include/kernels.cuh:52).
__device__ __forceinline__ int mv_rot(const MeshView& M, int h) { return mv_next(M, h ^ 1); }

constexpr int kMaxDeg = 4096;

// ---------------------------------------------------------------------------
// Rings of up to kRegRing spokes are walked once and kept in shared memory,
// then written starting at the spoke to the smallest neighbour; longer rings
// walk twice.  (A register array indexed through unrolled compare-and-select
// chains made the kernel instruction-bound: 71 % SM throughput at 53 us for
// 1M vertices.)
constexpr int kRegRing = 16;
constexpr int kRingThreads = 256;

__global__ void __launch_bounds__(kRingThreads) k_one_ring(MeshView M, int layout, int max_ring, int* ring,
                                                  unsigned long long* truncated) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.V) return;
  const int h0 = __ldg(M.vhe + i);
  if (h0 < 0) return;
  const int cap = max_ring - 1;
  const size_t stride = layout == MCL_LAYOUT_COLUMN ? (size_t)M.V : 1;
  int* row = layout == MCL_LAYOUT_COLUMN ? ring + i : ring + (size_t)i * max_ring;
  // the first kRegRing neighbours in walk order, one column per thread
  // (conflict-free), rotated to start at the smallest when written out
  __shared__ int sring[kRegRing][kRingThreads];
  int start = h0, best = 0x7fffffff, deg = 0, at = 0;
  int h = h0;
  do {
    const int w = mv_origin(M, h ^ 1);
    if (w < best) { best = w; start = h; at = deg; }
    if (deg < kRegRing) sring[deg][threadIdx.x] = w;
    h = mv_rot(M, h);
    ++deg;
  } while (h != h0 && deg < kMaxDeg);
  if (deg <= kRegRing && deg <= cap) {
    int src = at;
    for (int k = 0; k < deg; ++k) {
      row[(size_t)(k + 1) * stride] = sring[src][threadIdx.x];
      if (++src == deg) src = 0;
    }
    row[0] = deg;
    return;
  }
  const int cnt = deg < cap ? deg : cap;
  h = start;
  for (int k = 0; k < cnt; ++k) {
    row[(size_t)(k + 1) * stride] = mv_origin(M, h ^ 1);
    h = mv_rot(M, h);
  }
  row[0] = cnt;
  if (deg > cap) atomicAdd(truncated, 1ull);
}

__global__ void k_closest(const float2* pos, int V, int layout, int max_ring, const int* ring, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const int cnt = layout == MCL_LAYOUT_COLUMN ? ring[i] : ring[(size_t)i * max_ring];
  const float2 p = pos[i];
  int best = -1;
  float bd = 0.f;
  for (int k = 0; k < cnt; ++k) {
    const int j = layout == MCL_LAYOUT_COLUMN ? ring[(size_t)(k + 1) * V + i] : ring[(size_t)i * max_ring + k + 1];
    const float d = sqdist(p, pos[j]);
    if (best < 0 || d < bd || (d == bd && j < best)) { best = j; bd = d; }
  }
  out[i] = best;
}

// Mesh FRNN: depth-first search over the mesh from i through vertices within r
// (the reference's getFRNN, include/Host_Triangulation.h:525-560 and
// include/kernels.cuh:169-219).  The found set is kept in a thread-local list,
// then written sorted ascending.
constexpr int kFrnnLocal = 256;

// With rcomp != nullptr the radius of vertex i is rcomp[vcomp[i]] (one radius
// per mesh of a batch; a plain mesh has vcomp == nullptr and one radius).
__global__ void k_mesh_frnn(MeshView M, float r2, int layout, int max_frnn, int* out, unsigned long long* overflow,
                            const float* rcomp, const int* vcomp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.V) return;
  if (rcomp) {
    const float rc = rcomp[vcomp ? vcomp[i] : 0];
    r2 = __fmul_rn(rc, rc);
  }
  int found[kFrnnLocal];
  int nf = 0;
  int top = 0;  // stack = found[top..nf): vertices whose rings are still to scan
  bool over = false;
  const float2 pi = M.pos[i];
  int cur = i;
  for (int guard = 0; guard < (1 << 20); ++guard) {
    const int h0 = __ldg(M.vhe + cur);
    if (h0 >= 0) {
      int h = h0, deg = 0;
      do {
        const int w = mv_origin(M, h ^ 1);
        if (w != i) {
          bool seen = false;
          for (int k = 0; k < nf; ++k)
            if (found[k] == w) { seen = true; break; }
          if (!seen && sqdist(pi, M.pos[w]) <= r2) {
            if (nf < kFrnnLocal) found[nf++] = w;
            else over = true;
          }
        }
        h = mv_rot(M, h);
        ++deg;
      } while (h != h0 && deg < kMaxDeg);
    }
    if (top >= nf) break;
    cur = found[top++];
  }
  // insertion sort
  for (int a = 1; a < nf; ++a) {
    const int x = found[a];
    int b = a - 1;
    while (b >= 0 && found[b] > x) { found[b + 1] = found[b]; --b; }
    found[b + 1] = x;
  }
  const int cap = max_frnn - 1;
  const int cnt = nf < cap ? nf : cap;
  for (int k = 0; k < cnt; ++k) {
    if (layout == MCL_LAYOUT_COLUMN) out[(size_t)(k + 1) * M.V + i] = found[k];
    else out[(size_t)i * max_frnn + k + 1] = found[k];
  }
  if (layout == MCL_LAYOUT_COLUMN) out[i] = cnt;
  else out[(size_t)i * max_frnn] = cnt;
  if (over || nf > cap) atomicAdd(overflow, 1ull);
}

// Diffusion-limited aggregation contact (the reference's check_if_close_diffusion,
// experiments/diffusion_limited_aggregation.cu:51-60, over mesh FRNN
// neighbours): a free walker freezes when a vertex frozen before this call
// lies within its mesh's radius.  Decisions read frozen_in only, so the result
// does not depend on thread order.
__global__ void k_dla_freeze(MeshView M, ActV A, const unsigned char* vfix, const float* rcomp, const int* vcomp,
                             const unsigned char* frozen_in, unsigned char* frozen_out,
                             unsigned long long* newly) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= A.V_it) return;
  const int i = A.at(ii);
  unsigned char f = frozen_in[i];
  if (!f && !vfix[i] && __ldg(M.vhe + i) >= 0) {
    const float rc = rcomp[vcomp ? vcomp[i] : 0];
    const float r2 = __fmul_rn(rc, rc);
    int found[kFrnnLocal];
    int nf = 0, top = 0;
    const float2 pi = M.pos[i];
    int cur = i;
    for (int guard = 0; guard < (1 << 20) && !f; ++guard) {
      const int h0 = __ldg(M.vhe + cur);
      if (h0 >= 0) {
        int h = h0, deg = 0;
        do {
          const int w = mv_origin(M, h ^ 1);
          if (w != i) {
            bool seen = false;
            for (int k = 0; k < nf; ++k)
              if (found[k] == w) { seen = true; break; }
            if (!seen && sqdist(pi, M.pos[w]) <= r2) {
              if (frozen_in[w]) { f = 1; break; }
              if (nf < kFrnnLocal) found[nf++] = w;
            }
          }
          h = mv_rot(M, h);
          ++deg;
        } while (h != h0 && deg < kMaxDeg);
      }
      if (f || top >= nf) break;
      cur = found[top++];
    }
    if (f) atomicAdd(newly, 1ull);
  }
  frozen_out[i] = f;
}

// frozen[i] |= fnew[i] over the same vertices (second half of an in-place call)
__global__ void k_dla_commit(ActV A, unsigned char* frozen, const unsigned char* fnew) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= A.V_it) return;
  const int i = A.at(ii);
  frozen[i] = fnew[i];
}

// Mesh FRNN / one-ring for a list of query vertices: row q is verts[q].
__global__ void k_mesh_frnn_list(MeshView M, const float* rcomp, const int* vcomp, const int* verts, int n, int layout,
                                 int max_frnn, int* out, unsigned long long* overflow) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = verts[q];
  const int cap = max_frnn - 1;
  int* row = layout == MCL_LAYOUT_COLUMN ? out + q : out + (size_t)q * max_frnn;
  const size_t stride = layout == MCL_LAYOUT_COLUMN ? (size_t)n : 1;
  if (i < 0 || i >= M.V || __ldg(M.vhe + i) < 0) {
    row[0] = 0;
    return;
  }
  const float rc = rcomp[vcomp ? vcomp[i] : 0];
  const float r2 = __fmul_rn(rc, rc);
  int found[kFrnnLocal];
  int nf = 0, top = 0;
  bool over = false;
  const float2 pi = M.pos[i];
  int cur = i;
  for (int guard = 0; guard < (1 << 20); ++guard) {
    const int h0 = __ldg(M.vhe + cur);
    if (h0 >= 0) {
      int h = h0, deg = 0;
      do {
        const int w = mv_origin(M, h ^ 1);
        if (w != i) {
          bool seen = false;
          for (int k = 0; k < nf; ++k)
            if (found[k] == w) { seen = true; break; }
          if (!seen && sqdist(pi, M.pos[w]) <= r2) {
            if (nf < kFrnnLocal) found[nf++] = w;
            else over = true;
          }
        }
        h = mv_rot(M, h);
        ++deg;
      } while (h != h0 && deg < kMaxDeg);
    }
    if (top >= nf) break;
    cur = found[top++];
  }
  for (int a = 1; a < nf; ++a) {
    const int x = found[a];
    int b = a - 1;
    while (b >= 0 && found[b] > x) { found[b + 1] = found[b]; --b; }
    found[b + 1] = x;
  }
  const int cnt = nf < cap ? nf : cap;
  for (int k = 0; k < cnt; ++k) row[(size_t)(k + 1) * stride] = found[k];
  row[0] = cnt;
  if (over || nf > cap) atomicAdd(overflow, 1ull);
}

__global__ void k_one_ring_list(MeshView M, const int* verts, int n, int layout, int max_ring, int* out,
                                unsigned long long* truncated) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = verts[q];
  int* row = layout == MCL_LAYOUT_COLUMN ? out + q : out + (size_t)q * max_ring;
  const size_t stride = layout == MCL_LAYOUT_COLUMN ? (size_t)n : 1;
  const int h0 = (i >= 0 && i < M.V) ? __ldg(M.vhe + i) : -1;
  if (h0 < 0) {
    row[0] = 0;
    return;
  }
  int start = h0, best = 0x7fffffff, deg = 0, h = h0;
  do {
    const int w = mv_origin(M, h ^ 1);
    if (w < best) { best = w; start = h; }
    h = mv_rot(M, h);
    ++deg;
  } while (h != h0 && deg < kMaxDeg);
  const int cap = max_ring - 1;
  const int cnt = deg < cap ? deg : cap;
  h = start;
  for (int k = 0; k < cnt; ++k) {
    row[(size_t)(k + 1) * stride] = mv_origin(M, h ^ 1);
    h = mv_rot(M, h);
  }
  row[0] = cnt;
  if (deg > cap) atomicAdd(truncated, 1ull);
}

}  // namespace

// ---------------------------------------------------------------------------
// Grid.
struct mcl_grid {
  int64_t n;
  float minx, miny, cx, cy;
  int nx, ny;
  int flags;
  int morton;           // cells numbered along a Morton curve (else row-major)
  int mbits;            // Morton side = 1 << mbits
  int64_t ncells;       // size of the cell tables
  int* cell;            // per point: cell id (input order)
  int* count;           // per cell
  int* start;           // per cell
  int* cursor;          // per cell scatter cursor
  int* perm;            // d_ind: sorted slot of input point i
  int* src;             // per sorted slot: input index
  float2* tmp;          // sorted positions / velocities scratch
  float2* tmp2;
  void* scan_tmp;
  size_t scan_tmp_bytes;
  int built;            // mcl_grid_build ran: tmp holds the sorted copy
};

namespace {

struct GridView {
  float minx, miny, cx, cy;
  int nx, ny, morton, periodic;
};

__device__ __forceinline__ int cell_coord(float p, float mn, float c, int n, int periodic, int* outside = nullptr) {
  float kf = floorf(__fdiv_rn(__fsub_rn(p, mn), c));
  kf = fminf(fmaxf(kf, -1.0e9f), 1.0e9f);  // also maps NaN to a border cell
  int k = (int)kf;
  if (outside && (k < 0 || k >= n)) *outside = 1;
  if (periodic) {
    k %= n;
    if (k < 0) k += n;
  } else {
    k = k < 0 ? 0 : (k >= n ? n - 1 : k);
  }
  return k;
}

__device__ __forceinline__ int cell_id(const GridView& G, int x, int y) {
  return y * G.nx + x;
}

// outside (may be NULL): set when a point's cell coordinate lies outside the
// grid before wrapping or clamping (the point is outside the domain).
__global__ void k_grid_hash(GridView G, int n, const float2* pos, int* cell, int* count, int* outside = nullptr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 p = pos[i];
  int out = 0;
  const int c = cell_id(G, cell_coord(p.x, G.minx, G.cx, G.nx, G.periodic, &out),
                        cell_coord(p.y, G.miny, G.cy, G.ny, G.periodic, &out));
  cell[i] = c;
  atomicAdd(count + c, 1);
  if (out && outside) atomicOr(outside, 1);
}

// Exclusive scan of the cell counts, single-pass per block + block offsets.
__global__ void k_scan_blocks(const int* in, int* out, int* block_sums, int64_t n) {
  __shared__ int s[1024];
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  const int x = i < n ? in[i] : 0;
  s[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int y = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - x;
  if (threadIdx.x == 1023) block_sums[blockIdx.x] = s[1023];
}

__global__ void k_scan_add(int* out, const int* block_prefix, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += block_prefix[blockIdx.x];
}

__global__ void k_grid_scatter(int n, const int* cell, int* cursor, int* perm, int* src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int slot = atomicAdd(cursor + cell[i], 1);
  perm[i] = slot;
  src[slot] = i;
}

// Make the order inside each cell stable (ascending input index).
__global__ void k_grid_sort_cells(int64_t ncells, const int* start, const int* count, int* src, int* perm) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int b = start[c], k = count[c];
  for (int a = b + 1; a < b + k; ++a) {
    const int x = src[a];
    int j = a - 1;
    while (j >= b && src[j] > x) { src[j + 1] = src[j]; --j; }
    src[j + 1] = x;
  }
  for (int a = b; a < b + k; ++a) perm[src[a]] = a;
}

__global__ void k_gather(int n, const int* src, const float2* in, float2* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[src[i]];
}

// Fixed-radius query, one thread per sorted slot i (threads of a warp are
// neighbouring points of one cell row, so their candidates overlap in L1).
// Cells are row-major, so each stencil row is one contiguous range of sorted
// points (up to three with periodic wrap).  The stencil is the disk: for each
// cell row the x extent comes from the query's own position and the row's
// vertical distance, widened by a margin far above float rounding; cells it
// skips hold no point within r, so the result and its order equal the full
// (2w+1)^2 stencil's: rows bottom to top, cells left to right in stencil
// order, points of a cell in sorted order (the reference's SaveNeighborsFunctor
// order, gridCount2d.h:263-296).  Distances use the reference formula
// fl(fl(dx*dx) + fl(dy*dy)) <= fl(r*r) without FMA; periodic grids take the
// minimum image (|d| > L/2 -> d -= copysign(L, d)).  A candidate is tested
// without branches: its sorted index is written to the thread's shared row at
// slot nf and nf advances on a hit (a range takes this path only when the row
// has room for all of it).  Rows hold up to kStageCap ids and are flushed one
// warp per row (coalesced), ids and rows mapped through src when given;
// entries past kStageCap go straight to global memory.
constexpr int kStageCap = 48;
constexpr int kFrnnThreads = 128;

template <bool kPeriodic>
__global__ void __launch_bounds__(kFrnnThreads) k_grid_frnn(GridView G, int n, const float2* __restrict__ pos,
                                                           const int* __restrict__ start,
                                                           const int* __restrict__ count, float r, float Lx,
                                                           float Ly, int max_nb, int* __restrict__ counts,
                                                           int* __restrict__ ids, unsigned long long* overflow,
                                                           const int* __restrict__ src,
                                                           const int* __restrict__ outside, int wrap_by_segment) {
  __shared__ int stage[kFrnnThreads * (kStageCap + 1)];
  __shared__ int cnts[kFrnnThreads];
  const int t = threadIdx.x, row0 = blockIdx.x * kFrnnThreads, i = row0 + t;
  int* mine = stage + t * (kStageCap + 1);
  const int scap = max_nb < kStageCap ? max_nb : kStageCap;
  int nf = 0;
  const float r2 = __fmul_rn(r, r);
  // Minimum image by segment: with every point inside the domain and the
  // stencil well under half the domain (checked by the caller), a candidate's
  // |dx| exceeds half the domain exactly when its cell was reached across the
  // wrap, so the per-candidate test "|dx| > Lx/2: dx -= copysign(Lx, dx)" is
  // the constant shift of its row segment: dx + xs, with the same rounding.
  const bool seg = kPeriodic && wrap_by_segment && outside && __ldg(outside) == 0;
  if (i < n) {
    const float2 p = pos[i];
    const int row = src ? __ldg(src + i) : i;
    int* direct = ids + (size_t)row * max_nb;
    const float hx = 0.5f * Lx, hy = 0.5f * Ly;
    const float ix = 1.0f / G.cx, iy = 1.0f / G.cy;
    const float mx = 1e-3f * G.cx + 1e-5f * (fabsf(p.x) + fabsf(G.minx) + r);
    const float my = 1e-3f * G.cy + 1e-5f * (fabsf(p.y) + fabsf(G.miny) + r);
    const float px = p.x - G.minx, py = p.y - G.miny;
    int ylo = (int)floorf(fmaxf(fminf((py - r - my) * iy, 1e9f), -1e9f));
    int yhi = (int)floorf(fmaxf(fminf((py + r + my) * iy, 1e9f), -1e9f));
    if (!kPeriodic) {
      ylo = ylo < 0 ? 0 : (ylo >= G.ny ? G.ny - 1 : ylo);
      yhi = yhi < 0 ? 0 : (yhi >= G.ny ? G.ny - 1 : yhi);
    } else if (yhi - ylo + 1 > G.ny) {
      ylo = 0; yhi = G.ny - 1;  // the disk covers every row: visit each once
    }
    for (int yy = ylo; yy <= yhi; ++yy) {
      // vertical distance from p to the row's slab (0 inside), minus the margin;
      // without wrap the border rows also hold the points clamped into them,
      // so their slabs extend to infinity
      float slo = yy * G.cy, shi = slo + G.cy;
      if (!kPeriodic) {
        if (yy == 0) slo = -INFINITY;
        if (yy == G.ny - 1) shi = INFINITY;
      }
      const float dym = fmaxf(fmaxf(slo - py, py - shi) - my, 0.f);
      const float hw = (kPeriodic && yhi - ylo + 1 >= G.ny) ? r + mx : sqrtf(fmaxf(r2 - dym * dym, 0.f)) * 1.0001f + mx;
      int xlo = (int)floorf(fmaxf(fminf((px - hw) * ix, 1e9f), -1e9f));
      int xhi = (int)floorf(fmaxf(fminf((px + hw) * ix, 1e9f), -1e9f));
      int y = yy;
      float ys = 0.f;
      if (kPeriodic && seg) {
        if (y < 0) { y += G.ny; ys = Ly; }
        else if (y >= G.ny) { y -= G.ny; ys = -Ly; }
      } else if (kPeriodic) {
        y %= G.ny;
        if (y < 0) y += G.ny;
        if (xhi - xlo + 1 > G.nx) { xlo = 0; xhi = G.nx - 1; }
      } else {
        xlo = xlo < 0 ? 0 : (xlo >= G.nx ? G.nx - 1 : xlo);
        xhi = xhi < 0 ? 0 : (xhi >= G.nx ? G.nx - 1 : xhi);
      }
      const int base = y * G.nx;
#pragma unroll 1
      for (int sgi = 0; sgi < 2; ++sgi) {
        int sa, sb;
        float xs = 0.f;
        if (kPeriodic && seg) {
          // cells left of 0 are the row's end (+Lx), right of nx-1 its start (-Lx)
          const int s0 = xlo < 0 ? xlo + G.nx : xlo, last = s0 + (xhi - xlo);
          if (sgi == 0) { sa = s0; sb = last < G.nx ? last : G.nx - 1; xs = xlo < 0 ? Lx : 0.f; }
          else { if (last < G.nx) continue; sa = 0; sb = last - G.nx; xs = xlo < 0 ? 0.f : -Lx; }
        } else if (kPeriodic) {
          // [xlo, xhi] (at most nx cells) in stencil order: from the wrapped
          // start to the end of the row, then on from cell 0
          const int s0 = (xlo % G.nx + G.nx) % G.nx, last = s0 + (xhi - xlo);
          if (sgi == 0) { sa = s0; sb = last < G.nx ? last : G.nx - 1; }
          else if (sgi == 1) { if (last < G.nx) continue; sa = 0; sb = last - G.nx; }
          else continue;
        } else {
          if (sgi != 0) continue;
          sa = xlo; sb = xhi;
        }
        const int b = __ldg(start + base + sa);
        const int e = __ldg(start + base + sb) + __ldg(count + base + sb);
        if (seg && nf + (e - b) <= scap) {
#pragma unroll 4
          for (int j = b; j < e; ++j) {
            const float2 o = pos[j];
            const float dx = __fadd_rn(__fsub_rn(p.x, o.x), xs), dy = __fadd_rn(__fsub_rn(p.y, o.y), ys);
            const bool hit = (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2) & (j != i);
            mine[nf] = j;
            nf += hit ? 1 : 0;
          }
        } else if (nf + (e - b) <= scap) {
#pragma unroll 4
          for (int j = b; j < e; ++j) {
            const float2 o = pos[j];
            float dx = __fsub_rn(p.x, o.x), dy = __fsub_rn(p.y, o.y);
            if (kPeriodic) {
              dx = fabsf(dx) > hx ? __fsub_rn(dx, copysignf(Lx, dx)) : dx;
              dy = fabsf(dy) > hy ? __fsub_rn(dy, copysignf(Ly, dy)) : dy;
            }
            const bool hit = (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2) & (j != i);
            mine[nf] = j;
            nf += hit ? 1 : 0;
          }
        } else {
          for (int j = b; j < e; ++j) {
            const float2 o = pos[j];
            float dx = __fsub_rn(p.x, o.x), dy = __fsub_rn(p.y, o.y);
            if (kPeriodic) {
              dx = fabsf(dx) > hx ? __fsub_rn(dx, copysignf(Lx, dx)) : dx;
              dy = fabsf(dy) > hy ? __fsub_rn(dy, copysignf(Ly, dy)) : dy;
            }
            if ((__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2) & (j != i)) {
              if (nf < scap) mine[nf] = j;
              else if (nf < max_nb) direct[nf] = src ? __ldg(src + j) : j;
              ++nf;
            }
          }
        }
      }
    }
    counts[row] = nf < max_nb ? nf : max_nb;
    if (nf > max_nb) atomicAdd(overflow, 1ull);
  }
  cnts[t] = nf < scap ? nf : scap;
  __syncthreads();
  const int lane = t & 31;
  for (int rr = t >> 5; rr < kFrnnThreads && row0 + rr < n; rr += kFrnnThreads / 32) {
    const int cr = cnts[rr];
    const int row = src ? __ldg(src + row0 + rr) : row0 + rr;
    int* dst = ids + (size_t)row * max_nb;
    const int* from = stage + rr * (kStageCap + 1);
    for (int k = lane; k < cr; k += 32) dst[k] = src ? __ldg(src + from[k]) : from[k];
  }
}

// outside: the out-of-domain flag of the hashing of `pos` (NULL: unknown).
int launch_grid_frnn(const GridView& G, int n, const float2* pos, const int* start, const int* count, float r,
                     float Lx, float Ly, int max_nb, int* counts, int* ids, unsigned long long* ovf,
                     const int* src, cudaStream_t s, const int* outside) {
  const unsigned blocks = (unsigned)((n + kFrnnThreads - 1) / kFrnnThreads);
  // the minimum image by row segment is exact when every candidate cell lies
  // within 0.45 of the domain of the query point (stencil half-width + a
  // cell + the kernel's margins, with slack) and a row spans under nx cells
  auto fits = [&](float c, float L, int cells, float mn) {
    const double margin = 1e-3 * c + 1e-5 * (2.0 * std::fabs((double)mn) + L + r);
    return cells >= 20 && (1.0001 * r + margin + c) * 1.01 <= 0.45 * L;
  };
  const int by_segment = G.periodic && outside && fits(G.cx, Lx, G.nx, G.minx) && fits(G.cy, Ly, G.ny, G.miny);
  if (G.periodic)
    k_grid_frnn<true><<<blocks, kFrnnThreads, 0, s>>>(G, n, pos, start, count, r, Lx, Ly, max_nb, counts, ids, ovf, src,
                                                      outside, by_segment);
  else
    k_grid_frnn<false><<<blocks, kFrnnThreads, 0, s>>>(G, n, pos, start, count, r, Lx, Ly, max_nb, counts, ids, ovf,
                                                       src, outside, 0);
  QCK(cudaGetLastError());
  return MCL_OK;
}

__global__ void k_mean_occupancy(int64_t ncells, const int* count, unsigned long long* acc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int k = count[c];
  if (k > 0) {
    atomicAdd(acc, 1ull);
    atomicAdd(acc + 1, (unsigned long long)k);
  }
}

// Exclusive scan of up to a few hundred thousand ints in one block, entirely on
// the device (each thread scans a contiguous chunk, then the chunk totals).
__global__ void k_scan_one_block(const int* in, int* out, int64_t n) {
  __shared__ int tot[1024];
  const int64_t per = (n + blockDim.x - 1) / blockDim.x;
  const int64_t lo = threadIdx.x * per, hi = min(n, lo + per);
  int run = 0;
  for (int64_t i = lo; i < hi; ++i) run += in[i];
  tot[threadIdx.x] = run;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const int y = threadIdx.x >= (unsigned)o ? tot[threadIdx.x - o] : 0;
    __syncthreads();
    tot[threadIdx.x] += y;
    __syncthreads();
  }
  int acc = threadIdx.x ? tot[threadIdx.x - 1] : 0;
  for (int64_t i = lo; i < hi; ++i) {
    const int x = in[i];
    out[i] = acc;
    acc += x;
  }
}

// Exclusive scan of n ints, entirely on the device (no host round trip, so the
// grid build can sit inside a captured CUDA graph): per-block scans, one block
// scanning the block totals, then the block offsets added.  tmp holds nb ints
// and tmp2 nb ints, nb = ceil(n / 1024).
int scan_exclusive(const int* in, int* out, int64_t n, int* tmp, int* tmp2, cudaStream_t s) {
  const int64_t nb = (n + 1023) / 1024;
  k_scan_blocks<<<(unsigned)nb, 1024, 0, s>>>(in, out, tmp, n);
  if (nb > 1) {
    k_scan_one_block<<<1, 1024, 0, s>>>(tmp, tmp2, nb);
    k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(out, tmp2, n);
  }
  QCK(cudaGetLastError());
  return MCL_OK;
}

GridView view_of(const mcl_grid* g) {
  GridView G;
  G.minx = g->minx; G.miny = g->miny; G.cx = g->cx; G.cy = g->cy;
  G.nx = g->nx; G.ny = g->ny; G.morton = g->morton; G.periodic = (g->flags & MCL_GRID_PERIODIC) ? 1 : 0;
  return G;
}

}  // namespace

// ---------------------------------------------------------------------------
// Predicate diagnostics.
namespace {

struct StageCounters {
  unsigned long long orient_fp64, orient_exact, incircle_fp64, incircle_exact, sos;
};

__host__ __device__ inline int eval_pred(int kind, const float* q, const int* ids, int* stage) {
  StageCounters c = {0, 0, 0, 0, 0};
  int ovf = 0, s;
  if (kind == 0) {
    s = orient2d(q[0], q[1], q[2], q[3], q[4], q[5], &c, &ovf);
    *stage = c.orient_exact ? 2 : (c.orient_fp64 ? 1 : 0);
  } else if (kind == 1) {
    s = incircle(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], &c, &ovf);
    *stage = c.incircle_exact ? 2 : (c.incircle_fp64 ? 1 : 0);
  } else {
    s = incircle_sos(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], ids[0], ids[1], ids[2], ids[3], &c, &ovf);
    *stage = c.sos ? 3 : (c.incircle_exact ? 2 : (c.incircle_fp64 ? 1 : 0));
  }
  if (ovf) *stage = -1;
  return s;
}

__global__ void k_debug_pred(int kind, const float* pts, const int* ids, int64_t n, int* sign, int* stage) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int w = kind == 0 ? 6 : 8;
  int st = 0;
  const int s = eval_pred(kind, pts + w * i, ids ? ids + 4 * i : nullptr, &st);
  sign[i] = s;
  if (stage) stage[i] = st;
}

}  // namespace

extern "C" {

int mcl_debug_predicates_host(int kind, const float* pts, const int32_t* ids, int64_t n, int32_t* sign,
                              int32_t* stage) {
  if (!pts || !sign || kind < 0 || kind > 2 || (kind == 2 && !ids)) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  const int w = kind == 0 ? 6 : 8;
  for (int64_t i = 0; i < n; ++i) {
    int st = 0;
    sign[i] = eval_pred(kind, pts + w * i, ids ? ids + 4 * i : nullptr, &st);
    if (stage) stage[i] = st;
  }
  return MCL_OK;
}

int mcl_debug_predicates_device(int kind, const float* pts, const int32_t* ids, int64_t n, int32_t* sign,
                                int32_t* stage, void* stream) {
  if (!pts || !sign || kind < 0 || kind > 2 || (kind == 2 && !ids)) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  if (n == 0) return MCL_OK;
  k_debug_pred<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(kind, pts, ids, n, sign, stage);
  QCK(cudaGetLastError());
  return MCL_OK;
}

int mcl_one_ring(mcl_mesh* m, int layout, int max_ring, int32_t* ring, void* stream, int64_t* truncated) {
  if (!m || !ring || max_ring < 2 || (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* cnt = m->scratch;
  MeshView M{m->ev, m->en, m->vhe, m->pos[m->cur], (int)m->V, (int)m->E};
  QCK(cudaMemsetAsync(cnt, 0, 8, s));
  k_one_ring<<<(unsigned)((m->V + kRingThreads - 1) / kRingThreads), kRingThreads, 0, s>>>(M, layout, max_ring, ring,
                                                                                          cnt);
  QCK(cudaGetLastError());
  if (truncated) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, cnt, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *truncated = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_closest_neighbors(mcl_mesh* m, int layout, int max_ring, const int32_t* ring, int32_t* out, void* stream) {
  if (!m || !ring || !out || max_ring < 2) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  k_closest<<<(unsigned)((m->V + 255) / 256), 256, 0, (cudaStream_t)stream>>>(m->pos[m->cur], (int)m->V, layout,
                                                                              max_ring, ring, out);
  QCK(cudaGetLastError());
  return MCL_OK;
}

int mcl_mesh_frnn(mcl_mesh* m, float r, int layout, int max_frnn, int32_t* out, void* stream, int64_t* overflow) {
  if (!m || !out || max_frnn < 2 || !(r >= 0.f)) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* cnt = m->scratch;
  MeshView M{m->ev, m->en, m->vhe, m->pos[m->cur], (int)m->V, (int)m->E};
  QCK(cudaMemsetAsync(cnt, 0, 8, s));
  k_mesh_frnn<<<(unsigned)((m->V + 127) / 128), 128, 0, s>>>(M, r * r, layout, max_frnn, out, cnt, nullptr,
                                                               nullptr);
  QCK(cudaGetLastError());
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, cnt, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_batch_frnn(mcl_mesh* m, const float* r_dev, int layout, int max_frnn, int32_t* out, void* stream,
                   int64_t* overflow) {
  if (!m || !r_dev || !out || max_frnn < 2 || (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* cnt = m->scratch;
  MeshView M{m->ev, m->en, m->vhe, m->pos[m->cur], (int)m->V, (int)m->E};
  QCK(cudaMemsetAsync(cnt, 0, 8, s));
  k_mesh_frnn<<<(unsigned)((m->V + 127) / 128), 128, 0, s>>>(M, 0.f, layout, max_frnn, out, cnt, r_dev, m->vcomp);
  QCK(cudaGetLastError());
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, cnt, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_batch_frnn_list(mcl_mesh* m, const float* r_dev, const int32_t* verts_dev, int64_t n, int layout,
                        int max_frnn, int32_t* out_dev, void* stream, int64_t* overflow) {
  if (!m || !r_dev || (n > 0 && (!verts_dev || !out_dev)) || n < 0 || max_frnn < 2 ||
      (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* cnt = m->scratch + 2;
  QCK(cudaMemsetAsync(cnt, 0, 8, s));
  if (n > 0) {
    MeshView M{m->ev, m->en, m->vhe, m->pos[m->cur], (int)m->V, (int)m->E};
    k_mesh_frnn_list<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(M, r_dev, m->vcomp, verts_dev, (int)n, layout,
                                                                 max_frnn, out_dev, cnt);
    QCK(cudaGetLastError());
  }
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, cnt, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_one_ring_list(mcl_mesh* m, const int32_t* verts_dev, int64_t n, int layout, int max_ring, int32_t* out_dev,
                      void* stream, int64_t* truncated) {
  if (!m || (n > 0 && (!verts_dev || !out_dev)) || n < 0 || max_ring < 2 ||
      (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* cnt = m->scratch + 3;
  QCK(cudaMemsetAsync(cnt, 0, 8, s));
  if (n > 0) {
    MeshView M{m->ev, m->en, m->vhe, m->pos[m->cur], (int)m->V, (int)m->E};
    k_one_ring_list<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M, verts_dev, (int)n, layout, max_ring, out_dev, cnt);
    QCK(cudaGetLastError());
  }
  if (truncated) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, cnt, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *truncated = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_dla_freeze(mcl_mesh* m, const float* r_dev, uint8_t* frozen, void* stream, int64_t* newly_frozen) {
  if (!m || !r_dev || !frozen) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  if (!m->fnew && cudaMalloc((void**)&m->fnew, m->V) != cudaSuccess)
    return qfail(MCL_ERR_OUT_OF_MEMORY, "mcl_dla_freeze: scratch");
  unsigned long long* cnt = m->scratch + 1;
  MeshView M{m->ev, m->en, m->vhe, m->pos[m->cur], (int)m->V, (int)m->E};
  const ActV A = act_of(m);
  QCK(cudaMemsetAsync(cnt, 0, 8, s));
  if (A.V_it > 0) {
    k_dla_freeze<<<(unsigned)((A.V_it + 127) / 128), 128, 0, s>>>(M, A, m->vfix, r_dev, m->vcomp, frozen, m->fnew, cnt);
    k_dla_commit<<<(unsigned)((A.V_it + 255) / 256), 256, 0, s>>>(A, frozen, m->fnew);
  }
  QCK(cudaGetLastError());
  if (newly_frozen) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, cnt, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *newly_frozen = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_grid_create(int64_t n, float minx, float miny, float cx, float cy, int32_t nx, int32_t ny, int flags,
                    mcl_grid** out) {
  if (!out || n < 0 || nx < 1 || ny < 1 || !(cx > 0.f) || !(cy > 0.f) || (int64_t)nx * ny > (1ll << 30))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad grid");
  mcl_grid* g = new mcl_grid();
  std::memset(g, 0, sizeof(*g));
  g->n = n; g->minx = minx; g->miny = miny; g->cx = cx; g->cy = cy; g->nx = nx; g->ny = ny; g->flags = flags;
  int side = 1, bits = 0;
  while (side < std::max(nx, ny)) { side <<= 1; ++bits; }
  const int64_t mcells = (int64_t)side * side;
  g->morton = 0;  // row-major: a stencil row of cells is one contiguous range of sorted points
  g->mbits = bits;
  g->ncells = g->morton ? mcells : (int64_t)nx * ny;
  const int64_t nn = std::max<int64_t>(n, 1);
  const int64_t nb = (g->ncells + 1023) / 1024 + 1;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t b) { if (e == cudaSuccess) e = cudaMalloc(p, b); };
  A((void**)&g->cell, 4 * nn);
  A((void**)&g->count, 4 * (g->ncells + 1));  // + the out-of-domain flag of the last build
  A((void**)&g->start, 4 * g->ncells);
  A((void**)&g->cursor, 4 * g->ncells);
  A((void**)&g->perm, 4 * nn);
  A((void**)&g->src, 4 * nn);
  A((void**)&g->tmp, 8 * nn);
  A((void**)&g->tmp2, 8 * nn);
  A(&g->scan_tmp, 8 * nb);
  if (e == cudaSuccess) e = cudaMemset(g->count, 0, 4 * (g->ncells + 1));
  if (e == cudaSuccess) e = cudaMemset(g->start, 0, 4 * g->ncells);
  if (e != cudaSuccess) {
    mcl_grid_destroy(g);
    return qfail(MCL_ERR_OUT_OF_MEMORY, "grid allocation");
  }
  *out = g;
  return MCL_OK;
}

int mcl_grid_destroy(mcl_grid* g) {
  if (!g) return MCL_OK;
  void* ptrs[] = {g->cell, g->count, g->start, g->cursor, g->perm, g->src, g->tmp, g->tmp2, g->scan_tmp};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete g;
  return MCL_OK;
}

}  // extern "C"

namespace {
// Cell tables for the positions pos (input order) and their sorted copy in
// g->tmp; pos itself is not written.
int grid_build_tables(mcl_grid* g, const float2* pos, cudaStream_t s) {
  const int n = (int)g->n;
  const GridView G = view_of(g);
  QCK(cudaMemsetAsync(g->count, 0, 4 * (g->ncells + 1), s));
  k_grid_hash<<<(n + 255) / 256, 256, 0, s>>>(G, n, pos, g->cell, g->count, g->count + g->ncells);
  int* tmp = (int*)g->scan_tmp;
  const int64_t nb = (g->ncells + 1023) / 1024;
  int rc = scan_exclusive(g->count, g->start, g->ncells, tmp, tmp + nb + 1, s);
  if (rc != MCL_OK) return rc;
  QCK(cudaMemcpyAsync(g->cursor, g->start, 4 * g->ncells, cudaMemcpyDeviceToDevice, s));
  k_grid_scatter<<<(n + 255) / 256, 256, 0, s>>>(n, g->cell, g->cursor, g->perm, g->src);
  k_grid_sort_cells<<<(unsigned)((g->ncells + 255) / 256), 256, 0, s>>>(g->ncells, g->start, g->count, g->src,
                                                                         g->perm);
  k_gather<<<(n + 255) / 256, 256, 0, s>>>(n, g->src, pos, g->tmp);
  QCK(cudaGetLastError());
  return MCL_OK;
}
}  // namespace

extern "C" {

int mcl_grid_update(mcl_grid* g, mcl_float2* pos, mcl_float2* vel, void* stream) {
  if (!g || !pos) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)g->n;
  if (n == 0) return MCL_OK;
  const int rc = grid_build_tables(g, (const float2*)pos, s);
  if (rc != MCL_OK) return rc;
  QCK(cudaMemcpyAsync(pos, g->tmp, 8 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  if (vel) {
    k_gather<<<(n + 255) / 256, 256, 0, s>>>(n, g->src, (const float2*)vel, g->tmp2);
    QCK(cudaMemcpyAsync(vel, g->tmp2, 8 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  }
  QCK(cudaGetLastError());
  g->built = 1;
  return MCL_OK;
}

int mcl_grid_build(mcl_grid* g, const mcl_float2* pos, void* stream) {
  if (!g || !pos) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  if (g->n == 0) return MCL_OK;
  const int rc = grid_build_tables(g, (const float2*)pos, (cudaStream_t)stream);
  if (rc == MCL_OK) g->built = 1;
  return rc;
}

int mcl_grid_frnn_ids(mcl_grid* g, float r, int max_nb, int32_t* counts, int32_t* ids, void* stream,
                      int64_t* overflow) {
  if (!g || !counts || !ids || max_nb < 1 || !(r >= 0.f)) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  if (!g->built) return qfail(MCL_ERR_INVALID_ARGUMENT, "mcl_grid_frnn_ids: call mcl_grid_build first");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)g->n;
  if (n == 0) return MCL_OK;
  const GridView G = view_of(g);
  unsigned long long* ovf = (unsigned long long*)g->scan_tmp;
  QCK(cudaMemsetAsync(ovf, 0, 8, s));
  const int rc = launch_grid_frnn(G, n, g->tmp, g->start, g->count, r, g->cx * g->nx, g->cy * g->ny, max_nb, counts,
                                  ids, ovf, g->src, s, g->count + g->ncells);
  if (rc != MCL_OK) return rc;
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, ovf, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_grid_tables(mcl_grid* g, const int32_t** perm, const int32_t** start, const int32_t** count, int32_t* cx,
                    int32_t* cy) {
  if (!g) return qfail(MCL_ERR_INVALID_ARGUMENT, "null grid");
  if (perm) *perm = g->perm;
  if (start) *start = g->start;
  if (count) *count = g->count;
  if (cx) *cx = g->nx;
  if (cy) *cy = g->ny;
  return MCL_OK;
}

int mcl_grid_describe(mcl_grid* g, mcl_grid_desc* d) {
  if (!g || !d) return qfail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  d->min_x = g->minx; d->min_y = g->miny; d->cell_x = g->cx; d->cell_y = g->cy;
  d->cells_x = g->nx; d->cells_y = g->ny; d->morton = g->morton;
  d->periodic = (g->flags & MCL_GRID_PERIODIC) ? 1 : 0;
  d->table_size = g->ncells; d->num_points = g->n;
  d->perm_dev = g->perm; d->cell_start_dev = g->start; d->cell_count_dev = g->count;
  return MCL_OK;
}

int mcl_grid_frnn(mcl_grid* g, const mcl_float2* pos, float r, int max_nb, int32_t* counts, int32_t* ids, void* stream,
                  int64_t* overflow) {
  if (!g || !pos || !counts || !ids || max_nb < 1 || !(r >= 0.f)) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)g->n;
  if (n == 0) return MCL_OK;
  const GridView G = view_of(g);
  unsigned long long* ovf = (unsigned long long*)g->scan_tmp;
  QCK(cudaMemsetAsync(ovf, 0, 8, s));
  const int rc = launch_grid_frnn(G, n, (const float2*)pos, g->start, g->count, r, g->cx * g->nx, g->cy * g->ny,
                                  max_nb, counts, ids, ovf, nullptr, s, nullptr);
  if (rc != MCL_OK) return rc;
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, ovf, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

int mcl_grid_mean_occupancy(mcl_grid* g, float* mean) {
  if (!g || !mean) return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  unsigned long long* acc = (unsigned long long*)g->scan_tmp;
  QCK(cudaMemset(acc, 0, 16));
  k_mean_occupancy<<<(unsigned)((g->ncells + 255) / 256), 256>>>(g->ncells, g->count, acc);
  unsigned long long h[2];
  QCK(cudaMemcpy(h, acc, 16, cudaMemcpyDeviceToHost));
  *mean = h[0] ? (float)h[1] / (float)h[0] : 0.f;
  return MCL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batch FRNN over per-mesh grids (mcl_batch_frnn_grid): mesh c gets a uniform
// grid over [lo, hi)^2 with cells of its own radius (so the disk touches at
// most 3 x 3 cells), its cells numbered after those of the meshes before it;
// one counting sort orders every point of every mesh, then one query kernel
// answers every point with its own mesh's grid.  Same results as
// mcl_batch_frnn (rows ascending), without walking the mesh.
namespace {

__device__ __forceinline__ int bg_coord(float p, float lo, float c, int n) {
  float kf = floorf(__fdiv_rn(__fsub_rn(p, lo), c));
  kf = fminf(fmaxf(kf, -1.0e9f), 1.0e9f);
  const int k = (int)kf;
  return k < 0 ? 0 : (k >= n ? n - 1 : k);
}

__global__ void k_bgrid_hash(int V, const float2* pos, const unsigned char* vfix, const int* vcomp, const int4* par,
                             float lo, int* cell, int* count, int* out, int F) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  if (vfix[v]) {  // bounding corners hold no neighbour within any radius
    cell[v] = -1;
    out[(size_t)v * F] = 0;
    return;
  }
  const int4 q = par[vcomp ? vcomp[v] : 0];
  const float c = __int_as_float(q.x);
  const float2 p = pos[v];
  const int x = bg_coord(p.x, lo, c, q.y), y = bg_coord(p.y, lo, c, q.y);
  const int id = q.z + y * q.y + x;
  cell[v] = id;
  atomicAdd(count + id, 1);
}

__global__ void k_bgrid_scatter(int V, const int* cell, int* cursor, int* perm, int* src) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V || cell[v] < 0) return;
  const int slot = atomicAdd(cursor + cell[v], 1);
  perm[v] = slot;
  src[slot] = v;
}

// One thread per sorted slot (neighbouring points of one cell row of one
// mesh); disk-culled rows of the mesh's grid, branch-free candidate test,
// ids staged per thread in shared memory, sorted there and written out one row
// per warp step.  Rows: out[v*F] = count, out[v*F + 1 + k] ascending.
constexpr int kBStage = 48;

__global__ void __launch_bounds__(kFrnnThreads) k_bgrid_frnn(int n, const float2* __restrict__ spos,
                                                            const int* __restrict__ src, const int* __restrict__ vcomp,
                                                            const int4* __restrict__ par, const float* __restrict__ rc,
                                                            float lo, const int* __restrict__ start,
                                                            const int* __restrict__ count, int F, int* __restrict__ out,
                                                            unsigned long long* overflow) {
  __shared__ int stage[kFrnnThreads * (kBStage + 1)];
  __shared__ int cnts[kFrnnThreads];
  __shared__ int rows[kFrnnThreads];
  const int t = threadIdx.x, row0 = blockIdx.x * kFrnnThreads, i = row0 + t;
  int* mine = stage + t * (kBStage + 1);
  const int cap = F - 1;  // <= kBStage (checked by the host)
  int nf = 0;
  if (i < n) {
    const int v = __ldg(src + i);
    rows[t] = v;
    const int mesh = vcomp ? __ldg(vcomp + v) : 0;
    const int4 q = __ldg(par + mesh);
    const float c = __int_as_float(q.x), inv = 1.0f / c;
    const float r = __ldg(rc + mesh);
    const float r2 = __fmul_rn(r, r);
    const float2 p = spos[i];
    const int nx = q.y;
    const float mg = 1e-3f * c + 1e-5f * (fabsf(p.x) + fabsf(p.y) + fabsf(lo) + r);
    const float px = p.x - lo, py = p.y - lo;
    int ylo = (int)floorf(fmaxf(fminf((py - r - mg) * inv, 1e9f), -1e9f));
    int yhi = (int)floorf(fmaxf(fminf((py + r + mg) * inv, 1e9f), -1e9f));
    ylo = ylo < 0 ? 0 : (ylo >= nx ? nx - 1 : ylo);
    yhi = yhi < 0 ? 0 : (yhi >= nx ? nx - 1 : yhi);
    for (int yy = ylo; yy <= yhi; ++yy) {
      float slo = yy * c, shi = slo + c;
      if (yy == 0) slo = -INFINITY;
      if (yy == nx - 1) shi = INFINITY;
      const float dym = fmaxf(fmaxf(slo - py, py - shi) - mg, 0.f);
      const float hw = sqrtf(fmaxf(r2 - dym * dym, 0.f)) * 1.0001f + mg;
      int xlo = (int)floorf(fmaxf(fminf((px - hw) * inv, 1e9f), -1e9f));
      int xhi = (int)floorf(fmaxf(fminf((px + hw) * inv, 1e9f), -1e9f));
      xlo = xlo < 0 ? 0 : (xlo >= nx ? nx - 1 : xlo);
      xhi = xhi < 0 ? 0 : (xhi >= nx ? nx - 1 : xhi);
      const int base = q.z + yy * nx;
      const int b = __ldg(start + base + xlo);
      const int e = __ldg(start + base + xhi) + __ldg(count + base + xhi);
      if (nf + (e - b) <= cap) {
#pragma unroll 4
        for (int j = b; j < e; ++j) {
          const float2 o = spos[j];
          const float dx = __fsub_rn(p.x, o.x), dy = __fsub_rn(p.y, o.y);
          const bool hit = (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2) & (j != i);
          mine[nf] = j;
          nf += hit ? 1 : 0;
        }
      } else {
        for (int j = b; j < e; ++j) {
          const float2 o = spos[j];
          const float dx = __fsub_rn(p.x, o.x), dy = __fsub_rn(p.y, o.y);
          if ((__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2) & (j != i)) {
            if (nf < cap) mine[nf] = j;
            ++nf;
          }
        }
      }
    }
    if (nf > cap) atomicAdd(overflow, 1ull);
    const int m = nf < cap ? nf : cap;
    // vertex ids, ascending
    for (int a = 0; a < m; ++a) mine[a] = __ldg(src + mine[a]);
    for (int a = 1; a < m; ++a) {
      const int x = mine[a];
      int bb = a - 1;
      while (bb >= 0 && mine[bb] > x) { mine[bb + 1] = mine[bb]; --bb; }
      mine[bb + 1] = x;
    }
    nf = m;
  }
  cnts[t] = i < n ? nf : -1;
  __syncthreads();
  const int lane = t & 31;
  for (int rr = t >> 5; rr < kFrnnThreads && row0 + rr < n; rr += kFrnnThreads / 32) {
    const int cr = cnts[rr];
    int* dst = out + (size_t)rows[rr] * F;
    const int* from = stage + rr * (kBStage + 1);
    if (lane == 0) dst[0] = cr;
    for (int k = lane; k < cr; k += 32) dst[k + 1] = from[k];
  }
}

}  // namespace

extern "C" int mcl_batch_frnn_grid(mcl_mesh* m, const float* r_host, const float* r_dev, float lo, float hi,
                                   int max_frnn, int32_t* out_dev, void* stream, int64_t* overflow) {
  if (!m || !r_host || !r_dev || !out_dev || !(hi > lo) || max_frnn < 2)
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  if (max_frnn - 1 > kBStage) return qfail(MCL_ERR_CAPACITY, "mcl_batch_frnn_grid: max_frnn above 49");
  if (m->nact) return qfail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_frnn_grid: runs over every mesh of the batch");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nc = m->ncomp, V = m->V;
  // per-mesh grids: cells of the mesh's radius, at most 4096 per side
  std::vector<int4> par((size_t)nc);
  int64_t cells = 0;
  for (int64_t c = 0; c < nc; ++c) {
    const float r = r_host[c];
    if (!(r > 0.f)) return qfail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_frnn_grid: radius must be positive");
    int side = (int)std::min<double>(4096.0, std::ceil((double)(hi - lo) / r));
    side = std::max(side, 1);
    float cell = (hi - lo) / (float)side;
    if (cell < r) cell = r;  // a cell never narrower than the radius
    int v;
    std::memcpy(&v, &cell, 4);
    par[(size_t)c] = make_int4(v, side, (int)cells, 0);
    cells += (int64_t)side * side;
    if (cells > (1ll << 30)) return qfail(MCL_ERR_CAPACITY, "mcl_batch_frnn_grid: more than 2^30 cells");
  }
  if (!m->bg_cell) {
    auto A = [&](void** p, size_t b) { return cudaMalloc(p, b) == cudaSuccess; };
    if (!A((void**)&m->bg_cell, 4 * V) || !A((void**)&m->bg_src, 4 * V) || !A((void**)&m->bg_perm, 4 * V) ||
        !A((void**)&m->bg_pos, 8 * V) || !A((void**)&m->bg_par, sizeof(int4) * nc) ||
        cudaMallocHost((void**)&m->bg_par_host, sizeof(int4) * nc) != cudaSuccess)
      return qfail(MCL_ERR_OUT_OF_MEMORY, "mcl_batch_frnn_grid: point tables");
  }
  if (m->bg_cap < cells) {
    if (m->bg_count) { cudaFree(m->bg_count); cudaFree(m->bg_start); cudaFree(m->bg_cursor); cudaFree(m->bg_tmp); }
    m->bg_count = m->bg_start = m->bg_cursor = m->bg_tmp = nullptr;
    const int64_t nb = (cells + 1023) / 1024 + 1;
    if (cudaMalloc((void**)&m->bg_count, 4 * cells) != cudaSuccess ||
        cudaMalloc((void**)&m->bg_start, 4 * cells) != cudaSuccess ||
        cudaMalloc((void**)&m->bg_cursor, 4 * cells) != cudaSuccess ||
        cudaMalloc((void**)&m->bg_tmp, 8 * nb) != cudaSuccess) {
      m->bg_cap = 0;
      return qfail(MCL_ERR_OUT_OF_MEMORY, "mcl_batch_frnn_grid: cell tables");
    }
    m->bg_cap = cells;
  }
  // the parameters are uploaded only when they change, from a pinned buffer the
  // mesh keeps (a call captured in a CUDA graph then holds no host copy, or
  // reads memory that outlives the call)
  if (m->bg_cells != cells || std::memcmp(m->bg_par_host, par.data(), sizeof(int4) * nc) != 0) {
    QCK(cudaStreamSynchronize(s));  // the previous upload has been read
    std::memcpy(m->bg_par_host, par.data(), sizeof(int4) * nc);
    QCK(cudaMemcpyAsync(m->bg_par, m->bg_par_host, sizeof(int4) * nc, cudaMemcpyHostToDevice, s));
    m->bg_cells = cells;
  }
  const float2* pos = m->pos[m->cur];
  const int Vi = (int)V;
  QCK(cudaMemsetAsync(m->bg_count, 0, 4 * cells, s));
  k_bgrid_hash<<<(Vi + 255) / 256, 256, 0, s>>>(Vi, pos, m->vfix, m->vcomp, m->bg_par, lo, m->bg_cell, m->bg_count,
                                                out_dev, max_frnn);
  const int64_t nb = (cells + 1023) / 1024;
  int rc = scan_exclusive(m->bg_count, m->bg_start, cells, m->bg_tmp, m->bg_tmp + nb + 1, s);
  if (rc != MCL_OK) return rc;
  QCK(cudaMemcpyAsync(m->bg_cursor, m->bg_start, 4 * cells, cudaMemcpyDeviceToDevice, s));
  k_bgrid_scatter<<<(Vi + 255) / 256, 256, 0, s>>>(Vi, m->bg_cell, m->bg_cursor, m->bg_perm, m->bg_src);
  k_grid_sort_cells<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(cells, m->bg_start, m->bg_count, m->bg_src,
                                                                     m->bg_perm);
  const int npts = (int)(V - 4 * nc);
  k_gather<<<(npts + 255) / 256, 256, 0, s>>>(npts, m->bg_src, pos, m->bg_pos);
  unsigned long long* ovf = m->scratch + 4;
  QCK(cudaMemsetAsync(ovf, 0, 8, s));
  k_bgrid_frnn<<<(unsigned)((npts + kFrnnThreads - 1) / kFrnnThreads), kFrnnThreads, 0, s>>>(
      npts, m->bg_pos, m->bg_src, m->vcomp, m->bg_par, r_dev, lo, m->bg_start, m->bg_count, max_frnn, out_dev, ovf);
  QCK(cudaGetLastError());
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, ovf, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

// ---------------------------------------------------------------------------
// Grid neighbours without allocation.
//
// Some callers cannot allocate device memory at all: host frameworks that
// reserve the whole GPU up front and hand memory out only through their own
// pool, and real-time loops that must never block in an allocator.  For them
// this variant of GridCount2d::update + apply_f_frnn keeps its scratch (cell
// tables and per-point work arrays) in one fixed array that lives in the
// library's device image, so the call itself allocates nothing.  Limits:
// at most kNoAllocMaxPoints points and kNoAllocMaxCells cell-table entries
// (cells_x * cells_y, row-major cells as mcl_grid_create).  Every GPU that loads the
// library holds these 5.3 MB until the process exits.
constexpr int64_t kNoAllocMaxPoints = 262144;
constexpr int64_t kNoAllocMaxCells = 262144;
constexpr int64_t kNoAllocWords = 2 * kNoAllocMaxPoints + 3 * kNoAllocMaxCells + 64;
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocWords];

namespace {
int* g_noalloc_ptr[64];  // device address of the scratch array, per device id
std::mutex g_noalloc_mutex;

int noalloc_scratch(int** out) {
  int dev = 0;
  QCK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return qfail(MCL_ERR_NO_DEVICE, "device id out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return qfail(MCL_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<int*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return MCL_OK;
}
}  // namespace

extern "C" int mcl_grid_frnn_noalloc(const mcl_float2* pos, int64_t n, float min_x, float min_y, float cell_x,
                                     float cell_y, int32_t cells_x, int32_t cells_y, int flags, float r, int max_nb,
                                     mcl_float2* sorted_pos, int32_t* perm, int32_t* counts, int32_t* ids,
                                     void* stream, int64_t* overflow) {
  if (!pos || !sorted_pos || !perm || !counts || !ids || n < 0 || cells_x < 1 || cells_y < 1 || max_nb < 1 ||
      !(cell_x > 0.f) || !(cell_y > 0.f) || !(r >= 0.f))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  const int morton = 0;  // row-major cells, as mcl_grid_create
  const int64_t ncells = (int64_t)cells_x * cells_y;
  if (n > kNoAllocMaxPoints)
    return qfail(MCL_ERR_CAPACITY, "mcl_grid_frnn_noalloc: more than 262144 points");
  if (ncells > kNoAllocMaxCells)
    return qfail(MCL_ERR_CAPACITY, "mcl_grid_frnn_noalloc: cell table larger than 262144 entries");
  if (n == 0) return MCL_OK;
  int* base = nullptr;
  const int rc = noalloc_scratch(&base);
  if (rc != MCL_OK) return rc;
  int* cell = base;
  int* src = cell + kNoAllocMaxPoints;
  int* count = src + kNoAllocMaxPoints;
  int* start = count + kNoAllocMaxCells;
  int* cursor = start + kNoAllocMaxCells;
  unsigned long long* ovf = reinterpret_cast<unsigned long long*>(cursor + kNoAllocMaxCells);
  cudaStream_t s = (cudaStream_t)stream;
  GridView G;
  G.minx = min_x; G.miny = min_y; G.cx = cell_x; G.cy = cell_y;
  G.nx = cells_x; G.ny = cells_y; G.morton = morton; G.periodic = (flags & MCL_GRID_PERIODIC) ? 1 : 0;
  const int nn = (int)n;
  // the array keeps the previous call's contents: clear what must start at zero
  QCK(cudaMemsetAsync(count, 0, 4 * ncells, s));
  QCK(cudaMemsetAsync(ovf, 0, 8, s));
  k_grid_hash<<<(nn + 255) / 256, 256, 0, s>>>(G, nn, (const float2*)pos, cell, count);
  k_scan_one_block<<<1, 1024, 0, s>>>(count, start, ncells);
  QCK(cudaMemcpyAsync(cursor, start, 4 * ncells, cudaMemcpyDeviceToDevice, s));
  k_grid_scatter<<<(nn + 255) / 256, 256, 0, s>>>(nn, cell, cursor, perm, src);
  k_grid_sort_cells<<<(unsigned)((ncells + 255) / 256), 256, 0, s>>>(ncells, start, count, src, perm);
  k_gather<<<(nn + 255) / 256, 256, 0, s>>>(nn, src, (const float2*)pos, (float2*)sorted_pos);
  const int rc2 = launch_grid_frnn(G, nn, (const float2*)sorted_pos, start, count, r, cell_x * cells_x,
                                   cell_y * cells_y, max_nb, counts, ids, ovf, nullptr, s, nullptr);
  if (rc2 != MCL_OK) return rc2;
  if (overflow) {
    unsigned long long t = 0;
    QCK(cudaMemcpyAsync(&t, ovf, 8, cudaMemcpyDeviceToHost, s));
    QCK(cudaStreamSynchronize(s));
    *overflow = (int64_t)t;
  }
  return MCL_OK;
}

// ---------------------------------------------------------------------------
// The reference's AoS mesh arrays written on the device (DeviceTriangulation's
// public m_v / m_he / m_t, include/Device_Triangulation.h:139-142), in the
// layout and face numbering of mcl_mesh_download_aos: faces numbered in the
// order of their smallest half-edge.
namespace {

__device__ __forceinline__ bool aos_owner(const int4* ev, const int4* en, int64_t h, int* nxt, int* prv) {
  const int4 q = ev[h >> 1], w = en[h >> 1];
  const bool odd = h & 1;
  const int org = odd ? q.y : q.x, apex = odd ? q.w : q.z;
  *nxt = odd ? w.z : w.x;
  *prv = odd ? w.w : w.y;
  return apex >= 0 && org >= 0;
}

__global__ void k_aos_flags(const int4* ev, const int4* en, int64_t HE, int* flag) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= HE) return;
  int n, p;
  const bool inner = aos_owner(ev, en, h, &n, &p);
  flag[h] = inner && h < n && h < p ? 1 : 0;
}

__global__ void k_aos_write(const int4* ev, const int4* en, const int* vhe, int64_t V, int64_t HE, const int* fid,
                            int* v, int* he, int* t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < HE) {
    int n, p;
    const bool inner = aos_owner(ev, en, i, &n, &p);
    const int4 q = ev[i >> 1];
    const bool odd = i & 1;
    const int org = odd ? q.y : q.x, apex = odd ? q.w : q.z;
    int face = -1;
    if (inner) {
      const int64_t f = min(i, (int64_t)min(n, p));
      if (f >= 0 && f < HE) face = fid[f];
      if (t && i < n && i < p) t[fid[i]] = (int)i;
    }
    if (he) *reinterpret_cast<int4*>(he + 4 * i) = make_int4(n, org, face, apex >= 0 ? apex : -1);
  }
  if (v && i < V) *reinterpret_cast<int2*>(v + 2 * i) = make_int2((int)i, vhe[i]);
}

}  // namespace

extern "C" int mcl_mesh_export_aos(mcl_mesh* m, int32_t* v_dev, int32_t* he_dev, int32_t* t_dev, void* stream) {
  if (!m) return qfail(MCL_ERR_INVALID_ARGUMENT, "mcl_mesh_export_aos: null mesh");
  if (((uintptr_t)v_dev & 7) || ((uintptr_t)he_dev & 15))
    return qfail(MCL_ERR_INVALID_ARGUMENT, "mcl_mesh_export_aos: m_v must be 8-byte and m_he 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t HE = 2 * m->E, nb = (HE + 1023) / 1024;
  const int64_t need = 2 * HE + 2 * (nb + 2);
  if (m->aos_cap < need) {
    if (m->aos_tmp) QCK(cudaFree(m->aos_tmp));
    m->aos_tmp = nullptr;
    m->aos_cap = 0;
    if (cudaMalloc((void**)&m->aos_tmp, 4 * need) != cudaSuccess) {
      (void)cudaGetLastError();
      return qfail(MCL_ERR_OUT_OF_MEMORY, "mcl_mesh_export_aos: scratch");
    }
    m->aos_cap = need;
  }
  int* flag = m->aos_tmp;
  int* fid = flag + HE;
  int* tmp = fid + HE;
  const unsigned gb = (unsigned)((std::max(HE, m->V) + 255) / 256);
  k_aos_flags<<<(unsigned)((HE + 255) / 256), 256, 0, s>>>(m->ev, m->en, HE, flag);
  const int rc = scan_exclusive(flag, fid, HE, tmp, tmp + nb + 1, s);
  if (rc != MCL_OK) return rc;
  k_aos_write<<<gb, 256, 0, s>>>(m->ev, m->en, m->vhe, m->V, HE, fid, v_dev, he_dev, t_dev);
  QCK(cudaGetLastError());
  return MCL_OK;
}
