// Periodic (flat torus) kinetic Delaunay meshes on the GPU.
//
// The reference keeps its periodic triangulation as a stub
// (include/Host_PeriodicTriangulation.h: the constructor at :101-104 holds a
// CGAL periodic domain, commented out).  Here a periodic mesh is n points on
// the torus [2L, 3L)^2 (L a power of two), 3n edges and 2n faces: the planar
// engine's ev / en records plus one offset word per edge (periodic.cuh, which
// also holds the per-thread bodies of every kernel below).
//
//   build   the planar GPU build (mcl_mesh_build) of the points and of their
//           copies within a band around the domain, downloaded and restricted
//           to the torus on the host (periodic_from_planar); a quarter period
//           of band first, the whole 3 x 3 cover if that does not close up.
//   step    move + wrap (one launch over vertices), the wraps folded into the
//           edge words (one launch over edges), then rounds of classify +
//           claim / flip winners (one launch each) until no edge is
//           non-Delaunay; the host reads the round's counters between
//           launches.  A classification that finds faces turned over sends
//           their moved vertices back (one launch over vertices, then the
//           fold again) and classifies again; flips start from a mesh whose
//           faces are all positive.  Vertices sent back then follow in up to
//           kSubLevels sub-steps (half of what they still owe, the last all);
//           the few still away (listed in parallel, by ascending id) are
//           removed and reinserted at their targets by one thread
//           (k_preinsert).
//   queries one-ring with copy offsets, closest neighbour, mesh FRNN (one
//           launch for the outgoing half-edges, one per query).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine.cuh"
#include "periodic.cuh"

using mcl::PCount;
using mcl::PF2;
using mcl::PI4;
using mcl::PView;

struct mcl_periodic {
  int64_t n, E;
  float L;
  PF2* pos;
  PI4* ev;
  PI4* en;
  unsigned* eo;
  unsigned char* wv;
  unsigned char* wt;
  unsigned char* mark;
  PF2* pos_old;
  PF2* target;
  PF2* dsub;         // sub-step displacements
  PF2* dstage;       // host displacements copied in
  int* clist;        // a round's non-Delaunay edges
  int* wl[2];        // edge work-lists between rounds
  unsigned* qstamp;
  unsigned* cand;
  unsigned long long* claim;
  int* vhe;          // one outgoing half-edge per vertex (queries)
  PCount* cnt;
  PCount* cnt_host;  // pinned
  unsigned stamp;    // last round stamp used
};

namespace {

constexpr int kThreads = 256;
constexpr int kMaxRounds = 4096;
constexpr int kMaxRevertPasses = 256;
constexpr int kSubLevels = 5;  // sub-steps for vertices sent back
// vertices one thread removes and reinserts per step at most (the rest stay
// behind, counted): the single-thread kernel's time stays bounded
constexpr int kMaxReinsert = 1 << 16;
constexpr int kCenter = 4;  // copy index of the untranslated copy

#define PCK(call)                                       \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return mcl::cuda_fail(_e, #call); \
  } while (0)

__global__ void k_pmove(PView V, const PF2* d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_move(V, d, i);
}
__global__ void k_ptarget(PView V, const PF2* d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_target(V, d, i);
}
__global__ void k_presume(PView V, PF2* d, bool last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_resume(V, d, i, last);
}
// The vertices still away from their targets, listed by ascending id (the
// order the reinsertion takes them in), built in parallel: a count per chunk
// of kChunk vertices, one block scanning the counts (total appended), then
// each chunk writing its vertices in order.
constexpr int kChunk = 1024;
__device__ __forceinline__ bool p_behind(const PView& V, int i) {
  const PF2 here = V.pos[i], t = V.target[i];
  return !(here.x == t.x && here.y == t.y);
}
__global__ void __launch_bounds__(kChunk) k_pbehind_count(PView V, int* chunk) {
  const int i = blockIdx.x * kChunk + threadIdx.x;
  const int c = __syncthreads_count(i < V.n && p_behind(V, i));
  if (threadIdx.x == 0) chunk[blockIdx.x] = c;
}
// exclusive scan of chunk[0..nb) in place, the total in chunk[nb] (one block)
__global__ void __launch_bounds__(kChunk) k_pbehind_scan(int* chunk, int nb) {
  __shared__ int tot[kChunk];
  const int per = (nb + kChunk - 1) / kChunk, lo = threadIdx.x * per, hi = min(nb, lo + per);
  int run = 0;
  for (int i = lo; i < hi; ++i) run += chunk[i];
  tot[threadIdx.x] = run;
  __syncthreads();
  for (int o = 1; o < kChunk; o <<= 1) {
    const int y = threadIdx.x >= (unsigned)o ? tot[threadIdx.x - o] : 0;
    __syncthreads();
    tot[threadIdx.x] += y;
    __syncthreads();
  }
  int acc = threadIdx.x ? tot[threadIdx.x - 1] : 0;
  for (int i = lo; i < hi; ++i) {
    const int x = chunk[i];
    chunk[i] = acc;
    acc += x;
  }
  if (threadIdx.x == kChunk - 1) chunk[nb] = tot[kChunk - 1];
}
__global__ void __launch_bounds__(kChunk) k_pbehind_scatter(PView V, const int* chunk, int* list) {
  __shared__ int wbase[kChunk / 32];
  const int i = blockIdx.x * kChunk + threadIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool b = i < V.n && p_behind(V, i);
  const unsigned bal = __ballot_sync(0xffffffffu, b);
  if (lane == 0) wbase[warp] = __popc(bal);
  __syncthreads();
  if (warp == 0) {
    const int x = wbase[lane];
    int incl = x;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    wbase[lane] = incl - x;
  }
  __syncthreads();
  if (b) list[chunk[blockIdx.x] + wbase[warp] + __popc(bal & ((1u << lane) - 1u))] = i;
}
// one thread: the sequential removal and reinsertion of the listed vertices
__global__ void k_preinsert(PView V, int* vhe, const int* list, const int* count) {
  if (blockIdx.x == 0 && threadIdx.x == 0) mcl::p_body_reinsert(V, vhe, list, *count, kMaxReinsert);
}
__global__ void k_prevert(PView V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_revert(V, i);
}
__global__ void k_pwrap(PView V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.E) mcl::p_body_wrap(V, i);
}
// every edge (list < 0) or the entries of work-list `list`, grid-stride (the
// list's length is read on the device)
__global__ void k_pclassify(PView V, unsigned stamp, int list) {
  const long long items = list < 0 ? (long long)V.E : (long long)V.cnt->lcount[list];
  const int* wl = list == 1 ? V.wl1 : V.wl0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < items;
       i += (long long)gridDim.x * blockDim.x) {
    const int e = list < 0 ? (int)i : wl[i];
    if ((unsigned)e < (unsigned)V.E) mcl::p_body_classify(V, e, stamp);
  }
}
// the round's non-Delaunay edges; winners flip and queue their wings on `next`
__global__ void k_pflip(PView V, unsigned stamp, int next) {
  const long long items = (long long)V.cnt->nondelaunay;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < items;
       i += (long long)gridDim.x * blockDim.x) {
    const int e = V.clist[i];
    if ((unsigned)e < (unsigned)V.E) mcl::p_body_flip(V, e, stamp, next);
  }
}
__global__ void k_pvhe(PView V, int* vhe) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 2 * V.E) mcl::p_body_vhe(V, vhe, i);
}
__global__ void k_pring(PView V, const int* vhe, bool column, int max_ring, int* ring, unsigned char* offs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_ring(V, vhe, i, column, max_ring, ring, offs);
}
__global__ void k_pfrnn(PView V, const int* vhe, float r2, bool column, int max_frnn, int* out, unsigned char* offs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_frnn(V, vhe, i, r2, column, max_frnn, out, offs);
}
__global__ void k_pclosest(PView V, bool column, int max_ring, const int* ring, const unsigned char* offs, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V.n) mcl::p_body_closest(V, i, column, max_ring, ring, offs, out);
}

unsigned blocks(int64_t k) { return (unsigned)((k + kThreads - 1) / kThreads); }
// grid of the grid-stride list kernels: 16 blocks of 256 per SM of a GB300 at most
unsigned list_blocks(int64_t k) { return std::min<unsigned>(blocks(k), 152u * 16u); }

PView view(mcl_periodic* m) {
  return PView{(int)m->n, (int)m->E,  m->L,       2.0f * m->L, m->pos,    m->ev,   m->en,    m->eo,
               m->wv,      m->wt,      m->mark,    m->pos_old,  m->target, m->cand, m->claim, m->cnt,
               m->clist,   m->wl[0],   m->wl[1],   m->qstamp};
}

void free_periodic(mcl_periodic* m) {
  if (!m) return;
  cudaFree(m->pos);
  cudaFree(m->ev);
  cudaFree(m->en);
  cudaFree(m->eo);
  cudaFree(m->wv);
  cudaFree(m->wt);
  cudaFree(m->mark);
  cudaFree(m->pos_old);
  cudaFree(m->target);
  cudaFree(m->dsub);
  cudaFree(m->dstage);
  cudaFree(m->clist);
  cudaFree(m->wl[0]);
  cudaFree(m->wl[1]);
  cudaFree(m->qstamp);
  cudaFree(m->cand);
  cudaFree(m->claim);
  cudaFree(m->vhe);
  cudaFree(m->cnt);
  if (m->cnt_host) cudaFreeHost(m->cnt_host);
  delete m;
}

// L > 0, finite, a power of two, and the cover of the domain inside the
// +-1e7 bounding square of the planar build (4L < 1e7)
bool period_ok(float L) {
  if (!(L > 0.0f) || !std::isfinite(L) || L > 2097152.0f) return false;
  int ex = 0;
  return std::frexp(L, &ex) == 0.5f;
}

bool in_domain(mcl_float2 p, float L) {
  const float lo = 2.0f * L, hi = 3.0f * L;
  return p.x >= lo && p.x < hi && p.y >= lo && p.y < hi;
}

uint64_t bits_key(mcl_float2 p) {
  uint32_t x, y;
  std::memcpy(&x, &p.x, 4);
  std::memcpy(&y, &p.y, 4);
  return ((uint64_t)x << 32) | y;
}

mcl::Off copy_offset(int k) { return mcl::Off{k % 3 - 1, k / 3 - 1}; }

// The periodic mesh a planar triangulation of a cover stands for (see
// mcl_periodic_from_planar).  he: the planar AoS half-edges {next, v, t, op};
// tri: one half-edge per face.
bool periodic_from_planar(const int32_t* he, int64_t HE, const int32_t* tri, int64_t T, const int32_t* vpoint,
                          const int32_t* vcopy, int64_t V, int64_t n, std::vector<PI4>& ev, std::vector<PI4>& en,
                          std::vector<unsigned>& eo, std::string& why) {
  struct Face {
    int p[3];
    int k[3];
  };
  std::vector<Face> faces;
  faces.reserve((size_t)(2 * n));
  for (int64_t f = 0; f < T; ++f) {
    int h[3];
    h[0] = tri[f];
    if (h[0] < 0 || h[0] >= HE) { why = "a face without a valid half-edge"; return false; }
    h[1] = he[4 * (int64_t)h[0]];
    if (h[1] < 0 || h[1] >= HE) { why = "a broken next pointer"; return false; }
    h[2] = he[4 * (int64_t)h[1]];
    if (h[2] < 0 || h[2] >= HE || he[4 * (int64_t)h[2]] != h[0]) { why = "a face that is not a triangle"; return false; }
    Face fc;
    bool cover = true;
    for (int j = 0; j < 3; ++j) {
      const int v = he[4 * (int64_t)h[j] + 1];
      if (v < 0 || v >= V) { why = "a half-edge origin out of range"; return false; }
      fc.p[j] = vpoint[v];
      fc.k[j] = vcopy[v];
      if (fc.p[j] < 0 || fc.k[j] < 0) { cover = false; break; }
      if (fc.p[j] >= n || fc.k[j] > 8) { why = "a vertex map entry out of range"; return false; }
    }
    if (!cover) continue;
    int jmin = 0;
    for (int j = 1; j < 3; ++j)
      if (fc.p[j] < fc.p[jmin]) jmin = j;
    if (fc.k[jmin] != kCenter) continue;
    if (fc.p[0] == fc.p[1] || fc.p[1] == fc.p[2] || fc.p[0] == fc.p[2]) {
      why = "a face uses two copies of one point: too few points for the period";
      return false;
    }
    faces.push_back(fc);
  }
  if ((int64_t)faces.size() != 2 * n) {
    why = "the cover does not close up into a torus triangulation (" + std::to_string(faces.size()) + " faces for " +
          std::to_string(n) + " points)";
    return false;
  }
  // half-edge (f, j): origin corner j, target j + 1, apex j + 2
  struct Half {
    int u, v, tx, ty;  // canonical edge key
    int side;          // 0: this half-edge runs u -> v
    int64_t fj;        // 3 f + j
  };
  const int64_t H = 6 * n;
  std::vector<Half> hs((size_t)H);
  std::vector<int> org((size_t)H), apx((size_t)H);
  std::vector<mcl::Off> tof((size_t)H), xof((size_t)H);
  for (int64_t f = 0; f < 2 * n; ++f)
    for (int j = 0; j < 3; ++j) {
      const Face& fc = faces[(size_t)f];
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      const mcl::Off t = mcl::off_sub(copy_offset(fc.k[j1]), copy_offset(fc.k[j]));
      const mcl::Off x = mcl::off_sub(copy_offset(fc.k[j2]), copy_offset(fc.k[j]));
      if (!mcl::off_small(t) || !mcl::off_small(x)) { why = "an edge longer than the band"; return false; }
      const int a = fc.p[j], b = fc.p[j1];
      const bool first = a < b || (a == b && (t.x > 0 || (t.x == 0 && t.y > 0)));
      const int64_t fj = 3 * f + j;
      hs[(size_t)fj] = first ? Half{a, b, t.x, t.y, 0, fj} : Half{b, a, -t.x, -t.y, 1, fj};
      org[(size_t)fj] = a;
      apx[(size_t)fj] = fc.p[j2];
      tof[(size_t)fj] = t;
      xof[(size_t)fj] = x;
    }
  std::sort(hs.begin(), hs.end(), [](const Half& p, const Half& q) {
    if (p.u != q.u) return p.u < q.u;
    if (p.v != q.v) return p.v < q.v;
    if (p.tx != q.tx) return p.tx < q.tx;
    if (p.ty != q.ty) return p.ty < q.ty;
    return p.side < q.side;
  });
  std::vector<int64_t> hid((size_t)H);  // half-edge id of (f, j)
  for (int64_t e = 0; e < 3 * n; ++e) {
    const Half& p = hs[(size_t)(2 * e)];
    const Half& q = hs[(size_t)(2 * e + 1)];
    if (p.u != q.u || p.v != q.v || p.tx != q.tx || p.ty != q.ty || p.side != 0 || q.side != 1 ||
        (e > 0 && hs[(size_t)(2 * e - 1)].u == p.u && hs[(size_t)(2 * e - 1)].v == p.v &&
         hs[(size_t)(2 * e - 1)].tx == p.tx && hs[(size_t)(2 * e - 1)].ty == p.ty)) {
      why = "half-edges do not pair into 3n edges";
      return false;
    }
    hid[(size_t)p.fj] = 2 * e;
    hid[(size_t)q.fj] = 2 * e + 1;
  }
  ev.assign((size_t)(3 * n), PI4{0, 0, 0, 0});
  en.assign((size_t)(3 * n), PI4{0, 0, 0, 0});
  eo.assign((size_t)(3 * n), 0u);
  std::vector<mcl::Off> tt((size_t)H), xx((size_t)H);
  for (int64_t fj = 0; fj < H; ++fj) {
    const int64_t f = fj / 3;
    const int j = (int)(fj % 3);
    const int64_t h = hid[(size_t)fj];
    const int nx = (int)hid[(size_t)(3 * f + (j + 1) % 3)];
    const int pv = (int)hid[(size_t)(3 * f + (j + 2) % 3)];
    PI4& q = ev[(size_t)(h >> 1)];
    PI4& w = en[(size_t)(h >> 1)];
    if (h & 1) {
      q.y = org[(size_t)fj];
      q.w = apx[(size_t)fj];
      w.z = nx;
      w.w = pv;
    } else {
      q.x = org[(size_t)fj];
      q.z = apx[(size_t)fj];
      w.x = nx;
      w.y = pv;
    }
    tt[(size_t)h] = tof[(size_t)fj];
    xx[(size_t)h] = xof[(size_t)fj];
  }
  for (int64_t e = 0; e < 3 * n; ++e)
    eo[(size_t)e] = mcl::eo_pack(tt[(size_t)(2 * e)], xx[(size_t)(2 * e)], xx[(size_t)(2 * e + 1)]);
  return true;
}

// structural check of host arrays before they go to the device
bool periodic_valid(int64_t n, const int32_t* ev, const int32_t* en, const uint32_t* eo, std::string& why) {
  const int64_t E = 3 * n, H = 6 * n;
  for (int64_t e = 0; e < E; ++e) {
    for (int k = 0; k < 4; ++k) {
      if (ev[4 * e + k] < 0 || ev[4 * e + k] >= n) { why = "ev out of range at edge " + std::to_string(e); return false; }
      if (en[4 * e + k] < 0 || en[4 * e + k] >= H) { why = "en out of range at edge " + std::to_string(e); return false; }
    }
    const unsigned w = eo[e];
    if ((w >> 24) != 0 || !mcl::off_small(mcl::eo_b(w)) || !mcl::off_small(mcl::eo_c(w)) ||
        !mcl::off_small(mcl::eo_x1(w))) {
      why = "eo out of range at edge " + std::to_string(e);
      return false;
    }
  }
  return true;
}

int alloc_upload(const mcl_float2* pos, int64_t n, float L, const int32_t* ev, const int32_t* en,
                 const uint32_t* eo, mcl_periodic** out) {
  mcl_periodic* m = new mcl_periodic();
  std::memset(m, 0, sizeof(*m));
  m->n = n;
  m->E = 3 * n;
  m->L = L;
  const int64_t E = m->E;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  A((void**)&m->pos, 8 * (size_t)n);
  A((void**)&m->ev, 16 * (size_t)E);
  A((void**)&m->en, 16 * (size_t)E);
  A((void**)&m->eo, 4 * (size_t)E);
  A((void**)&m->wv, (size_t)n);
  A((void**)&m->wt, (size_t)n);
  A((void**)&m->mark, (size_t)n);
  A((void**)&m->pos_old, 8 * (size_t)n);
  A((void**)&m->target, 8 * (size_t)n);
  A((void**)&m->dsub, 8 * (size_t)n);
  A((void**)&m->dstage, 8 * (size_t)n);
  A((void**)&m->clist, 4 * (size_t)E);
  A((void**)&m->wl[0], 4 * (size_t)E);
  A((void**)&m->wl[1], 4 * (size_t)E);
  A((void**)&m->qstamp, 4 * (size_t)E);
  A((void**)&m->cand, 4 * (size_t)E);
  A((void**)&m->claim, 16 * (size_t)E);
  A((void**)&m->vhe, 4 * (size_t)n);
  A((void**)&m->cnt, sizeof(PCount));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&m->cnt_host, sizeof(PCount));
  if (e == cudaSuccess) e = cudaMemcpy(m->pos, pos, 8 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->ev, ev, 16 * (size_t)E, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->en, en, 16 * (size_t)E, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->eo, eo, 4 * (size_t)E, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->wv, 0x88, (size_t)n);
  if (e == cudaSuccess) e = cudaMemset(m->wt, 0x88, (size_t)n);
  if (e == cudaSuccess) e = cudaMemset(m->mark, 0, (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpy(m->pos_old, pos, 8 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->target, pos, 8 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->cand, 0, 4 * (size_t)E);
  if (e == cudaSuccess) e = cudaMemset(m->claim, 0, 16 * (size_t)E);
  if (e == cudaSuccess) e = cudaMemset(m->qstamp, 0, 4 * (size_t)E);
  if (e == cudaSuccess) e = cudaMemset(m->cnt, 0, sizeof(PCount));
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    free_periodic(m);
    return mcl::cuda_fail(e, "periodic mesh upload");
  }
  *out = m;
  return MCL_OK;
}

// Rounds of classification after a move: faces turned over send their moved
// vertices back (then the fold again), otherwise the winners of the
// non-Delaunay edges flip, until no edge is non-Delaunay.  Counters
// accumulate in z across calls.
struct Settle {
  PCount c{};
  unsigned long long inverted_first = 0;
  bool classified = false;
  int rounds = 0;
  int64_t incircle_tests = 0;  // the edges classified in rounds without a face turned over
  std::string msg;
};

int settle(mcl_periodic* m, cudaStream_t s, const PView& V, Settle& z) {
  int revert_passes = 0, cur = -1;  // the work-list to classify (-1: every edge)
  bool flipped = false;
  for (int r = 0; r < kMaxRounds; ++r) {
    if (m->stamp >= 0xFFFFFFFEu) {  // stamps about to wrap: forget every old claim and queue mark
      PCK(cudaMemsetAsync(m->claim, 0, 16 * (size_t)m->E, s));
      PCK(cudaMemsetAsync(m->cand, 0, 4 * (size_t)m->E, s));
      PCK(cudaMemsetAsync(m->qstamp, 0, 4 * (size_t)m->E, s));
      m->stamp = 0;
    }
    const unsigned stamp = ++m->stamp;
    PCK(cudaMemsetAsync(&m->cnt->inverted, 0, 2 * sizeof(unsigned long long), s));  // inverted, nondelaunay
    k_pclassify<<<list_blocks(m->E), kThreads, 0, s>>>(V, stamp, cur);
    PCK(cudaGetLastError());
    PCK(cudaMemcpyAsync(m->cnt_host, m->cnt, sizeof(PCount), cudaMemcpyDeviceToHost, s));
    PCK(cudaStreamSynchronize(s));
    z.c = *m->cnt_host;
    ++z.rounds;
    const int64_t classified = cur < 0 ? m->E : (int64_t)z.c.lcount[cur];
    if (z.c.error) {
      const int rc = (int)z.c.error;
      z.msg = "mcl_periodic_step: " + std::string(mcl_status_string(rc)) + " (site " + std::to_string(z.c.error_site) +
              ")";
      return rc;
    }
    if (!z.classified) {
      z.inverted_first = z.c.inverted;
      z.classified = true;
    }
    if (z.c.inverted) {
      // flips only start from a mesh whose faces are all positive
      if (flipped) {
        z.msg = "mcl_periodic_step: a face turned over after flips (the mesh was not valid)";
        return MCL_ERR_DEGENERATE_INPUT;
      }
      if (revert_passes == kMaxRevertPasses) {
        z.msg = "mcl_periodic_step: sending vertices back did not end";
        return MCL_ERR_NO_CONVERGENCE;
      }
      k_prevert<<<blocks(m->n), kThreads, 0, s>>>(V);
      k_pwrap<<<blocks(m->E), kThreads, 0, s>>>(V);
      PCK(cudaGetLastError());
      ++revert_passes;
      cur = -1;
      continue;
    }
    z.incircle_tests += classified;
    if (!z.c.nondelaunay) return MCL_OK;
    const int next = cur == 0 ? 1 : 0;
    PCK(cudaMemsetAsync(&m->cnt->lcount[next], 0, sizeof(unsigned long long), s));
    k_pflip<<<list_blocks((int64_t)z.c.nondelaunay), kThreads, 0, s>>>(V, stamp, next);
    PCK(cudaGetLastError());
    cur = next;
    flipped = true;
  }
  z.msg = "mcl_periodic_step: flip rounds did not converge";
  return MCL_ERR_NO_CONVERGENCE;
}

}  // namespace

extern "C" {

int mcl_periodic_from_planar(const mcl_aos_view* a, const int32_t* vertex_point, const int32_t* vertex_copy,
                             int64_t n, int32_t* ev_out, int32_t* en_out, uint32_t* eo_out) {
  if (!a || !a->he || !a->t || !vertex_point || !vertex_copy || !ev_out || !en_out || !eo_out || n < 1 ||
      n > (1 << 28))
    return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_from_planar: bad arguments");
  std::vector<PI4> ev, en;
  std::vector<unsigned> eo;
  std::string why;
  if (!periodic_from_planar(a->he, a->HE, a->t, a->T, vertex_point, vertex_copy, a->V, n, ev, en, eo, why))
    return mcl::fail(MCL_ERR_DEGENERATE_INPUT, "mcl_periodic_from_planar: " + why);
  std::memcpy(ev_out, ev.data(), 16 * ev.size());
  std::memcpy(en_out, en.data(), 16 * en.size());
  std::memcpy(eo_out, eo.data(), 4 * eo.size());
  return MCL_OK;
}

int mcl_periodic_create(const mcl_float2* pos, int64_t n, float L, const int32_t* ev, const int32_t* en,
                        const uint32_t* eo, mcl_periodic** out) {
  if (!pos || !ev || !en || !eo || !out || n < 1 || n > (1 << 28) || !period_ok(L))
    return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_create: bad arguments (L must be a power of two)");
  for (int64_t i = 0; i < n; ++i)
    if (!in_domain(pos[i], L)) return mcl::fail(MCL_ERR_DEGENERATE_INPUT, "a point outside [2L, 3L)^2");
  std::string why;
  if (!periodic_valid(n, ev, en, eo, why)) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "malformed periodic mesh: " + why);
  return alloc_upload(pos, n, L, ev, en, eo, out);
}

int mcl_periodic_build(const mcl_float2* pts, int64_t n, float L, mcl_periodic** out) {
  if (!pts || !out || n < 1 || n > (1 << 26) || !period_ok(L))
    return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_build: bad arguments (L must be a power of two <= 2^21)");
  for (int64_t i = 0; i < n; ++i)
    if (!in_domain(pts[i], L)) return mcl::fail(MCL_ERR_DEGENERATE_INPUT, "a point outside [2L, 3L)^2");
  const float lo = 2.0f * L, hi = 3.0f * L;
  std::string why;
  for (const float band : {0.25f * L, L}) {
    // the points (copy 4) first, then their translates inside the band
    std::vector<mcl_float2> cp;
    std::vector<int32_t> cpoint, ccopy;
    cp.reserve((size_t)(3 * n));
    for (int k = 0; k < 9; ++k) {
      const mcl::Off o = copy_offset(k == 0 ? kCenter : (k <= kCenter ? k - 1 : k));
      for (int64_t i = 0; i < n; ++i) {
        const mcl_float2 q{pts[i].x + (float)o.x * L, pts[i].y + (float)o.y * L};
        if (!(q.x >= lo - band && q.x < hi + band && q.y >= lo - band && q.y < hi + band)) continue;
        cp.push_back(q);
        cpoint.push_back((int32_t)i);
        ccopy.push_back((int32_t)(3 * (o.y + 1) + (o.x + 1)));
      }
    }
    std::unordered_map<uint64_t, int64_t> where;
    where.reserve(cp.size() * 2);
    for (size_t c = 0; c < cp.size(); ++c)
      if (!where.emplace(bits_key(cp[c]), (int64_t)c).second)
        return mcl::fail(MCL_ERR_DEGENERATE_INPUT, "mcl_periodic_build: duplicate point");
    std::vector<mcl_float2> sorted = cp;
    mcl_mesh* pm = nullptr;
    int rc = mcl_mesh_build(sorted.data(), (int64_t)sorted.size(), &pm);
    if (rc != MCL_OK) return rc;
    int64_t V = 0, HE = 0, T = 0;
    rc = mcl_mesh_sizes(pm, &V, &HE, &T);
    std::vector<mcl_float2> ppos;
    std::vector<int32_t> pv, phe, pt;
    if (rc == MCL_OK) {
      ppos.resize((size_t)V);
      pv.resize((size_t)(2 * V));
      phe.resize((size_t)(4 * HE));
      pt.resize((size_t)T);
      rc = mcl_mesh_download_aos(pm, ppos.data(), pv.data(), phe.data(), pt.data());
    }
    mcl_mesh_destroy(pm);
    if (rc != MCL_OK) return rc;
    std::vector<int32_t> vpoint((size_t)V, -1), vcopy((size_t)V, -1);
    for (int64_t v = 4; v < V; ++v) {
      const int32_t pi = pv[(size_t)(2 * v)];
      if (pi < 0 || pi >= V) return mcl::fail(MCL_ERR_CUDA, "mcl_periodic_build: planar vertex without a position");
      const auto it = where.find(bits_key(ppos[(size_t)pi]));
      if (it == where.end()) return mcl::fail(MCL_ERR_CUDA, "mcl_periodic_build: planar vertex not in the cover");
      vpoint[(size_t)v] = cpoint[(size_t)it->second];
      vcopy[(size_t)v] = ccopy[(size_t)it->second];
    }
    std::vector<PI4> ev, en;
    std::vector<unsigned> eo;
    if (!periodic_from_planar(phe.data(), HE, pt.data(), T, vpoint.data(), vcopy.data(), V, n, ev, en, eo, why))
      continue;
    return alloc_upload(pts, n, L, reinterpret_cast<const int32_t*>(ev.data()),
                        reinterpret_cast<const int32_t*>(en.data()), eo.data(), out);
  }
  return mcl::fail(MCL_ERR_DEGENERATE_INPUT, "mcl_periodic_build: " + why);
}

int mcl_periodic_destroy(mcl_periodic* m) {
  if (!m) return MCL_OK;
  cudaDeviceSynchronize();
  free_periodic(m);
  return MCL_OK;
}

int mcl_periodic_sizes(const mcl_periodic* m, int64_t* n, int64_t* E, float* L) {
  if (!m) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null periodic mesh");
  if (n) *n = m->n;
  if (E) *E = m->E;
  if (L) *L = m->L;
  return MCL_OK;
}

int mcl_periodic_download(mcl_periodic* m, mcl_float2* pos, int32_t* ev, int32_t* en, uint32_t* eo) {
  if (!m) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null periodic mesh");
  PCK(cudaDeviceSynchronize());
  if (pos) PCK(cudaMemcpy(pos, m->pos, 8 * (size_t)m->n, cudaMemcpyDeviceToHost));
  if (ev) PCK(cudaMemcpy(ev, m->ev, 16 * (size_t)m->E, cudaMemcpyDeviceToHost));
  if (en) PCK(cudaMemcpy(en, m->en, 16 * (size_t)m->E, cudaMemcpyDeviceToHost));
  if (eo) PCK(cudaMemcpy(eo, m->eo, 4 * (size_t)m->E, cudaMemcpyDeviceToHost));
  return MCL_OK;
}

int mcl_periodic_positions(mcl_periodic* m, mcl_float2** pos_dev) {
  if (!m || !pos_dev) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  *pos_dev = reinterpret_cast<mcl_float2*>(m->pos);
  return MCL_OK;
}

int mcl_periodic_step(mcl_periodic* m, const mcl_float2* d_dev, void* stream, mcl_step_stats* stats,
                      int64_t* wrapped) {
  if (!m || !d_dev) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  const PView V = view(m);
  Settle z;
  PCK(cudaMemsetAsync(m->cnt, 0, sizeof(PCount), s));
  k_ptarget<<<blocks(m->n), kThreads, 0, s>>>(V, reinterpret_cast<const PF2*>(d_dev));
  k_pmove<<<blocks(m->n), kThreads, 0, s>>>(V, reinterpret_cast<const PF2*>(d_dev));
  k_pwrap<<<blocks(m->E), kThreads, 0, s>>>(V);
  PCK(cudaGetLastError());
  int rc = settle(m, s, V, z);
  // sub-steps: vertices sent back move again by half of what they still owe,
  // the last level by all of it (landing exactly on the target)
  int64_t behind_first = -1, behind = 0;
  for (int level = 1; rc == MCL_OK; ++level) {
    const bool last = level >= kSubLevels;
    PCK(cudaMemsetAsync(&m->cnt->behind, 0, sizeof(unsigned long long), s));
    k_presume<<<blocks(m->n), kThreads, 0, s>>>(V, m->dsub, last);
    PCK(cudaGetLastError());
    PCK(cudaMemcpyAsync(m->cnt_host, m->cnt, sizeof(PCount), cudaMemcpyDeviceToHost, s));
    PCK(cudaStreamSynchronize(s));
    behind = (int64_t)m->cnt_host->behind;
    if (behind_first < 0) behind_first = behind;
    if (behind == 0 || level > kSubLevels) break;
    k_pmove<<<blocks(m->n), kThreads, 0, s>>>(V, m->dsub);
    k_pwrap<<<blocks(m->E), kThreads, 0, s>>>(V);
    PCK(cudaGetLastError());
    rc = settle(m, s, V, z);
  }
  const int64_t substep_arrivals = behind_first > behind ? behind_first - behind : 0;
  // the rest: removed and reinserted at their targets, one by one
  int64_t reinserted = 0;
  if (rc == MCL_OK && behind > 0) {
    PCK(cudaMemsetAsync(&m->cnt->behind, 0, sizeof(unsigned long long), s));
    PCK(cudaMemsetAsync(&m->cnt->reinserted, 0, sizeof(unsigned long long), s));
    PCK(cudaMemsetAsync(m->vhe, 0xFF, 4 * (size_t)m->n, s));  // vhe = -1: the largest candidate wins
    k_pvhe<<<blocks(2 * m->E), kThreads, 0, s>>>(V, m->vhe);
    // the flip rounds are over: clist holds the list, wl[1] the chunk counts
    const int nb = (int)((m->n + kChunk - 1) / kChunk);
    k_pbehind_count<<<nb, kChunk, 0, s>>>(V, m->wl[1]);
    k_pbehind_scan<<<1, kChunk, 0, s>>>(m->wl[1], nb);
    k_pbehind_scatter<<<nb, kChunk, 0, s>>>(V, m->wl[1], m->clist);
    k_preinsert<<<1, 32, 0, s>>>(V, m->vhe, m->clist, m->wl[1] + nb);
    PCK(cudaGetLastError());
    PCK(cudaMemsetAsync(&m->cnt->behind, 0, sizeof(unsigned long long), s));
    k_presume<<<blocks(m->n), kThreads, 0, s>>>(V, m->dsub, true);  // counts who is still behind
    PCK(cudaGetLastError());
    PCK(cudaMemcpyAsync(m->cnt_host, m->cnt, sizeof(PCount), cudaMemcpyDeviceToHost, s));
    PCK(cudaStreamSynchronize(s));
    const PCount& r = *m->cnt_host;
    if (r.error) {
      rc = (int)r.error;
      z.msg = "mcl_periodic_step: removal and reinsertion failed (site " + std::to_string(r.error_site) + ")";
    }
    reinserted = (int64_t)r.reinserted;
    behind = (int64_t)r.behind;
    z.c.flips = r.flips;
    z.c.error_site = r.error_site;
  }
  const PCount& c = z.c;
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->inverted_faces = (int64_t)((z.inverted_first + 2) / 3);  // each face is seen from its three edges
    stats->reverted_vertices = behind;
    stats->removed_vertices = reinserted;
    stats->substep_vertices = substep_arrivals;
    stats->lawson_flips = (int64_t)c.flips;
    stats->lawson_rounds = z.rounds;
    stats->incircle_tests = z.incircle_tests;
    stats->incircle_fp64 = (int64_t)c.incircle_fp64;
    stats->incircle_exact = (int64_t)c.incircle_exact;
    stats->orient_fp64 = (int64_t)c.orient_fp64;
    stats->orient_exact = (int64_t)c.orient_exact;
    stats->sos_decisions = (int64_t)c.sos;
    stats->status = rc;
    stats->error_site = (int64_t)c.error_site;
  }
  if (wrapped) *wrapped = (int64_t)c.wrapped;
  if (rc == MCL_OK && c.overflow) {
    rc = MCL_ERR_PREDICATE;
    z.msg = "mcl_periodic_step: exact predicate capacity exceeded";
  }
  return rc == MCL_OK ? MCL_OK : mcl::fail(rc, z.msg);
}

int mcl_periodic_step_host(mcl_periodic* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats,
                           int64_t* wrapped) {
  if (!m || !d_host) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  PCK(cudaMemcpyAsync(m->dstage, d_host, 8 * (size_t)m->n, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return mcl_periodic_step(m, reinterpret_cast<const mcl_float2*>(m->dstage), stream, stats, wrapped);
}

int mcl_periodic_one_ring(mcl_periodic* m, int max_ring, int layout, int32_t* ring_dev, uint8_t* offs_dev,
                          void* stream, int64_t* truncated) {
  if (!m || !ring_dev || max_ring < 1 || (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_one_ring: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const PView V = view(m);
  PCK(cudaMemsetAsync(m->cnt, 0, sizeof(PCount), s));
  PCK(cudaMemsetAsync(m->vhe, 0xFF, 4 * (size_t)m->n, s));  // vhe = -1: the largest candidate wins
  k_pvhe<<<blocks(2 * m->E), kThreads, 0, s>>>(V, m->vhe);
  k_pring<<<blocks(m->n), kThreads, 0, s>>>(V, m->vhe, layout == MCL_LAYOUT_COLUMN, max_ring, ring_dev, offs_dev);
  PCK(cudaGetLastError());
  PCK(cudaMemcpyAsync(m->cnt_host, m->cnt, sizeof(PCount), cudaMemcpyDeviceToHost, s));
  PCK(cudaStreamSynchronize(s));
  if (m->cnt_host->error)
    return mcl::fail((int)m->cnt_host->error,
                     "mcl_periodic_one_ring: malformed mesh (site " + std::to_string(m->cnt_host->error_site) + ")");
  if (truncated) *truncated = (int64_t)m->cnt_host->truncated;
  return MCL_OK;
}

int mcl_periodic_frnn(mcl_periodic* m, float r, int max_frnn, int layout, int32_t* out_dev, uint8_t* offs_dev,
                      void* stream, int64_t* truncated) {
  if (!m || !out_dev || max_frnn < 1 || !(r >= 0.0f) || !(r < 0.5f * m->L) ||
      (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_frnn: bad arguments (0 <= r < L/2)");
  cudaStream_t s = (cudaStream_t)stream;
  const PView V = view(m);
  PCK(cudaMemsetAsync(m->cnt, 0, sizeof(PCount), s));
  PCK(cudaMemsetAsync(m->vhe, 0xFF, 4 * (size_t)m->n, s));  // vhe = -1: the largest candidate wins
  k_pvhe<<<blocks(2 * m->E), kThreads, 0, s>>>(V, m->vhe);
  k_pfrnn<<<blocks(m->n), kThreads, 0, s>>>(V, m->vhe, r * r, layout == MCL_LAYOUT_COLUMN, max_frnn, out_dev, offs_dev);
  PCK(cudaGetLastError());
  PCK(cudaMemcpyAsync(m->cnt_host, m->cnt, sizeof(PCount), cudaMemcpyDeviceToHost, s));
  PCK(cudaStreamSynchronize(s));
  if (m->cnt_host->error)
    return mcl::fail((int)m->cnt_host->error,
                     "mcl_periodic_frnn: malformed mesh (site " + std::to_string(m->cnt_host->error_site) + ")");
  if (truncated) *truncated = (int64_t)m->cnt_host->truncated;
  return MCL_OK;
}

int mcl_periodic_closest(mcl_periodic* m, int max_ring, int layout, const int32_t* ring_dev, const uint8_t* offs_dev,
                         int32_t* closest_dev, void* stream) {
  if (!m || !ring_dev || !offs_dev || !closest_dev || max_ring < 1 ||
      (layout != MCL_LAYOUT_COLUMN && layout != MCL_LAYOUT_ROW))
    return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_closest: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  k_pclosest<<<blocks(m->n), kThreads, 0, s>>>(view(m), layout == MCL_LAYOUT_COLUMN, max_ring, ring_dev, offs_dev,
                                               closest_dev);
  PCK(cudaGetLastError());
  return MCL_OK;
}

}  // extern "C"
