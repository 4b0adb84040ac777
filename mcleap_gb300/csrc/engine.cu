// GB300 kinetic Delaunay engine: the persistent step kernel and its phases.
//
// One cooperative launch runs a whole kinetic step on the device:
//
//   move      new = old + d (or + v*dt), corners fixed   [DeviceTriangulation::movePoints,
//                                                          include/Device_Triangulation.h:395-410]
//   classify  every edge: orientation of both faces, incircle of the quad;
//             non-Delaunay edges go to a work-list       [delonize / untangle checks,
//                                                          include/Device_Triangulation.h:31-116]
//   repair    only when a face is inverted (the reference's untangle,
//             include/Device_Triangulation.h:422-495, handles only its B/C cases):
//             (1) revert vertices of non-positive faces to their old positions
//                 until every face is positive;
//             (2) remove the reverted vertices (flip each to degree 3, merge);
//             (3) Lawson to Delaunay;
//             (4) reinsert them at their new positions in parallel rounds
//                 (locate by walking, 1-to-3 / 2-to-4 split, Lawson).
//   lawson    parallel flip rounds over the work-list until it is empty
//             [delonize2, include/Device_Triangulation.h:324-351]: a candidate
//             flips when its hashed priority beats every candidate sharing a
//             face with it, so each round flips an independent set and the
//             highest-priority candidate always flips (no livelock).
//
// Rounds are separated by grid-wide barriers; nothing returns to the host
// between rounds.  The same insertion rounds build the initial triangulation.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace cg = cooperative_groups;

namespace mcl {

constexpr int kThreads = 256;
constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Warp-aggregated append to a global work-list: one atomicAdd per warp that
// has items, no block barrier (so warps never wait for each other between
// loop iterations and memory latency overlaps freely).  All 32 lanes of the
// warp must call it together; lanes without items pass k = 0.
template <int K>
__device__ __forceinline__ void warp_push(const int (&mine)[K], int k, int* gl, int* gcount, int gcap,
                                          DevState* st) {
  const int lane = threadIdx.x & 31;
  int x = k;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  const int total = __shfl_sync(kFull, x, 31);
  if (total == 0) return;
  int base = 0;
  if (lane == 31) base = atomicAdd(gcount, total);
  base = __shfl_sync(kFull, base, 31);
  const int off = base + x - k;
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (j < k) {
      if (off + j < gcap) __stcg(gl + off + j, mine[j]);
      else if (atomicCAS(&st->status, MCL_OK, MCL_ERR_CAPACITY) == MCL_OK) st->site = __LINE__;
    }
  }
}

#define set_error(P, code) flag_error_at(P, code, __LINE__)

// A per-thread count added to a global counter with one atomic per warp (every
// lane calls it): after a pass in which most threads count something, one
// atomic per thread on a single address would queue for tens of microseconds.
template <typename T>
__device__ __forceinline__ void warp_add(T* p, long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(p, (T)v);
}

// A warp's appends to a global list gathered in a shared-memory buffer of
// kWarpBuf entries and written out with one atomicAdd per flush (when the next
// append could overflow it, and at the end of the pass): a pass whose every
// warp appends on most iterations (the classification of a step that moves
// every vertex by a random walk) would otherwise queue thousands of atomics on
// one counter.  `n` is the same in every lane; calls are warp-uniform.
constexpr int kWarpBuf = 128;
struct WarpBuf {
  int* buf;  // this warp's kWarpBuf slots
  int n;
};
__device__ __forceinline__ void wb_flush(WarpBuf& b, int* gl, int* gcount, int gcap, DevState* st) {
  if (b.n == 0) return;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(gcount, b.n);
  base = __shfl_sync(kFull, base, 0);
  for (int i = lane; i < b.n; i += 32) {
    if (base + i < gcap) __stcg(gl + base + i, b.buf[i]);
    else if (atomicCAS(&st->status, MCL_OK, MCL_ERR_CAPACITY) == MCL_OK) st->site = __LINE__;
  }
  __syncwarp();  // every lane has read the buffer before it is refilled
  b.n = 0;
}
template <int K>
__device__ __forceinline__ void wb_push(WarpBuf& b, const int (&mine)[K], int k, int* gl, int* gcount, int gcap,
                                        DevState* st) {
  static_assert(32 * K <= kWarpBuf, "one append must fit an empty buffer");
  const int lane = threadIdx.x & 31;
  int x = k;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  const int total = __shfl_sync(kFull, x, 31);
  if (total == 0) return;
  if (b.n + total > kWarpBuf) wb_flush(b, gl, gcount, gcap, st);
  const int off = b.n + x - k;
#pragma unroll
  for (int j = 0; j < K; ++j)
    if (j < k) b.buf[off + j] = mine[j];
  __syncwarp();  // the entries are visible to the lanes of a later flush
  b.n += total;
}

// This thread's position in the spread order used by whole-grid loops over a
// work-list: warp slot w of block b has spread index w * gridDim.x + b, so a
// short list is dealt out one warp per block (across every SM) instead of
// filling the first blocks.  Its item chains are latency-bound, and packed
// onto a few SMs their scattered loads, stores and atomics queue behind each
// other in those SMs' memory pipelines.  A permutation of the global thread
// ids; the warp's first lane has index spread_tid() - lane.
__device__ __forceinline__ int spread_tid() {
  return (int)(((threadIdx.x >> 5) * gridDim.x + blockIdx.x) << 5) + (int)(threadIdx.x & 31);
}

__device__ __forceinline__ bool enqueue_once(const KParams& P, int e, unsigned stamp) {
  return atomicMax(P.qmark + e, stamp) < stamp;
}

// Append v to a global list from divergent code: the threads that reach the
// call together share one atomicAdd (their coalesced group's leader).
__device__ __forceinline__ void push_coalesced(const KParams& P, int* list, int* count, int cap, int v) {
  cg::coalesced_group grp = cg::coalesced_threads();
  int base = 0;
  if (grp.thread_rank() == 0) base = atomicAdd(count, (int)grp.size());
  base = grp.shfl(base, 0);
  const int at = base + (int)grp.thread_rank();
  if (at < cap) __stcg(list + at, v);
  else flag_error(P, MCL_ERR_CAPACITY);
}

// The repair's final Lawson pass starts from every edge its removals and
// splits touched: each is marked (stamp mk in qmark, no return value waited
// for) and appended, with the others of its removal or split, to work-list 0
// after the classification's non-Delaunay edges (one atomicAdd per removal or
// split).  Appends may repeat an edge; before the pass the list is deduplicated
// when it is short, and rebuilt from the marks by a pass over every edge when
// it is long or did not fit (mark_ovf).  mk == 0 marks nothing.
__device__ __forceinline__ void mark_edge(const KParams& P, int e, unsigned mk) {
  if (mk && e >= 0 && e < P.E) atomicMax(P.qmark + e, mk);
}
__device__ __forceinline__ int reserve_marks(const KParams& P, unsigned mk, int cnt) {
  return (mk && P.append_marks) ? atomicAdd(&P.st->wl_count[0], cnt) : -1;
}
__device__ __forceinline__ void append_mark(const KParams& P, int base, int j, int cnt, int e) {
  if (base < 0) return;
  if (base + cnt <= P.E) __stcg(P.wl0 + base + j, e);
  else if (j == 0) P.st->mark_ovf = 1;
}

// Called by every thread of the block (it holds a block barrier).
__device__ void flush_counters(const KParams& P, LocalCounters& lc) {
  // the common counter is reduced over the block (one atomic per block: one
  // per warp on a single address cost microseconds at the end of every step),
  // atomics for the rare ones
  __shared__ unsigned long long part[kThreads / 32];
  unsigned long long inc = lc.incircle;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) inc += __shfl_down_sync(kFull, inc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    if (t) atomicAdd(&P.st->c[C_INCIRCLE], t);
  }
  if (lc.incircle_fp64) atomicAdd(&P.st->c[C_INCIRCLE_FP64], (unsigned long long)lc.incircle_fp64);
  if (lc.incircle_exact) atomicAdd(&P.st->c[C_INCIRCLE_EXACT], (unsigned long long)lc.incircle_exact);
  if (lc.orient_fp64) atomicAdd(&P.st->c[C_ORIENT_FP64], (unsigned long long)lc.orient_fp64);
  if (lc.orient_exact) atomicAdd(&P.st->c[C_ORIENT_EXACT], (unsigned long long)lc.orient_exact);
  if (lc.sos) atomicAdd(&P.st->c[C_SOS], (unsigned long long)lc.sos);
  if (lc.overflow) {
    atomicAdd(&P.st->c[C_OVERFLOW], 1ull);
    set_error(P, MCL_ERR_PREDICATE);
  }
}

// ---------------------------------------------------------------------------
// New position of v for a fused move: pos_old + displacement (or + v*dt);
// fixed vertices (bounding corners) stay.  pos_old, disp, vel and dt are
// read-only for the whole launch, so they go through the read-only cache.
// Every load is issued before the fixed-vertex test (no load waits on another).
__device__ __forceinline__ float2 moved_pos(const KParams& P, int v) {
  const float2 p = __ldg(P.pos_old + v);
  const bool fixed = __ldg(P.vfix + v) != 0;
  float2 q = p;
  if (P.move_mode == MOVE_DISPLACE) {
    const float2 d = __ldg(P.disp + v);
    q.x = fadd(p.x, d.x);
    q.y = fadd(p.y, d.y);
  } else if (P.move_mode == MOVE_INTEGRATE) {
    const float2 u = __ldg(P.vel + v);
    const float t = __ldg(P.dt + v);
    q.x = fadd(p.x, fmul(u.x, t));
    q.y = fadd(p.y, fmul(u.y, t));
  }
  return fixed ? p : q;
}

// Phase A of a flip round for edge e (already known to be non-Delaunay): claim
// both faces with a priority key, remember the face ids for phase B.
__device__ __forceinline__ void claim_edge_with(const KParams& P, int e, int4 w, unsigned sc) {
  const int fa = min(2 * e, min(w.x, w.y)), fb = min(2 * e + 1, min(w.z, w.w));
  const unsigned long long key = ((unsigned long long)sc << 32) | (unsigned)(~mix32((unsigned)e ^ sc));
  atomicMax(P.claim + fa, key);
  atomicMax(P.claim + fb, key);
  __stcg(P.efa + e, make_int2(fa, fb));
  __stcg(P.cand + e, sc);
}
__device__ __forceinline__ void claim_edge(const KParams& P, int e, unsigned sc) {
  claim_edge_with(P, e, ld_en(P, e), sc);
}

// Full predicate ladder for one edge: counts its non-positive faces into `bad`
// and returns true when both faces are positive and the edge is non-Delaunay.
template <bool kFixedPos>
__device__ __forceinline__ bool resolve_edge(const KParams& P, int e, LocalCounters& lc, int& bad) {
  const int4 q = ld_ev(P, e);
  const float2 a = ldpos_t<kFixedPos>(P, q.x), b = ldpos_t<kFixedPos>(P, q.y);
  const float2 c = q.z >= 0 ? ldpos_t<kFixedPos>(P, q.z) : a;
  const float2 d = q.w >= 0 ? ldpos_t<kFixedPos>(P, q.w) : a;
  const int sa = q.z >= 0 ? orient_v(P, a, b, c, lc) : 1;
  const int sb = q.w >= 0 ? orient_v(P, b, a, d, lc) : 1;
  if (sa <= 0 || sb <= 0) {
    bad += (sa <= 0) + (sb <= 0);
    return false;
  }
  if (q.z < 0 || q.w < 0) return false;
  lc.incircle++;
  return incircle_sos(a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, q.x, q.y, q.z, q.w, &lc, &lc.overflow) > 0;
}

// ---------------------------------------------------------------------------
// Phase: (move +) classify every edge.  With a move, a vertex pass writes the
// new positions first (one grid barrier).  Counts non-positive faces;
// non-Delaunay edges of positive faces are queued on work-list 0 and claim
// their faces for the first flip round (stamp sc).
//
// The edge loop evaluates only the FP32 filters: an out-of-line call to the
// FP64 / exact / perturbation stages inside the loop would cost more than the
// whole filter.  Edges the filters cannot decide (a few per million) go to the
// hard list, which is resolved with the full ladder after the barrier; the
// caller must call phase_classify_hard before reading `inverted`.
__device__ __forceinline__ void timeline(const KParams& P, int slot) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && slot < kTimeline) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    P.st->ts[slot] = t;
  }
}

// the latest time any block reached this point
__device__ __forceinline__ void timeline_max(const KParams& P, int slot) {
  if (threadIdx.x == 0 && slot >= 43 && slot < 47) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    atomicMax(&P.st->tsmax[slot - 43], t);
  }
}

// Edges per thread and iteration of the classification pass; vertices per
// thread and iteration of its move pass.
constexpr int kClassifyUnroll = 4;
constexpr int kMoveUnroll = 4;

// The classification streams the edge records through shared memory one
// iteration ahead of their use (cp.async, 16 bytes per record, L2-coherent):
// kEvStages iterations of kClassifyUnroll records per thread.  Each thread
// copies and reads only its own slots, so completion is a cp.async.wait_group
// of the thread itself and no block barrier is involved.  The first
// iteration's records are requested before the move pass, which hides them.
constexpr int kEvStages = 2;
__shared__ int4 s_ev[kEvStages][kClassifyUnroll][kThreads];
// the classification's append buffers (non-Delaunay edges, edges of a face
// turned over): kWarpBuf entries per warp each
__shared__ int s_wbuf[2][kThreads / 32][kWarpBuf];

__device__ __forceinline__ void cp_async16(int4* smem, const int4* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Request the records of the classification iteration at `base` into stage
// `st` (one commit group, empty past the end).
__device__ __forceinline__ void stage_edges(const KParams& P, int base, int st) {
#pragma unroll
  for (int j = 0; j < kClassifyUnroll; ++j) {
    const int ei = base + j * blockDim.x + threadIdx.x;
    if (ei < P.E_it) cp_async16(&s_ev[st][j][threadIdx.x], P.ev + edge_at(P, ei));
  }
  cp_async_commit();
}

// Iterate the outgoing half-edges of v counter-clockwise.
template <typename F>
__device__ bool for_spokes(const KParams& P, int v, F f) {
  const int s0 = ld_i(P.vhe + v);
  if (s0 < 0 || s0 >= 2 * P.E) return false;
  int h = s0;
  for (int k = 0; k < 1024; ++k) {
    f(h);
    h = he_prev(P, h) ^ 1;
    if (h < 0 || h >= 2 * P.E) return false;
    if (h == s0) return true;
  }
  return false;
}

// A step moves few vertices (an aggregation whose walkers froze, a single
// point moved): classify only the edges of their stars and the sides opposite
// them (the edges whose quads hold a moved vertex), each once per launch
// (stamp qstamp in `win`), with the full predicate ladder; work-lists and
// claims as the full pass makes them.  Worth it while the movers touch well
// under all the edges.
constexpr int kSparseEdgesPerMover = 32;

__device__ __forceinline__ void push_one(const KParams& P, int* list, int* count, int e) {
  const int at = atomicAdd(count, 1);
  if (at < P.E) list[at] = e;
  else flag_error(P, MCL_ERR_CAPACITY);
}

template <bool kFixedPos>
__device__ void classify_one(const KParams& P, int e, unsigned qstamp, unsigned sc, LocalCounters& lc, int& bad) {
  if (e < 0 || e >= P.E || atomicMax(P.win + e, qstamp) >= qstamp) return;
  const int4 q = ld_ev(P, e);
  if (q.x < 0) return;
  if (bad_v(P, q.x) || bad_v(P, q.y) || q.z >= P.V || q.w >= P.V) {
    flag_error(P, MCL_ERR_DEGENERATE_INPUT);
    return;
  }
  const int bad0 = bad;
  if (resolve_edge<kFixedPos>(P, e, lc, bad) && enqueue_once(P, e, qstamp)) {
    claim_edge(P, e, sc);
    push_one(P, P.wl0, &P.st->wl_count[0], e);
  }
  if (bad != bad0) push_one(P, P.wl1, &P.st->wl_count[1], e);
}

template <bool kFixedPos>
__device__ void classify_movers(const KParams& P, int nm, unsigned qstamp, unsigned sc, LocalCounters& lc) {
  const int stride = gridDim.x * blockDim.x;
  int bad = 0;
  for (int i = spread_tid(); i < nm; i += stride) {
    const int v = ld_i(P.vl0 + i);
    const bool ok = for_spokes(P, v, [&](int h) {
      classify_one<kFixedPos>(P, h >> 1, qstamp, sc, lc, bad);
      classify_one<kFixedPos>(P, he_next(P, h) >> 1, qstamp, sc, lc, bad);
    });
    if (!ok) flag_error(P, MCL_ERR_DEGENERATE_INPUT);
  }
  warp_add(&P.st->inverted, bad);
}

template <bool kFixedPos>
__device__ void phase_classify(cg::grid_group& g, const KParams& P, unsigned qstamp, unsigned sc,
                               LocalCounters& lc) {
  const int stride = gridDim.x * blockDim.x;
  constexpr int U = kClassifyUnroll;
  const int first = blockIdx.x * blockDim.x * U;
  stage_edges(P, first, 0);
  if (P.move_mode != MOVE_NONE) {
    // kMoveUnroll vertices per thread and iteration, every load before any
    // store (the pass is a stream: its loads must overlap)
    // The vertices that actually move are listed (work-list vl0, free until
    // the repair) when the last launch moved few: when they are few, only the
    // edges whose quads hold one of them are classified (every other edge
    // kept the positions of the last step, which left the mesh Delaunay).
    // A launch that moves most vertices after one that did lists nothing
    // (listing them would wait on an append per warp and iteration); the
    // movers are counted either way, for the next launch's choice.
    constexpr int UM = kMoveUnroll;
    const bool listing =
        P.sparse_ok && (long long)ld_i(&P.st->movers_last) * kSparseEdgesPerMover < (long long)P.E_it;
    int moved = 0;
    for (int base = blockIdx.x * blockDim.x * UM; base < P.V_it; base += stride * UM) {
      int v[UM];
      float2 np[UM];
#pragma unroll
      for (int j = 0; j < UM; ++j) {
        const int i = base + j * blockDim.x + threadIdx.x;
        v[j] = i < P.V_it ? vert_at(P, i) : -1;
        if (v[j] >= 0) np[j] = moved_pos(P, v[j]);
      }
      int mv[UM];
      int km = 0;
#pragma unroll
      for (int j = 0; j < UM; ++j)
        if (v[j] >= 0) {
          __stcg(P.pos + v[j], np[j]);
          const float2 po = __ldg(P.pos_old + v[j]);
          if (__float_as_uint(np[j].x) != __float_as_uint(po.x) || __float_as_uint(np[j].y) != __float_as_uint(po.y))
            mv[km++] = v[j];
        }
      moved += km;
      if (listing && __any_sync(kFull, km > 0)) warp_push(mv, km, P.vl0, &P.st->vl_count[0], P.V, P.st);
    }
    warp_add(&P.st->movers_now, moved);
    if (kFixedPos) timeline_max(P, 43);
    g.sync();
    if (kFixedPos) timeline_max(P, 44);
    const int nm = ld_i(&P.st->vl_count[0]);
    if (listing && (long long)nm * kSparseEdgesPerMover < (long long)P.E_it) {
      cp_async_wait<0>();  // the prefetched records are not used
      classify_movers<kFixedPos>(P, nm, qstamp, sc, lc);
      if (kFixedPos) timeline_max(P, 45);
      return;
    }
  }
  int bad = 0;
  unsigned ninc = 0;
  int def0 = -1, def1 = -1;  // edges deferred to the full ladder after the loop
  WarpBuf wnd{s_wbuf[0][threadIdx.x >> 5], 0}, winv{s_wbuf[1][threadIdx.x >> 5], 0};
  // kClassifyUnroll edges per thread and iteration, their records and
  // positions loaded before any is evaluated (memory-level parallelism: the
  // pass is latency-bound on the position gathers); edge j of the iteration
  // at base is base + j * blockDim.x + threadIdx.x, so every load stays
  // coalesced across the warp.
  int it = 0;
  for (int base = first; base < P.E_it; base += stride * U, ++it) {
    stage_edges(P, base + stride * U, (it + 1) % kEvStages);
    cp_async_wait<kEvStages - 1>();  // this iteration's records have landed
    int4 q[U];
    int e[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int ei = base + j * blockDim.x + threadIdx.x;
      e[j] = ei < P.E_it ? edge_at(P, ei) : -1;
      q[j] = e[j] >= 0 ? s_ev[it % kEvStages][j][threadIdx.x] : make_int4(-1, -1, -1, -1);
    }
    float2 pa[U], pb[U], pc[U], pd[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int4 r = q[j];
      const bool ok = r.x >= 0 && !(bad_v(P, r.x) || bad_v(P, r.y) || r.z >= P.V || r.w >= P.V);
      if (r.x >= 0 && !ok) {
        flag_error(P, MCL_ERR_DEGENERATE_INPUT);
        q[j].x = -1;
      }
      if (ok) {
        pa[j] = ldpos_t<kFixedPos>(P, r.x);
        pb[j] = ldpos_t<kFixedPos>(P, r.y);
        pc[j] = r.z >= 0 ? ldpos_t<kFixedPos>(P, r.z) : pa[j];
        pd[j] = r.w >= 0 ? ldpos_t<kFixedPos>(P, r.w) : pa[j];
      }
    }
    int mine[U];
    int k = 0;
    int hard[U];
    int kh = 0;
    int inv[U];
    int ki = 0;
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int4 r = q[j];
      if (r.x < 0) continue;
      const float2 a = pa[j], b = pb[j], c = pc[j], d = pd[j];
      const int sa = r.z >= 0 ? orient2d_fp32(a.x, a.y, b.x, b.y, c.x, c.y) : 1;
      const int sb = r.w >= 0 ? orient2d_fp32(b.x, b.y, a.x, a.y, d.x, d.y) : 1;
      bool defer = false;
      if (sa == 2 || sb == 2) {
        defer = true;
      } else if (sa <= 0 || sb <= 0) {
        bad += (sa <= 0) + (sb <= 0);
        inv[ki++] = e[j];
      } else if (r.z >= 0 && r.w >= 0) {
        ++ninc;
        const int si = incircle_fp32(a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y);
        if (si == 2) {
          defer = true;
        } else if (si > 0) {
          // each edge comes once in this pass and qstamp is the launch's
          // first stamp: the queue mark is a plain store (no atomic waited for)
          __stcg(P.qmark + e[j], qstamp);
          claim_edge(P, e[j], sc);
          mine[k++] = e[j];
        }
      }
      if (defer) {
        if (def0 < 0) def0 = e[j];
        else if (def1 < 0) def1 = e[j];
        else hard[kh++] = e[j];
      }
    }
    if (__any_sync(kFull, k > 0)) wb_push(wnd, mine, k, P.wl0, &P.st->wl_count[0], P.E, P.st);
    if (__any_sync(kFull, kh > 0)) warp_push(hard, kh, P.hard, &P.st->hard_count, P.E, P.st);
    // edges with a non-positive face: the repair's first send-back pass
    // starts from them (work-list 1 is free until the flip rounds)
    if (__any_sync(kFull, ki > 0)) wb_push(winv, inv, ki, P.wl1, &P.st->wl_count[1], P.E, P.st);
  }
  wb_flush(wnd, P.wl0, &P.st->wl_count[0], P.E, P.st);
  wb_flush(winv, P.wl1, &P.st->wl_count[1], P.E, P.st);
  cp_async_wait<0>();  // nothing left in flight into the staging slots
  // the deferred edges, with the full predicate ladder (out of the loop, so
  // the out-of-line calls do not weigh on the loop above)
  {
    int mine[2];
    int k = 0;
    int inv[2];
    int ki = 0;
    const int defs[2] = {def0, def1};
    for (int j = 0; j < 2; ++j) {
      const int e = defs[j];
      if (e < 0) continue;
      const int bad0 = bad;
      if (resolve_edge<kFixedPos>(P, e, lc, bad) && enqueue_once(P, e, qstamp)) {
        claim_edge(P, e, sc);
        mine[k++] = e;
      }
      if (bad != bad0) inv[ki++] = e;
    }
    if (__any_sync(kFull, k > 0)) warp_push(mine, k, P.wl0, &P.st->wl_count[0], P.E, P.st);
    if (__any_sync(kFull, ki > 0)) warp_push(inv, ki, P.wl1, &P.st->wl_count[1], P.E, P.st);
  }
  lc.incircle += ninc;
  warp_add(&P.st->inverted, bad);
  if (kFixedPos) timeline_max(P, 45);
}

// Resolve the hard list of phase_classify (after its barrier) with the full
// predicate ladder.  Returns after a barrier when there was anything to do.
template <bool kFixedPos>
__device__ void phase_classify_hard(cg::grid_group& g, const KParams& P, unsigned qstamp, unsigned sc,
                                    LocalCounters& lc) {
  const int n = ld_i(&P.st->hard_count);
  if (n == 0) return;  // uniform: read after the classification barrier
  const int stride = gridDim.x * blockDim.x;
  int bad = 0;
  const int lane = threadIdx.x & 31;
  for (int base = spread_tid() - lane; base < n; base += stride) {
    const int i = base + lane;
    int mine[1];
    int k = 0;
    int inv[1];
    int ki = 0;
    if (i < n) {
      const int e = ld_i(P.hard + i);
      const int bad0 = bad;
      if (resolve_edge<kFixedPos>(P, e, lc, bad) && enqueue_once(P, e, qstamp)) {
        claim_edge(P, e, sc);
        mine[k++] = e;
      }
      if (bad != bad0) inv[ki++] = e;
    }
    if (__any_sync(kFull, k > 0)) warp_push(mine, k, P.wl0, &P.st->wl_count[0], P.E, P.st);
    if (__any_sync(kFull, ki > 0)) warp_push(inv, ki, P.wl1, &P.st->wl_count[1], P.E, P.st);
  }
  if (bad) atomicAdd(&P.st->inverted, bad);
  g.sync();
}

__device__ __forceinline__ void timeline_remove(const KParams& P, int slot) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && slot < 64) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    P.st->ts_remove[slot] = t;
  }
}

__device__ __forceinline__ void timeline_insert(const KParams& P, int round, int k) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && round < 16) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    P.st->ts_insert[4 * round + k] = t;
  }
}

// ---------------------------------------------------------------------------
// Lawson flip rounds starting from work-list `src`.  A round is two phases:
//   A  every queued edge that is still non-Delaunay claims its two faces with
//      a hashed priority (atomicMax on the face's smallest half-edge);
//   B  an edge that holds both claims flips and queues its four wing edges;
//      other candidates queue themselves again.
// Winners share no face, so their writes never overlap; the candidate with the
// highest priority always wins both faces, so every round flips at least once.
// If pre_sc != 0 the first round's phase A was done by the classification.
// One flip round over `in[0..n)` by the threads [t0, t0+nt) (a whole grid or a
// single block); `sync` is the matching barrier.
template <bool kFixedPos, typename Sync>
__device__ __forceinline__ int lawson_round(const KParams& P, const int* in, int n, int* out, int* out_count,
                                            unsigned sc, unsigned sq, bool do_phase_a, int t0, int nt,
                                            LocalCounters& lc, Sync sync) {
  if (do_phase_a) {
    for (int i = t0; i < n; i += nt) {
      const int e = ld_i(in + i);
      const int4 q = ld_ev(P, e);
      const int4 w = ld_en(P, e);  // loaded with q: no load waits for the predicate
      if (edge_illegal<kFixedPos>(P, q, lc)) claim_edge_with(P, e, w, sc);
    }
    sync();
  }
  int flips = 0;
  const int lane = threadIdx.x & 31;
  WarpBuf wb{s_wbuf[0][threadIdx.x >> 5], 0};
  for (int base = t0 - lane; base < n; base += nt) {
    const int i = base + lane;
    int mine[4];
    int k = 0;
    if (i < n) {
      const int e = ld_i(in + i);
      // Everything a winner needs is loaded together with its claim test: a
      // winner shares no face with another winner, so no flip of this round
      // writes its records, and only its own flip can move vhe[a] off 2e
      // or vhe[b] off 2e+1.
      const unsigned c = (unsigned)ld_i(reinterpret_cast<const int*>(P.cand) + e);
      const int2 f = __ldcg(P.efa + e);
      const int4 q = ld_ev(P, e);
      const int4 w = ld_en(P, e);
      if (c == sc) {
        const unsigned long long key = ((unsigned long long)sc << 32) | (unsigned)(~mix32((unsigned)e ^ sc));
        const unsigned long long ka = __ldcg(P.claim + f.x), kb = __ldcg(P.claim + f.y);
        const int vha = bad_v(P, q.x) ? -1 : ld_i(P.vhe + q.x);
        const int vhb = bad_v(P, q.y) ? -1 : ld_i(P.vhe + q.y);
        if (ka == key && kb == key) {
          if (flip_edge_with(P, e, q, w, vha, vhb)) ++flips;
          const int wing[4] = {w.x >> 1, w.y >> 1, w.z >> 1, w.w >> 1};
          // the four queue marks issued together, their answers used after
          unsigned was[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) was[j] = atomicMax(P.qmark + wing[j], sq);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (was[j] < sq) mine[k++] = wing[j];
        } else if (enqueue_once(P, e, sq)) {
          mine[k++] = e;
        }
      }
    }
    if (__any_sync(kFull, k > 0)) wb_push(wb, mine, k, out, out_count, P.E, P.st);
  }
  wb_flush(wb, out, out_count, P.E, P.st);
  return flips;
}

// Rounds with at most this many queued edges run inside one block (block
// barriers instead of grid barriers); the rest of the grid waits.
constexpr int kTailItems = 2048;
// Default repair sub-steps per kinetic step (phase_substeps).  Off: on the
// uniform random-walk benchmarks (1M points, sigma = 0.1 x spacing; 512 meshes,
// 8.5M points) 4 and 8 sub-steps leave 25% and 4% of the sent-back vertices
// to removal, but each sub-step costs about as much as the removal and
// reinsertion rounds it saves (latency-bound star walks and flip rounds), so
// the step time does not improve.
constexpr int kSubsteps = 0;

// ---------------------------------------------------------------------------
// Lawson flip rounds starting from work-list `src`.  A round is two phases:
//   A  every queued edge that is still non-Delaunay claims its two faces with
//      a hashed priority (atomicMax on the face's smallest half-edge);
//   B  an edge that holds both claims flips and queues its four wing edges;
//      other candidates queue themselves again.
// Winners share no face, so their writes never overlap; the candidate with the
// highest priority always wins both faces, so every round flips at least once.
// If pre_sc != 0 the first round's phase A was done by the classification.
// With kLast (the launch's final phase) the grid does not wait for a
// single-block tail: the other blocks return at once and block 0 returns
// when the tail is done; only block 0's `stamp` is then current.
template <bool kFixedPos, bool kLast = false>
__device__ void phase_lawson(cg::grid_group& g, const KParams& P, int src, unsigned& stamp,
                             LocalCounters& lc, unsigned pre_sc) {
  const int stride = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  int flips = 0;
  for (int round = 0;; ++round) {
    const int n = ld_i(&P.st->wl_count[src]);
    if (n == 0) break;
    if (round >= P.max_rounds) {
      if (gtid == 0) set_error(P, MCL_ERR_NO_CONVERGENCE);
      break;
    }
    if (n <= P.tail_items) {
      // tail: block 0 finishes every remaining round on its own
      if (blockIdx.x == 0) {
        int s2 = src;
        unsigned st2 = stamp;
        for (int r2 = round; r2 < P.max_rounds; ++r2) {
          const int m = ld_i(&P.st->wl_count[s2]);
          if (m == 0) break;
          const int d2 = s2 ^ 1;
          // the first round's phase A may have been done by the classification
          // (then wl_count[d2] is still zero)
          const bool pre = r2 == 0 && pre_sc;
          const unsigned sc = pre ? pre_sc : st2++;
          const unsigned sq = st2++;
          if (threadIdx.x == 0) {
            if (!pre) P.st->wl_count[d2] = 0;
            P.st->c[C_LAWSON_ROUNDS] += 1;
          }
          __syncthreads();
          flips += lawson_round<kFixedPos>(P, s2 ? P.wl1 : P.wl0, m, d2 ? P.wl1 : P.wl0, &P.st->wl_count[d2], sc, sq,
                                           !pre, threadIdx.x, blockDim.x, lc, [] { __syncthreads(); });
          __syncthreads();
          timeline(P, 2 + (r2 < 40 ? r2 : 40));
          s2 = d2;
        }
        if (kLast) stamp = st2;
        else if (threadIdx.x == 0) P.st->tail_stamp = st2;
      }
      if (!kLast) {
        g.sync();
        stamp = (unsigned)ld_i(reinterpret_cast<const int*>(&P.st->tail_stamp));
      }
      break;
    }
    const int dst = src ^ 1;
    const int* in = src ? P.wl1 : P.wl0;
    int* out = dst ? P.wl1 : P.wl0;
    unsigned sc;
    bool phase_a = true;
    if (round == 0 && pre_sc) {
      sc = pre_sc;  // wl_count[dst] is still zero from the end of the last launch or phase
      phase_a = false;
      if (gtid == 0) P.st->c[C_LAWSON_ROUNDS] += 1;
    } else {
      sc = stamp++;
      if (gtid == 0) {
        P.st->wl_count[dst] = 0;
        P.st->c[C_LAWSON_ROUNDS] += 1;
      }
    }
    const unsigned sq = stamp++;
    flips += lawson_round<kFixedPos>(P, in, n, out, &P.st->wl_count[dst], sc, sq, phase_a, spread_tid(), stride, lc,
                                     [&] { g.sync(); });
    g.sync();
    timeline(P, 2 + (round < 40 ? round : 40));
    src = dst;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) flips += __shfl_down_sync(kFull, flips, o);
  if ((threadIdx.x & 31) == 0 && flips) atomicAdd(&P.st->c[C_LAWSON_FLIPS], (unsigned long long)flips);
}


// ---------------------------------------------------------------------------
// Repair (1): revert vertices of non-positive faces until all faces are positive.
__device__ __forceinline__ bool marked(const KParams& P, int v, unsigned fs) {
  return (unsigned)ld_i(P.vmark + v) == fs;
}

__device__ __forceinline__ float2 qpos(const KParams& P, int v, unsigned fs) {
  return marked(P, v, fs) ? P.pos_old[v] : ldpos(P, v);
}

// The list of the vertices the next fixpoint pass checks (their stars):
// pass p writes list p & 1 (vl0 / vl1) with count fix_list[p % 3].
__device__ __forceinline__ void list_for_next_pass(const KParams& P, int v, int pass) {
  push_coalesced(P, (pass & 1) ? P.vl1 : P.vl0, &P.st->fix_list[pass % 3], P.V, v);
}

// Where a fixpoint pass's marks go: appended at once from divergent code
// (MarkNow), or kept by the thread (at most two per work item) for one
// warp-wide buffered append afterwards (MarkLater).  A fresh vertex joins the
// list of every vertex sent back (`hard`) and the next pass's list; a vertex
// listed again joins the next pass's list.
struct MarkNow {
  const KParams& P;
  int pass;
  __device__ void fresh_vertex(int v) const {
    push_coalesced(P, P.hard, &P.st->fix_all, P.E, v);
    list_for_next_pass(P, v, pass);
  }
  __device__ void relist(int v) const { list_for_next_pass(P, v, pass); }
};
struct MarkLater {
  int nv[2], rl[2];
  int kn = 0, kr = 0;
  __device__ void fresh_vertex(int v) { nv[kn++ & 1] = v; }
  __device__ void relist(int v) { rl[kr++ & 1] = v; }
};

// A newly marked vertex records the pass that marked it in vloc (free until
// the insertion rounds) and goes to the sink.
template <typename Sink>
__device__ void mark_vertex(const KParams& P, int v, int& fresh, unsigned fs, int pass, Sink& sink) {
  if (!marked(P, v, fs) && (unsigned)atomicExch(P.vmark + v, (int)fs) != fs) {
    __stcg(P.vloc + v, pass);
    sink.fresh_vertex(v);
    ++fresh;
  }
}

// A non-positive face sends back one vertex per pass: the unmarked free vertex
// that moved farthest (ties: smallest id).  A face whose vertices are all back
// at their old positions is positive (the mesh was valid there), so every pass
// that still sees a bad face marks a vertex and the fixpoint ends.  Sending
// back fewer vertices means fewer removals and reinsertions; the result does
// not depend on the choice (every sent-back vertex is reinserted at its
// target).
// A bad face whose free vertices all turned out marked (by other faces of the
// same pass, after its orientation was read) is checked again next pass
// through the star of one of them.
template <typename Sink>
__device__ void mark_face(const KParams& P, int a, int b, int c, int& fresh, unsigned fs, int pass, Sink& sink) {
  const int t[3] = {a, b, c};
  int pick = -1, any = -1;
  float best = -1.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int v = t[k];
    if (P.vfix[v]) continue;
    if (marked(P, v, fs)) {
      any = v;
      continue;
    }
    const float2 pn = ldpos(P, v), po = P.pos_old[v];
    const float dx = __fsub_rn(pn.x, po.x), dy = __fsub_rn(pn.y, po.y);
    const float m2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (m2 > best || (m2 == best && v < pick)) { best = m2; pick = v; }
  }
  if (pick >= 0) {
    mark_vertex(P, pick, fresh, fs, pass, sink);
  } else if (any >= 0) {
    // vloc of a marked vertex holds a pass of this launch: list it once per pass
    if (atomicExch(P.vloc + any, pass) != pass) sink.relist(any);
    ++fresh;
  }
}

__device__ bool phase_fixpoint(cg::grid_group& g, const KParams& P, LocalCounters& lc, unsigned fs) {
  const int stride = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int pass = 0; pass < 256; ++pass) {
    // counters are triple-buffered: slot (pass+1)%3 was last read two barriers ago
    const int slot = pass % 3;
    if (gtid == 0) {
      P.st->fix_new[(pass + 1) % 3] = 0;
      P.st->fix_bad[(pass + 1) % 3] = 0;
      P.st->fix_list[(pass + 1) % 3] = 0;
      P.st->c[C_FIX_PASSES] += 1;
    }
    int fresh = 0, bad = 0;
    if (pass == 0) {
      // every face the classification found non-positive, once per edge
      // side (its edges are on work-list 1)
      // (most warps mark on most iterations: the marks go through the
      // warp's append buffers, idle after the classification)
      const int nb = ld_i(&P.st->wl_count[1]);
      const int lane = threadIdx.x & 31;
      WarpBuf whard{s_wbuf[0][threadIdx.x >> 5], 0}, wnext{s_wbuf[1][threadIdx.x >> 5], 0};
      int* nlist = (pass & 1) ? P.vl1 : P.vl0;
      int* ncount = &P.st->fix_list[pass % 3];
      for (int base = spread_tid() - lane; base < nb; base += stride) {
        const int ii = base + lane;
        MarkLater ml;
        if (ii < nb) {
          const int e = ld_i(P.wl1 + ii);
          const int4 q = ld_ev(P, e);
          if (q.x >= 0 && (bad_v(P, q.x) || bad_v(P, q.y) || q.z >= P.V || q.w >= P.V)) {
            flag_error(P, MCL_ERR_DEGENERATE_INPUT);
          } else if (q.x >= 0) {
            const float2 a = qpos(P, q.x, fs), b = qpos(P, q.y, fs);
            if (q.z >= 0 && orient_v(P, a, b, qpos(P, q.z, fs), lc) <= 0) {
              ++bad;
              mark_face(P, q.x, q.y, q.z, fresh, fs, pass, ml);
            }
            if (q.w >= 0 && orient_v(P, b, a, qpos(P, q.w, fs), lc) <= 0) {
              ++bad;
              mark_face(P, q.y, q.x, q.w, fresh, fs, pass, ml);
            }
          }
        }
        if (__any_sync(kFull, ml.kn > 0)) {
          wb_push(whard, ml.nv, ml.kn, P.hard, &P.st->fix_all, P.E, P.st);
          wb_push(wnext, ml.nv, ml.kn, nlist, ncount, P.V, P.st);
        }
        if (__any_sync(kFull, ml.kr > 0)) wb_push(wnext, ml.rl, ml.kr, nlist, ncount, P.V, P.st);
      }
      wb_flush(whard, P.hard, &P.st->fix_all, P.E, P.st);
      wb_flush(wnext, nlist, ncount, P.V, P.st);
    } else {
      // only a face with a vertex sent back (or listed again) in the last pass
      // can have changed sign: the stars of the last pass's list
      const int nl = ld_i(&P.st->fix_list[(pass - 1) % 3]);
      const int* lst = ((pass - 1) & 1) ? P.vl1 : P.vl0;
      for (int ii = spread_tid(); ii < nl; ii += stride) {
        const int v = ld_i(lst + ii);
        const float2 pv = qpos(P, v, fs);
        const bool ok = for_spokes(P, v, [&](int h) {
          const int d = he_origin(P, h ^ 1), a = he_apex(P, h);
          if (bad_v(P, d) || a < 0 || bad_v(P, a)) return;  // hull side: no face
          if (orient_v(P, pv, qpos(P, d, fs), qpos(P, a, fs), lc) <= 0) {
            ++bad;
            MarkNow now{P, pass};
            mark_face(P, v, d, a, fresh, fs, pass, now);
          }
        });
        if (!ok) flag_error(P, MCL_ERR_DEGENERATE_INPUT);
      }
    }
    warp_add(&P.st->fix_new[slot], fresh);
    warp_add(&P.st->fix_bad[slot], bad);
    g.sync();
    if (pass < 16) timeline_remove(P, 48 + pass);
    const int nfresh = ld_i(&P.st->fix_new[slot]);
    const int nbad = ld_i(&P.st->fix_bad[slot]);
    if (nfresh == 0) {
      if (nbad) {
        if (gtid == 0) set_error(P, MCL_ERR_DEGENERATE_INPUT);
        return false;
      }
      return true;
    }
  }
  if (gtid == 0) set_error(P, MCL_ERR_NO_CONVERGENCE);
  return false;
}

// ---------------------------------------------------------------------------
// Removal by ear clipping: retriangulate the star polygon of v (its link cycle,
// v left out) with exact orientation tests.  Used when no spoke flip is valid,
// which happens with exactly collinear neighbours (points clamped onto the
// same line of the box, lattices).  A simple polygon always has an ear whose
// closed triangle holds no other polygon vertex, so this always completes.
// The k spoke edges become k-3 diagonals plus the 3 free edges of v.
constexpr int kEarMax = 128;
// Loads per group issued before any of their values is stored: a loop that
// stores each loaded value (to local or shared memory) before the next load
// waits for every load in turn.
constexpr int kGather = 8;

// The star polygon under ear clipping: cyclic links and corner positions.
// Any star up to kEarMax corners: local arrays.
struct LocalPoly {
  int nx_[kEarMax], pv_[kEarMax];
  float2 q_[kEarMax];
  __device__ __forceinline__ int nx(int j) const { return nx_[j]; }
  __device__ __forceinline__ int pv(int j) const { return pv_[j]; }
  __device__ __forceinline__ void set_nx(int j, int x) { nx_[j] = x; }
  __device__ __forceinline__ void set_pv(int j, int x) { pv_[j] = x; }
  __device__ __forceinline__ float2 q(int j) const { return q_[j]; }
  __device__ __forceinline__ void set_q(int j, float2 x) { q_[j] = x; }
};

// Stars of up to kSmallStar corners: links packed four bits each in
// registers and positions in this thread's slots of the classification's
// shared staging array (idle during repair), which the ear search reads
// O(k^2) times.
constexpr int kSmallStar = 16;
struct SmallPoly {
  unsigned long long nx_ = 0, pv_ = 0;
  __device__ __forceinline__ static float2* slot(int j) {
    return reinterpret_cast<float2*>(&s_ev[(j >> 3) & 1][(j >> 1) & 3][threadIdx.x]) + (j & 1);
  }
  __device__ __forceinline__ int nx(int j) const { return (int)((nx_ >> (4 * j)) & 15u); }
  __device__ __forceinline__ int pv(int j) const { return (int)((pv_ >> (4 * j)) & 15u); }
  __device__ __forceinline__ void set_nx(int j, int x) {
    nx_ = (nx_ & ~(15ull << (4 * j))) | ((unsigned long long)x << (4 * j));
  }
  __device__ __forceinline__ void set_pv(int j, int x) {
    pv_ = (pv_ & ~(15ull << (4 * j))) | ((unsigned long long)x << (4 * j));
  }
  __device__ __forceinline__ float2 q(int j) const { return *slot(j); }
  __device__ __forceinline__ void set_q(int j, float2 x) { *slot(j) = x; }
};

// Clip the star polygon of v given its k spokes sp (counter-clockwise), the
// link half-edges lk (lk[i] = next(sp[i]), the side of face i opposite v),
// their origins w and, in poly, their positions; pv is v's position, at which
// its star is valid; bnd is scratch of size k.
//
// Ears by a constant-time test while v stays strictly inside the kernel of the
// remaining polygon (checked at the start: every face of the star positive):
// then the corners are in strictly increasing angle around v, and a convex
// corner b between a and c whose diagonal a -> c has v strictly on its left
// spans an angle below 180 degrees from v; the cone of that angle is convex,
// holds the triangle abc and no other corner, so abc is an ear, and the new
// side a -> c keeps v strictly inside the kernel.  Only when no corner passes
// does the general test run (every other corner checked against the
// triangle, O(k) per candidate); an ear it clips whose diagonal does not have
// v strictly on its left ends the constant-time tests for this star.
template <typename Poly>
__device__ int clip_star(const KParams& P, int v, float2 pv, LocalCounters& lc, unsigned mk, int k, const int* sp,
                         const int* lk, const int* w, Poly& poly, int* bnd) {
  if (k < 3) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
  const int mbase = reserve_marks(P, mk, 2 * k - 3);  // its latency overlaps the clipping
  for (int j = 0; j < k; ++j) {
    poly.set_nx(j, j + 1 == k ? 0 : j + 1);
    poly.set_pv(j, j == 0 ? k - 1 : j - 1);
    bnd[j] = lk[j];
  }
  int remaining = k, j = 0, used = 3;
  // v strictly inside the kernel of the remaining polygon (checked: every
  // side w_i -> w_i+1 has v strictly on its left)
  bool kernel = true;
  for (int i = 0; i < k && kernel; ++i) kernel = orient_v(P, poly.q(i), poly.q(poly.nx(i)), pv, lc) > 0;
  while (remaining > 3) {
    bool found = false;
    if (kernel) {
      for (int t = 0; t < remaining && !found; ++t) {
        const int a = poly.pv(j), b = j, c = poly.nx(j);
        const float2 qa = poly.q(a), qb = poly.q(b), qc = poly.q(c);
        found = orient_v(P, qa, qc, pv, lc) > 0 && orient_v(P, qa, qb, qc, lc) > 0;
        if (!found) j = poly.nx(j);
      }
    }
    for (int t = 0; t < remaining && !found; ++t) {
      const int a = poly.pv(j), b = j, c = poly.nx(j);
      const float2 qa = poly.q(a), qb = poly.q(b), qc = poly.q(c);
      if (orient_v(P, qa, qb, qc, lc) > 0) {
        bool empty = true;
        for (int m = poly.nx(c); m != a && empty; m = poly.nx(m)) {
          const float2 qm = poly.q(m);
          if (orient_v(P, qa, qb, qm, lc) >= 0 && orient_v(P, qb, qc, qm, lc) >= 0 &&
              orient_v(P, qc, qa, qm, lc) >= 0)
            empty = false;
        }
        found = empty;
        if (found && kernel && orient_v(P, qa, qc, pv, lc) <= 0) kernel = false;
      }
      if (!found) j = poly.nx(j);
    }
    if (!found) return MCL_ERR_NO_CONVERGENCE | (__LINE__ << 8);
    const int a = poly.pv(j), b = j, c = poly.nx(j);
    const int g = sp[used++] >> 1;
    const int d0 = 2 * g, d1 = 2 * g + 1;  // d0: w_c -> w_a inside the ear, d1: w_a -> w_c outside
    __stcg(P.ev + g, make_int4(w[c], w[a], w[b], -1));
    __stcg(P.en + g, make_int4(bnd[a], bnd[b], -1, -1));
    he_set_face(P, bnd[a], w[c], bnd[b], d0);
    he_set_face(P, bnd[b], w[a], d0, bnd[a]);
    mark_edge(P, g, mk);
    bnd[a] = d1;
    poly.set_nx(a, c);
    poly.set_pv(c, a);
    --remaining;
    j = c;
  }
  {
    const int a = j, b = poly.nx(a), c = poly.nx(b);
    he_set_face(P, bnd[a], w[c], bnd[b], bnd[c]);
    he_set_face(P, bnd[b], w[a], bnd[c], bnd[a]);
    he_set_face(P, bnd[c], w[b], bnd[a], bnd[b]);
    __stcg(P.vhint + v, bnd[a]);
  }
  for (int i0 = 0; i0 < k; i0 += kGather) {
    // the corners' anchors kGather at a time, loaded before any is rewritten
    // (the corners are distinct, so no store of a group aliases its loads)
    int vh[kGather];
#pragma unroll
    for (int u = 0; u < kGather; ++u) vh[u] = i0 + u < k ? ld_i(P.vhe + w[i0 + u]) : -1;
#pragma unroll
    for (int u = 0; u < kGather; ++u) {
      const int i = i0 + u;
      if (i >= k) continue;
      if (vh[u] == (sp[i] ^ 1)) __stcg(P.vhe + w[i], lk[i]);
      mark_edge(P, lk[i] >> 1, mk);  // the hole's sides face new triangles
    }
  }
  if (mbase >= 0) {
    // the list entries: the sides and the diagonals (the spoke slots sp[3..k)
    // were reused for them); the slots were reserved at the start
    for (int t = 0; t < 2 * k - 3; ++t) append_mark(P, mbase, t, 2 * k - 3, t < k ? lk[t] >> 1 : sp[t - k + 3] >> 1);
  }
  for (int r = 0; r < 3; ++r) {
    const int e = sp[r] >> 1;
    __stcg(P.vfree + 3 * v + r, e);
    __stcg(P.ev + e, make_int4(-1, -1, -1, -1));
    __stcg(P.en + e, make_int4(-1, -1, -1, -1));
  }
  // the neighbour that later point location starts from: the nearest that is
  // not a bounding corner (a corner's half-edges run along the hull, far from
  // v; so do the edges between consecutive hull points)
  int anchor = w[0];
  {
    const float2 p0 = pv;
    float best = INFINITY;
    for (int i0 = 0; i0 < k; i0 += kGather) {
      unsigned char fx[kGather];
#pragma unroll
      for (int u = 0; u < kGather; ++u) fx[u] = i0 + u < k ? P.vfix[w[i0 + u]] : 1;
#pragma unroll
      for (int u = 0; u < kGather; ++u) {
        if (fx[u]) continue;
        const int i = i0 + u;
        const float2 qi = poly.q(i);
        const float dx = __fsub_rn(qi.x, p0.x), dy = __fsub_rn(qi.y, p0.y);
        const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
        if (d2 < best) { best = d2; anchor = w[i]; }
      }
    }
  }
  __stcg(P.vaux + v, anchor);
  __stcg(P.vhe + v, -1);
  return MCL_OK;
}

__device__ int remove_vertex_ears(const KParams& P, int v, LocalCounters& lc, unsigned mk) {
  int sp[kEarMax], lk[kEarMax], w[kEarMax], bnd[kEarMax];
  LocalPoly poly;
  const int s0 = ld_i(P.vhe + v);
  if (bad_h(P, s0)) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
  int k = 0, h = s0;
  do {
    if (k >= kEarMax) return MCL_ERR_CAPACITY | (__LINE__ << 8);
    sp[k] = h;
    lk[k] = he_next(P, h);
    if (bad_h(P, lk[k])) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
    w[k] = he_origin(P, lk[k]);
    if (bad_v(P, w[k])) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
    poly.set_q(k, ldpos(P, w[k]));
    ++k;
    h = he_prev(P, h) ^ 1;
    if (bad_h(P, h)) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
  } while (h != s0);
  return clip_star(P, v, ldpos(P, v), lc, mk, k, sp, lk, w, poly, bnd);
}

// A star walked once per removal round and kept by its thread across the
// round's barriers (claim, verify, remove): the thread handling list entry i
// handles the same entry in all three sub-phases, and a round's winners own
// every face of their stars, so nothing else writes them meanwhile.
constexpr int kStarCache = 32;
struct StarCache {
  int v;                 // cached vertex, -1: none
  int k;                 // its spokes; 0 when more than kStarCache
  int sp[kStarCache];    // spokes, counter-clockwise
  int lk[kStarCache];    // next(sp[i])
  int fm[kStarCache];    // smallest half-edge of face i (its claim slot)
};

// Walk v's star once (one record load per spoke), claiming each face with key.
__device__ bool claim_star(const KParams& P, int v, unsigned long long key, StarCache& sc) {
  sc.v = v;
  sc.k = 0;
  const int s0 = ld_i(P.vhe + v);
  if (bad_h(P, s0)) return false;
  int h = s0, k = 0;
  do {
    const int4 r = ld_en(P, h >> 1);
    const int nxt = (h & 1) ? r.z : r.x, prv = (h & 1) ? r.w : r.y;
    if (bad_h(P, nxt) || bad_h(P, prv)) return false;
    const int f = min(h, min(nxt, prv));
    atomicMax(P.claim + f, key);
    if (k < kStarCache) {
      sc.sp[k] = h;
      sc.lk[k] = nxt;
      sc.fm[k] = f;
    }
    ++k;
    h = prv ^ 1;
  } while (h != s0 && k < 1024);
  if (h != s0) return false;
  sc.k = k <= kStarCache ? k : 0;
  return true;
}

// The positions of corners w[0..k) into poly, kGather loads in flight at a time.
template <typename Poly>
__device__ __forceinline__ void gather_corners(const KParams& P, int k, const int* w, Poly& poly) {
  for (int i0 = 0; i0 < k; i0 += kGather) {
    float2 t[kGather];
#pragma unroll
    for (int u = 0; u < kGather; ++u) t[u] = i0 + u < k ? ldpos(P, w[i0 + u]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kGather; ++u)
      if (i0 + u < k) poly.set_q(i0 + u, t[u]);
  }
}

// Removal of v from its cached star (sc.k spokes): origins and positions of
// the link loaded together, then the ear clipping.
__device__ int remove_cached(const KParams& P, int v, const StarCache& sc, LocalCounters& lc, unsigned mk) {
  const int k = sc.k;
  int w[kStarCache], bnd[kStarCache];
  // link origins, then their positions, kGather loads in flight at a time (a
  // loop that stores each loaded value before the next load waits for every
  // load in turn)
  for (int i0 = 0; i0 < k; i0 += kGather) {
    int t[kGather];
#pragma unroll
    for (int u = 0; u < kGather; ++u) t[u] = i0 + u < k ? he_origin(P, sc.lk[i0 + u]) : 0;
#pragma unroll
    for (int u = 0; u < kGather; ++u)
      if (i0 + u < k) w[i0 + u] = t[u];
  }
  for (int i = 0; i < k; ++i)
    if (bad_v(P, w[i])) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
  const float2 pv = ldpos(P, v);
  if (k <= kSmallStar) {
    SmallPoly poly;
    gather_corners(P, k, w, poly);
    return clip_star(P, v, pv, lc, mk, k, sc.sp, sc.lk, w, poly, bnd);
  }
  LocalPoly poly;
  gather_corners(P, k, w, poly);
  return clip_star(P, v, pv, lc, mk, k, sc.sp, sc.lk, w, poly, bnd);
}

// ---------------------------------------------------------------------------
// Repair (2): removal of a vertex from a valid triangulation: ear clipping of
// its star polygon, or, for stars above kEarMax spokes, flipping its spokes
// until it has degree 3, then merging its three faces.  Runs in one thread;
// the caller owns every face of the vertex's star.
__device__ int remove_vertex(const KParams& P, int v, LocalCounters& lc, int& flips, unsigned mk) {
  {
    // Ear clipping first: one walk around the star, then local work on the
    // loaded polygon (the spoke flips below walk the star again after every
    // flip, a chain of dependent loads per flip).  Stars of more than
    // kEarMax spokes take the flips.
    const int rc = remove_vertex_ears(P, v, lc, mk);
    if ((rc & 0xff) != MCL_ERR_CAPACITY) {
      ++flips;  // counted as one repair operation
      return rc;
    }
  }
  const float2 pv = ldpos(P, v);
  int nearest = -1;  // the nearest neighbour that is not a bounding corner
  float nearest_d2 = INFINITY;
  for (int guard = 0; guard < 4096; ++guard) {
    const int s0 = ld_i(P.vhe + v);
    if (s0 < 0 || s0 >= 2 * P.E) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
    int deg = 0;
    int h = s0;
    int flipped = -1;
    do {
      ++deg;
      if (guard == 0) {
        const int w = he_origin(P, h ^ 1);
        if (!bad_v(P, w) && !P.vfix[w]) {
          const float2 q = ldpos(P, w);
          const float dx = __fsub_rn(q.x, pv.x), dy = __fsub_rn(q.y, pv.y);
          const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
          if (d2 < nearest_d2) { nearest_d2 = d2; nearest = w; }
        }
      }
      if (flipped < 0) {
        // flipping spoke h = v->w replaces faces (v,w,*) and (w,v,*) by (d,c,a), (c,d,b)
        const int e = h >> 1;
        const int4 q = ld_ev(P, e);
        if (bad_v(P, q.x) || bad_v(P, q.y) || q.z >= P.V || q.w >= P.V) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
        if (q.z >= 0 && q.w >= 0) {
          const float2 a = ldpos(P, q.x), b = ldpos(P, q.y), c = ldpos(P, q.z), d = ldpos(P, q.w);
          if (orient_v(P, d, c, a, lc) > 0 && orient_v(P, c, d, b, lc) > 0) flipped = e;
        }
      }
      h = he_prev(P, h) ^ 1;
      if (h < 0 || h >= 2 * P.E) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
    } while (h != s0 && deg < 1024);
    if (deg >= 1024) return MCL_ERR_CAPACITY | (__LINE__ << 8);
    if (deg == 3) break;
    if (deg < 3) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
    if (flipped < 0) {
      // no spoke flip is valid (exactly collinear neighbours): clip ears
      const int rc = remove_vertex_ears(P, v, lc, mk);
      if (rc != MCL_OK && atomicCAS(&P.st->dbg[0], 0, v + 1) == 0) {
        P.st->dbg[1] = deg;
        int hh = s0;
        for (int k = 0; k < deg && k < 64; ++k) {
          P.st->dbg[2 + k] = he_origin(P, hh ^ 1);
          hh = he_prev(P, hh) ^ 1;
        }
      }
      ++flips;  // counted as one repair operation
      return rc;
    }
    if (!flip_edge(P, flipped)) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
    if (mk) {
      P.st->mark_ovf = 1;  // spoke flips are marked, not appended: rebuild the list from the marks
      const int4 wg = ld_en(P, flipped);  // the flipped edge's four wings
      mark_edge(P, flipped, mk);
      mark_edge(P, wg.x >> 1, mk);
      mark_edge(P, wg.y >> 1, mk);
      mark_edge(P, wg.z >> 1, mk);
      mark_edge(P, wg.w >> 1, mk);
    }
    ++flips;
  }
  // merge the three faces (v,x,y), (v,y,z), (v,z,x) into (x,y,z)
  const int s0 = ld_i(P.vhe + v);
  const int s1 = he_prev(P, s0) ^ 1;
  const int s2 = he_prev(P, s1) ^ 1;
  if ((he_prev(P, s2) ^ 1) != s0) return MCL_ERR_NO_CONVERGENCE | (__LINE__ << 8);
  const int lxy = he_next(P, s0), lyz = he_next(P, s1), lzx = he_next(P, s2);
  if (bad_h(P, s1) || bad_h(P, s2) || bad_h(P, lxy) || bad_h(P, lyz) || bad_h(P, lzx)) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
  const int x = he_origin(P, lxy), y = he_origin(P, lyz), z = he_origin(P, lzx);
  if (bad_v(P, x) || bad_v(P, y) || bad_v(P, z)) return MCL_ERR_DEGENERATE_INPUT | (__LINE__ << 8);
  he_set_face(P, lxy, z, lyz, lzx);
  he_set_face(P, lyz, x, lzx, lxy);
  he_set_face(P, lzx, y, lxy, lyz);
  mark_edge(P, lxy >> 1, mk);
  mark_edge(P, lyz >> 1, mk);
  mark_edge(P, lzx >> 1, mk);
  if (mk) P.st->mark_ovf = 1;
  if (ld_i(P.vhe + x) == (s0 ^ 1)) __stcg(P.vhe + x, lxy);
  if (ld_i(P.vhe + y) == (s1 ^ 1)) __stcg(P.vhe + y, lyz);
  if (ld_i(P.vhe + z) == (s2 ^ 1)) __stcg(P.vhe + z, lzx);
  const int es[3] = {s0 >> 1, s1 >> 1, s2 >> 1};
  for (int k = 0; k < 3; ++k) {
    P.vfree[3 * v + k] = es[k];
    __stcg(P.ev + es[k], make_int4(-1, -1, -1, -1));
    __stcg(P.en + es[k], make_int4(-1, -1, -1, -1));
  }
  P.vhint[v] = lxy;
  // the neighbour that later point location starts from: the nearest of the
  // star it had when its removal began that is not a bounding corner (the
  // last three can be far: consecutive points on the hull)
  P.vaux[v] = nearest >= 0 ? nearest : (!P.vfix[x] ? x : (!P.vfix[y] ? y : z));
  __stcg(P.vhe + v, -1);
  return MCL_OK;
}

__device__ bool phase_remove(cg::grid_group& g, const KParams& P, unsigned& stamp, LocalCounters& lc, unsigned mk) {
  const int stride = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, nwarps = stride >> 5, wid = spread_tid() >> 5;
  int src = 0;
  StarCache sc;
  for (int round = 0;; ++round) {
    const int n = ld_i(&P.st->vl_count[src]);
    if (n == 0) return true;
    if (round >= P.max_rounds) {
      if (gtid == 0) set_error(P, MCL_ERR_NO_CONVERGENCE);
      return false;
    }
    const int dst = src ^ 1;
    const int* in = src ? P.vl1 : P.vl0;
    int* out = dst ? P.vl1 : P.vl0;
    const unsigned sk = stamp++;
    if (gtid == 0) {
      P.st->vl_count[dst] = 0;
      P.st->c[C_REMOVE_ROUNDS] += 1;
    }
    // A removal is a long divergent chain (star loads, ear search, writes), so
    // a warp runs its lanes' removals largely one after another: entries are
    // dealt in tiles of T lanes per warp (entry i: warp (i / T) mod warps,
    // lane i mod T), by default as few lanes as let one pass take the list.
    const int T = P.rm_tile > 0 ? min(P.rm_tile, 32) : max(1, min(32, (n + nwarps - 1) / nwarps));
    const int i0 = lane < T ? wid * T + lane : n, di = nwarps * T;
    // claim every face of the star (the thread keeps the last star it walked)
    sc.v = -1;
    for (int i = i0; i < n; i += di) {
      const int v = ld_i(in + i);
      const unsigned long long key = ((unsigned long long)sk << 32) | (unsigned)(~mix32((unsigned)v ^ sk));
      if (!claim_star(P, v, key, sc)) {
        sc.v = -1;
        set_error(P, MCL_ERR_DEGENERATE_INPUT);
      }
    }
    g.sync();
    if (round < 16) timeline_remove(P, 4 * round);
    for (int i = i0; i < n; i += di) {
      const int v = ld_i(in + i);
      const unsigned long long key = ((unsigned long long)sk << 32) | (unsigned)(~mix32((unsigned)v ^ sk));
      bool win = true, ok = true;
      if (sc.v == v && sc.k > 0) {
        // the claims kGather at a time, all loads of a group in flight together
        for (int j0 = 0; j0 < sc.k; j0 += kGather) {
          unsigned long long c[kGather];
#pragma unroll
          for (int u = 0; u < kGather; ++u) c[u] = j0 + u < sc.k ? __ldcg(P.claim + sc.fm[j0 + u]) : key;
#pragma unroll
          for (int u = 0; u < kGather; ++u) win &= c[u] == key;
        }
      } else {
        ok = for_spokes(P, v, [&](int h) {
          if (__ldcg(P.claim + face_min(P, h)) != key) win = false;
        });
      }
      P.vlocf[v] = (ok && win) ? 1 : 0;
      if (!ok) set_error(P, MCL_ERR_DEGENERATE_INPUT);
    }
    g.sync();
    if (round < 16) timeline_remove(P, 4 * round + 1);
    int removed = 0, flips = 0;
    unsigned long long slow = 0;  // the slowest removal of this thread: cycles << 16 | spokes
    WarpBuf wb{s_wbuf[0][threadIdx.x >> 5], 0};
    for (int base = wid * T; base < n; base += di) {
      const int i = lane < T ? base + lane : n;
      int mine[1];
      int k = 0;
      if (i < n) {
        const int v = ld_i(in + i);
        if (__ldcg(P.vlocf + v) == 1) {
          int rc;
          const long long t0 = clock64();
          int deg = sc.k;
          if (sc.v == v && sc.k > 0) {
            rc = remove_cached(P, v, sc, lc, mk);
            ++flips;  // counted as one repair operation
          } else {
            rc = remove_vertex(P, v, lc, flips, mk);
            deg = 0;
            if (round < 16) atomicAdd(&P.st->rm_uncached[round], 1ull);
          }
          const unsigned long long dt = (unsigned long long)(clock64() - t0);
          slow = max(slow, (dt << 16) | (unsigned long long)(deg & 0xffff));
          if (rc != MCL_OK) flag_error_at(P, rc & 0xff, 100000 + (rc >> 8));
          else ++removed;
        } else if (ld_i(&P.st->status) == MCL_OK) {
          mine[k++] = v;
        }
      }
      wb_push(wb, mine, k, out, &P.st->vl_count[dst], P.V, P.st);
    }
    wb_flush(wb, out, &P.st->vl_count[dst], P.V, P.st);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) slow = max(slow, __shfl_down_sync(kFull, slow, o));
    if (round < 16 && lane == 0 && slow) atomicMax(&P.st->rm_slow[round], slow);
    warp_add(&P.st->c[C_REMOVED], removed);
    warp_add(&P.st->c[C_REMOVAL_FLIPS], flips);
    g.sync();
    if (round < 16) timeline_remove(P, 4 * round + 2);
    src = dst;
  }
}

// ---------------------------------------------------------------------------
// Point location: visibility walk with exact orientation tests from half-edge h.
// Returns a half-edge of the face containing p; *on is the half-edge p lies on
// (or -1).  Errors are returned as negative MCL codes.  With max_steps > 0 the
// walk stops after that many steps, returns -1 and leaves the face it reached
// in *resume (a parallel round then waits for the longest walk only that long).
// salt != 0: the edge tested first in each face is drawn from a hash of
// (salt, step) (a stochastic walk, which terminates on any triangulation);
// salt == 0: it rotates with the step (enough on a Delaunay triangulation).
__device__ int locate(const KParams& P, float2 p, int h, int* on, LocalCounters& lc, int max_steps = 0,
                      int* resume = nullptr, unsigned salt = 0) {
  *on = -1;
  for (int it = 0; it < P.walk_cap; ++it) {
    if (max_steps > 0 && it == max_steps) {
      *resume = h;
      return -1;
    }
    if (h < 0 || h >= 2 * P.E) return -MCL_ERR_DEGENERATE_INPUT;
    // the face's three corners and its other two half-edges from h's two
    // records (loaded together): origin(next(h)) = origin(twin(h)) and
    // origin(prev(h)) = apex(h)
    const int4 r = ld_ev(P, h >> 1), nn = ld_en(P, h >> 1);
    const bool odd = h & 1;
    const int hs[3] = {h, odd ? nn.z : nn.x, odd ? nn.w : nn.y};
    const int o[3] = {odd ? r.y : r.x, odd ? r.x : r.y, odd ? r.w : r.z};
    for (int k = 0; k < 3; ++k) {
      if (hs[k] < 0 || hs[k] >= 2 * P.E) return -MCL_ERR_DEGENERATE_INPUT;
      if (o[k] < 0 || o[k] >= P.V) return -MCL_ERR_DEGENERATE_INPUT;
    }
    const float2 q[3] = {ldpos(P, o[0]), ldpos(P, o[1]), ldpos(P, o[2])};
    int s[3] = {1, 1, 1};
    int cross = -1;
    const int start = salt ? (int)(mix32(salt + (unsigned)it * 0x9e3779b9u) % 3u) : it % 3;
    // Every edge with p on its far side is a valid step; an edge with a
    // bounding corner is taken only when no other is (stepping through a
    // corner's fan of long hull triangles can take hundreds of steps).
    bool corner_cross = false;
    for (int k = 0; k < 3; ++k) {
      const int i = (start + k) % 3;
      s[i] = orient_v(P, q[i], q[(i + 1) % 3], p, lc);
      if (s[i] < 0) {
        const bool corner = P.vfix[o[i]] || P.vfix[o[(i + 1) % 3]];
        if (cross < 0 || (corner_cross && !corner)) {
          cross = i;
          corner_cross = corner;
        }
        if (!corner) break;
      }
    }
    if (cross >= 0) {
      const int t = hs[cross] ^ 1;
      if (he_apex(P, t) < 0) return -MCL_ERR_DEGENERATE_INPUT;  // outside the bounding square
      h = t;
      continue;
    }
    int zeros = 0, zi = -1;
    for (int i = 0; i < 3; ++i)
      if (s[i] == 0) { ++zeros; zi = i; }
    if (zeros >= 2) return -MCL_ERR_DEGENERATE_INPUT;  // coincides with a vertex
    if (zeros == 1) {
      if (he_apex(P, hs[zi] ^ 1) < 0) return -MCL_ERR_DEGENERATE_INPUT;  // on the bounding square
      *on = hs[zi];
    }
    return h;
  }
  return -(MCL_ERR_NO_CONVERGENCE | (__LINE__ << 8));
}

// 1-to-3 split of the face of half-edge h0 by v with free edges f0, f1, f2.
__device__ void split13(const KParams& P, int v, int h0, const int* f) {
  const int h1 = he_next(P, h0), h2 = he_prev(P, h0);
  const int x0 = he_origin(P, h0), x1 = he_origin(P, h1), x2 = he_origin(P, h2);
  const int f0 = f[0], f1 = f[1], f2 = f[2];
  __stcg(P.ev + f0, make_int4(v, x0, x1, x2));
  __stcg(P.ev + f1, make_int4(v, x1, x2, x0));
  __stcg(P.ev + f2, make_int4(v, x2, x0, x1));
  __stcg(P.en + f0, make_int4(h0, 2 * f1 + 1, 2 * f2, h2));
  __stcg(P.en + f1, make_int4(h1, 2 * f2 + 1, 2 * f0, h0));
  __stcg(P.en + f2, make_int4(h2, 2 * f0 + 1, 2 * f1, h1));
  he_set_face(P, h0, v, 2 * f1 + 1, 2 * f0);
  he_set_face(P, h1, v, 2 * f2 + 1, 2 * f1);
  he_set_face(P, h2, v, 2 * f0 + 1, 2 * f2);
  __stcg(P.vhe + v, 2 * f0);
}

// 2-to-4 split of the edge of half-edge g (v lies on it) with free edges f0..f2.
__device__ void split24(const KParams& P, int v, int g, const int* f) {
  const int h0 = g, h1 = g ^ 1;
  const int n0 = he_next(P, h0), p0 = he_prev(P, h0);
  const int n1 = he_next(P, h1), p1 = he_prev(P, h1);
  const int a = he_origin(P, h0), b = he_origin(P, h1);
  const int c = he_apex(P, h0), d = he_apex(P, h1);
  const int f0 = f[0], f1 = f[1], f2 = f[2];
  // faces: (a,v,c) (v,b,c) (b,v,d) (v,a,d)
  he_set_origin(P, h1, v);
  he_set_face(P, h0, c, 2 * f1, p0);
  he_set_face(P, h1, d, n1, 2 * f2 + 1);
  he_set_face(P, p0, v, h0, 2 * f1);
  he_set_face(P, n0, v, 2 * f1 + 1, 2 * f0);
  he_set_face(P, p1, v, 2 * f0 + 1, 2 * f2);
  he_set_face(P, n1, v, 2 * f2 + 1, h1);
  __stcg(P.ev + f0, make_int4(v, b, c, d));
  __stcg(P.en + f0, make_int4(n0, 2 * f1 + 1, 2 * f2, p1));
  __stcg(P.ev + f1, make_int4(v, c, a, b));
  __stcg(P.en + f1, make_int4(p0, h0, 2 * f0, n0));
  __stcg(P.ev + f2, make_int4(v, d, b, a));
  __stcg(P.en + f2, make_int4(p1, 2 * f0 + 1, h1, n1));
  __stcg(P.vhe + v, 2 * f0);
  if (ld_i(P.vhe + b) == h1) __stcg(P.vhe + b, n0);
}

// Start of the point location of a pending vertex: the hole half-edge recorded
// at its removal when that edge is still live, else the neighbour recorded at
// removal (vaux) and, when that one was removed too, its own recorded
// neighbour, and so on: each hop stays about one spacing from the old
// position, so the walk stays short instead of starting at the bounding square.
__device__ __forceinline__ bool face_has_corner(const KParams& P, int h) {
  const int a = he_origin(P, h), b = he_origin(P, h ^ 1), c = he_apex(P, h);
  return (a >= 0 && P.vfix[a]) || (b >= 0 && P.vfix[b]) || (c >= 0 && P.vfix[c]);
}

// In later rounds of an insertion phase the hint is where the vertex's last
// walk ended (located, or paused): it is taken as it is, or a walk paused in a
// corner's fan would be sent back to its anchor every round and never arrive.
__device__ int insert_start(const KParams& P, int v, bool resume) {
  int h = __ldcg(P.vhint + v);
  const bool hint_ok = h >= 0 && h < 2 * P.E && he_origin(P, h) >= 0 && he_apex(P, h) >= 0;
  if (resume && hint_ok) return h;
  // the live anchor: the neighbour recorded at removal, or its own anchor if
  // that one was removed too
  int x = __ldcg(P.vaux + v), h0 = -1;
  for (int hop = 0; hop < 64 && x >= 0 && x < P.V; ++hop) {
    h0 = ld_i(P.vhe + x);
    if (h0 >= 0 && h0 < 2 * P.E) break;
    h0 = -1;
    x = __ldcg(P.vaux + x);
  }
  // a first start on a bounding corner's fan of long hull triangles makes the
  // walk step along the hull one triangle at a time: prefer a face with no
  // corner.  The hint's edge slot may have been freed by a later removal and
  // reused far away, so it is taken only when it is not farther from the
  // target than the anchor.
  if (hint_ok && !face_has_corner(P, h)) {
    if (h0 < 0) return h;
    const float2 t = ldpos(P, v), ph = ldpos(P, he_origin(P, h)), px = ldpos(P, x);
    const float dh = __fadd_rn(__fmul_rn(ph.x - t.x, ph.x - t.x), __fmul_rn(ph.y - t.y, ph.y - t.y));
    const float dx = __fadd_rn(__fmul_rn(px.x - t.x, px.x - t.x), __fmul_rn(px.y - t.y, px.y - t.y));
    if (dh <= dx) return h;
  }
  if (h0 >= 0) {
    int g = h0;
    for (int k = 0; k < 64; ++k) {
      if (he_apex(P, g) >= 0 && !face_has_corner(P, g)) return g;
      g = he_next(P, g ^ 1);  // next outgoing half-edge of x
      if (g < 0 || g >= 2 * P.E || g == h0) break;
    }
    return hint_ok ? h : h0;
  }
  if (hint_ok) return h;
  // half-edge 0 of the vertex's mesh is never freed: a side of its bounding square
  return P.vroot ? __ldg(P.vroot + v) : 0;
}

// Steps a point location may take in one insertion round before it waits for
// the next round (which starts where it stopped).
constexpr int kWalkSlice = 48;

// With mk != 0 (repair) the rounds only split: the edges each split touches
// are marked with mk for one Lawson pass after the last round (the walks of
// later rounds run on a valid, not yet Delaunay, triangulation; their edge
// order is randomised, so they cannot cycle).  With mk == 0 (the initial
// build) every round ends with Lawson over the edges it touched.
__device__ bool phase_insert(cg::grid_group& g, const KParams& P, unsigned& stamp,
                             LocalCounters& lc, unsigned mk = 0) {
  const int stride = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  int src = 0;
  for (int round = 0;; ++round) {
    const int n = ld_i(&P.st->vl_count[src]);
    if (n == 0) return true;
    if (round >= P.max_rounds) {
      if (gtid == 0) set_error(P, MCL_ERR_NO_CONVERGENCE);
      return false;
    }
    const int dst = src ^ 1;
    const int* in = src ? P.vl1 : P.vl0;
    int* out = dst ? P.vl1 : P.vl0;
    const unsigned sk = stamp++;
    const unsigned sq = stamp++;
    if (gtid == 0) {
      P.st->vl_count[dst] = 0;
      if (!mk) P.st->wl_count[0] = 0;  // with mk the list gathers the marks of every round
      P.st->c[C_INSERT_ROUNDS] += 1;
    }
    // locate and claim
    for (int i = spread_tid(); i < n; i += stride) {
      const int v = ld_i(in + i);
      int on = -1;
      int resume = -1;
      // a walk paused in the last round goes on from where it stopped; any
      // other start is the closer of the hint (the face located last round,
      // which can reach far along the hull) and the anchor
      const bool paused = round > 0 && __ldcg(P.vlocf + v) == 4;
      const int h = locate(P, ldpos(P, v), insert_start(P, v, paused), &on, lc, kWalkSlice, &resume,
                           mk ? mix32((unsigned)v ^ sk) | 1u : 0u);
      if (h == -1) {
        // not there yet: go on from here in the next round
        P.vloc[v] = resume;
        P.vlocf[v] = 4;
        continue;
      }
      if (h < 0) {
        flag_error_at(P, (-h) & 0xff, 200000 + ((-h) >> 8));
        P.vlocf[v] = -1;
        continue;
      }
      P.vloc[v] = on >= 0 ? on : h;
      P.vlocf[v] = on >= 0 ? 2 : 0;  // bit 1: on the edge of vloc, bit 0: winner
      const unsigned long long key = ((unsigned long long)sk << 32) | (unsigned)(~mix32((unsigned)v ^ sk));
      if (on >= 0) {
        atomicMax(P.claim + face_min(P, on), key);
        atomicMax(P.claim + face_min(P, on ^ 1), key);
      } else {
        atomicMax(P.claim + face_min(P, h), key);
      }
    }
    g.sync();
    timeline_insert(P, round, 0);
    for (int i = spread_tid(); i < n; i += stride) {
      const int v = ld_i(in + i);
      const int fl = __ldcg(P.vlocf + v);
      if (fl < 0) continue;
      const unsigned long long key = ((unsigned long long)sk << 32) | (unsigned)(~mix32((unsigned)v ^ sk));
      const int h = __ldcg(P.vloc + v);
      bool win = __ldcg(P.claim + face_min(P, h)) == key;
      if (fl & 2) win = win && __ldcg(P.claim + face_min(P, h ^ 1)) == key;
      if (win) P.vlocf[v] = fl | 1;
    }
    g.sync();
    timeline_insert(P, round, 1);
    int inserted = 0;
    WarpBuf wagain{s_wbuf[1][threadIdx.x >> 5], 0};
    for (int base = spread_tid() - (int)(threadIdx.x & 31); base < n; base += stride) {
      const int i = base + (int)(threadIdx.x & 31);
      int mine[8];
      int k = 0;
      int again[1];
      int ka = 0;
      if (i < n) {
        const int v = ld_i(in + i);
        const int fl = __ldcg(P.vlocf + v);
        if (fl >= 0 && (fl & 1)) {
          const int f[3] = {__ldcg(P.vfree + 3 * v), __ldcg(P.vfree + 3 * v + 1), __ldcg(P.vfree + 3 * v + 2)};
          int link[4];
          int nl = 0;
          if ((unsigned)f[0] >= (unsigned)P.E || (unsigned)f[1] >= (unsigned)P.E || (unsigned)f[2] >= (unsigned)P.E ||
              bad_h(P, __ldcg(P.vloc + v))) {
            flag_error(P, MCL_ERR_DEGENERATE_INPUT);
          } else if (fl & 2) {
            const int gg = __ldcg(P.vloc + v);
            link[nl++] = he_prev(P, gg);
            link[nl++] = he_next(P, gg);
            link[nl++] = he_prev(P, gg ^ 1);
            link[nl++] = he_next(P, gg ^ 1);
            split24(P, v, gg, f);
          } else {
            const int h = __ldcg(P.vloc + v);
            link[nl++] = h;
            link[nl++] = he_next(P, h);
            link[nl++] = he_prev(P, h);
            split13(P, v, h, f);
          }
          ++inserted;
          for (int j = 0; j < nl; ++j)
            if (bad_h(P, link[j])) { link[j] = 0; flag_error(P, MCL_ERR_DEGENERATE_INPUT); }
          if (mk) {
            // on a triangulation that is not Delaunay the new spokes need not
            // be legal either: the split edge (now v's spoke to a) and f0..f2
            int edges[8];
            int cnt = 0;
            for (int j = 0; j < nl; ++j) edges[cnt++] = link[j] >> 1;
            for (int j = 0; j < 3; ++j) edges[cnt++] = f[j];
            if (fl & 2) edges[cnt++] = __ldcg(P.vloc + v) >> 1;
            const int mbase = reserve_marks(P, mk, cnt);
            for (int j = 0; j < cnt; ++j) {
              mark_edge(P, edges[j], mk);
              append_mark(P, mbase, j, cnt, edges[j]);
            }
          } else {
            for (int j = 0; j < nl; ++j)
              if (enqueue_once(P, link[j] >> 1, sq)) mine[k++] = link[j] >> 1;
            for (int j = 0; j < 3; ++j)
              if (enqueue_once(P, f[j], sq)) mine[k++] = f[j];
          }
        } else if (fl >= 0) {
          __stcg(P.vhint + v, __ldcg(P.vloc + v));
          again[ka++] = v;
        }
      }
      warp_push(mine, k, P.wl0, &P.st->wl_count[0], P.E, P.st);
      wb_push(wagain, again, ka, out, &P.st->vl_count[dst], P.V, P.st);
    }
    wb_flush(wagain, out, &P.st->vl_count[dst], P.V, P.st);
    (void)inserted;
    g.sync();
    timeline_insert(P, round, 2);
    if (!mk) {
      phase_lawson<false>(g, P, 0, stamp, lc, 0);
      g.sync();
    }
    timeline_insert(P, round, 3);
    src = dst;
  }
}

// ---------------------------------------------------------------------------
// End of a launch: publish this launch's counters and status for the host,
// add them to the running totals, and leave the working state clean for the
// next launch (so no reset launch or memset precedes the next step).
// The step counters of the last launch in the public record layout.
__device__ void publish_stats(const DevState* st, mcl_step_stats* out) {
  const unsigned long long* c = st->last;
  out->inverted_faces = (int64_t)c[C_INVERTED];
  out->reverted_vertices = (int64_t)c[C_REVERTED];
  out->removed_vertices = (int64_t)c[C_REMOVED];
  out->lawson_flips = (int64_t)c[C_LAWSON_FLIPS];
  out->lawson_rounds = (int64_t)c[C_LAWSON_ROUNDS];
  out->removal_flips = (int64_t)c[C_REMOVAL_FLIPS];
  out->insert_rounds = (int64_t)c[C_INSERT_ROUNDS];
  out->incircle_tests = (int64_t)c[C_INCIRCLE];
  out->incircle_fp64 = (int64_t)c[C_INCIRCLE_FP64];
  out->incircle_exact = (int64_t)c[C_INCIRCLE_EXACT];
  out->orient_fp64 = (int64_t)c[C_ORIENT_FP64];
  out->orient_exact = (int64_t)c[C_ORIENT_EXACT];
  out->sos_decisions = (int64_t)c[C_SOS];
  out->status = st->last_status;
  out->error_site = st->last_site;
  out->failed_launches = st->last_status != MCL_OK ? 1 : 0;
  out->substep_vertices = (int64_t)c[C_SUBSTEP_DONE];
}

__device__ void finish_launch(const KParams& P, unsigned stamp) {
  DevState* st = P.st;
  // L2-coherent reads: other blocks' atomics and stores are not in this SM's L1
  for (int i = 0; i < C_COUNT; ++i) {
    const unsigned long long c = __ldcg(&st->c[i]);
    st->last[i] = c;
    st->tot[i] += c;
    st->c[i] = 0;
  }
  const int status = __ldcg(&st->status);
  st->calls += 1;
  if (status != MCL_OK) st->failed += 1;
  const bool repaired = st->last[C_INVERTED] != 0;
  for (int i = 0; i < 4; ++i) {
    if (!repaired) st->ts[43 + i] = __ldcg(&st->tsmax[i]);
    st->tsmax[i] = 0;
  }
  st->last_status = status;
  st->last_site = __ldcg(&st->site);
  if (P.stats_out) publish_stats(st, P.stats_out);  // host-mapped: no copy launch
  st->status = 0;
  st->site = 0;
  st->wl_count[0] = st->wl_count[1] = 0;
  st->vl_count[0] = st->vl_count[1] = 0;
  st->inverted = 0;
  st->hard_count = 0;
  for (int i = 0; i < 3; ++i) st->fix_new[i] = st->fix_bad[i] = st->fix_list[i] = 0;
  st->fix_all = 0;
  st->mark_ovf = 0;
  st->movers_last = __ldcg(&st->movers_now);
  st->movers_now = 0;
  st->epoch = stamp;
}

// ---------------------------------------------------------------------------
// Repair (1b): bring sent-back vertices to their targets in sub-steps, so that
// most of them need no removal.  A Delaunay mesh whose vertex moves on a line
// meets a flip (an incircle event) before any face around the vertex
// degenerates, so moving part of the way, restoring the Delaunay property
// around the vertex and moving on passes the obstruction that sent it back.
// A sub-step moves every pending vertex toward its target (all the way, or
// 9/10 of the way to the first face of its star that would degenerate, times
// 2^-lvl after lvl send-backs in a row); sends back, pass by pass until every
// face is positive, each mover with a non-positive face in its star (lvl + 1);
// runs Lawson rounds over the stars of the movers that stayed; and keeps those
// not yet at their targets pending (lvl 0).  Vertices sent back more than
// kSubstepLevels times in a row, or still pending after P.substeps sub-steps,
// are left on vl0 for removal and reinsertion.  The mesh ends as the Delaunay triangulation of
// the targets either way; this path only saves removals.
//
// In: vl0 = pending vertices at valid positions (pos), targets in `target`,
// vlocf = 0 for each, the mesh Delaunay.  Out: vl0 = vertices left for
// removal (at their last valid positions), the mesh valid and Delaunay.
constexpr int kSubstepLevels = 5;

__device__ void phase_substeps(cg::grid_group& g, const KParams& P, unsigned& stamp, LocalCounters& lc) {
  const int stride = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int* const mv[2] = {P.vl2, P.vl2 + P.V};  // movers of a sub-step pass
  int* const rv = P.vl2 + 2 * P.V;          // movers sent back in the current pass
  int* const left = P.vl2 + 3 * P.V;        // past kSubstepLevels halvings
  int src = 0;
  int done = 0;
  for (int s = 0; s < P.substeps; ++s) {
    const int n = ld_i(&P.st->vl_count[src]);
    if (n == 0) break;
    const int dst = src ^ 1;
    const int* in = src ? P.vl1 : P.vl0;
    int* out = dst ? P.vl1 : P.vl0;
    const unsigned qs = stamp++;
    if (gtid == 0) {
      P.st->vl_count[dst] = 0;
      P.st->sub_count[0] = 0;
      P.st->sub_count[1] = 0;
      for (int k = 0; k < 3; ++k) P.st->sub_rev[k] = 0;
      if (s == 0) P.st->sub_count[2] = 0;
      P.st->wl_count[0] = 0;
      P.st->wl_count[1] = 0;
      P.st->c[C_SUBSTEPS] += 1;
    }
    g.sync();
    // (a) move each pending vertex toward its target: all the way when no
    // face of its star degenerates on the way, else 9/10 of the way to the
    // first face that would (the flip that clears it comes before); after
    // lvl consecutive send-backs, 2^-lvl of that
    for (int base = spread_tid() - lane; base < n; base += stride) {
      const int i = base + lane;
      int mine[1];
      int k = 0;
      if (i < n) {
        const int v = ld_i(in + i);
        const float2 p = ldpos(P, v), t = __ldcg(P.target + v);
        const int lvl = ld_i(P.vlocf + v);
        double fmax = 1.0;
        bool blocked = false;
        for_spokes(P, v, [&](int h) {
          const int d = he_origin(P, h ^ 1), a = he_apex(P, h);
          if (bad_v(P, d) || a < 0 || bad_v(P, a)) return;
          const float2 q = ldpos(P, d), r = ldpos(P, a);
          // orientation of (x, q, r) is affine in x: its value at p and at t
          const double o0 = ((double)q.x - p.x) * ((double)r.y - p.y) - ((double)q.y - p.y) * ((double)r.x - p.x);
          const double o1 = ((double)q.x - t.x) * ((double)r.y - t.y) - ((double)q.y - t.y) * ((double)r.x - t.x);
          if (o1 <= 0.0) {
            blocked = true;
            const double f = o0 > 0.0 ? o0 / (o0 - o1) : 0.0;
            fmax = f < fmax ? f : fmax;
          }
        });
        float2 c = t;
        if (blocked || lvl > 0) {
          const float f = (float)((blocked ? 0.9 * fmax : 1.0) * ldexp(1.0, -lvl));
          c.x = fadd(p.x, fmul(fsub(t.x, p.x), f));
          c.y = fadd(p.y, fmul(fsub(t.y, p.y), f));
        }
        __stcg(P.vprev + v, p);
        __stcg(P.pos + v, c);
        mine[k++] = v;
      }
      warp_push(mine, k, mv[0], &P.st->sub_count[0], P.V, P.st);
    }
    g.sync();
    // (b) send back, pass by pass, every mover with a non-positive face in its
    // star: every position is read (detect) before any is restored (apply)
    int cur = 0;
    for (int pass = 0;; ++pass) {
      if (pass == 64) {
        if (gtid == 0) set_error(P, MCL_ERR_NO_CONVERGENCE);
        return;
      }
      const int m = ld_i(&P.st->sub_count[cur]);
      const int nxt = cur ^ 1;
      const int slot = pass % 3;
      for (int base = spread_tid() - lane; base < m; base += stride) {
        const int i = base + lane;
        int stay[1], back[1], pend[1], gone[1];
        int ks = 0, kb = 0, kp = 0, kg = 0;
        if (i < m) {
          const int v = ld_i(mv[cur] + i);
          const float2 pv = ldpos(P, v);
          bool good = true;
          const bool ok = for_spokes(P, v, [&](int h) {
            if (!good) return;
            const int d = he_origin(P, h ^ 1), a = he_apex(P, h);
            if (bad_v(P, d) || a < 0 || bad_v(P, a)) {
              good = false;
              return;
            }
            if (orient_v(P, pv, ldpos(P, d), ldpos(P, a), lc) <= 0) good = false;
          });
          if (!ok) flag_error(P, MCL_ERR_DEGENERATE_INPUT);
          if (good) {
            stay[ks++] = v;
          } else {
            const int lvl = ld_i(P.vlocf + v) + 1;
            __stcg(P.vlocf + v, lvl);
            back[kb++] = v;
            if (lvl > kSubstepLevels) gone[kg++] = v;
            else pend[kp++] = v;
          }
        }
        warp_push(stay, ks, mv[nxt], &P.st->sub_count[nxt], P.V, P.st);
        warp_push(back, kb, rv, &P.st->sub_rev[slot], P.V, P.st);
        warp_push(pend, kp, out, &P.st->vl_count[dst], P.V, P.st);
        warp_push(gone, kg, left, &P.st->sub_count[2], P.V, P.st);
      }
      g.sync();
      const int nrev = ld_i(&P.st->sub_rev[slot]);
      cur = nxt;
      if (nrev == 0) break;
      for (int i = spread_tid(); i < nrev; i += stride) {
        const int v = ld_i(rv + i);
        __stcg(P.pos + v, __ldcg(P.vprev + v));
      }
      if (gtid == 0) {
        P.st->sub_count[nxt ^ 1] = 0;  // the list just read becomes the next survivors' list
        P.st->sub_rev[(pass + 1) % 3] = 0;
      }
      g.sync();
    }
    // (c) movers that stayed: at their targets they are done, else they stay
    // pending (lvl 0); (d) their stars are queued for Lawson rounds
    const int m = ld_i(&P.st->sub_count[cur]);
    for (int base = spread_tid() - lane; base < m; base += stride) {
      const int i = base + lane;
      int pend[1];
      int kp = 0;
      int h0 = -1;
      if (i < m) {
        const int v = ld_i(mv[cur] + i);
        const float2 pv = ldpos(P, v), t = __ldcg(P.target + v);
        if (__float_as_uint(pv.x) == __float_as_uint(t.x) && __float_as_uint(pv.y) == __float_as_uint(t.y)) {
          ++done;
        } else {
          __stcg(P.vlocf + v, 0);
          pend[kp++] = v;
        }
        h0 = ld_i(P.vhe + v);
        if (h0 < 0 || h0 >= 2 * P.E) {
          flag_error(P, MCL_ERR_DEGENERATE_INPUT);
          h0 = -1;
        }
      }
      warp_push(pend, kp, out, &P.st->vl_count[dst], P.V, P.st);
      // the stars in lock step across the warp: spokes and link edges
      int h = h0;
      bool active = h0 >= 0;
      for (int it = 0; it < 1024 && __any_sync(kFull, active); ++it) {
        int mine[2];
        int k = 0;
        if (active) {
          const int es = h >> 1, el = he_next(P, h) >> 1;
          if (enqueue_once(P, es, qs)) mine[k++] = es;
          if (el >= 0 && el < P.E && enqueue_once(P, el, qs)) mine[k++] = el;
          h = he_prev(P, h) ^ 1;
          if (h < 0 || h >= 2 * P.E || h == h0) active = false;
        }
        warp_push(mine, k, P.wl0, &P.st->wl_count[0], P.E, P.st);
      }
    }
    g.sync();
    phase_lawson<false>(g, P, 0, stamp, lc, 0);
    src = dst;
  }
  // left for removal: still pending, and past the halving limit
  const int np = ld_i(&P.st->vl_count[src]);
  const int nl = ld_i(&P.st->sub_count[2]);
  for (int i = gtid; i < np + nl; i += stride) {
    const int v = i < np ? ld_i((src ? P.vl1 : P.vl0) + i) : ld_i(left + (i - np));
    if (src || i >= np) __stcg(P.vl2 + i, v);  // staged through the first mover list
  }
  g.sync();
  if (src || nl) {
    for (int i = gtid; i < np + nl; i += stride)
      if (src || i >= np) __stcg(P.vl0 + i, ld_i(P.vl2 + i));
  }
  if (gtid == 0) P.st->vl_count[0] = np + nl;
  warp_add(&P.st->c[C_SUBSTEP_DONE], done);
  g.sync();
}

// Repair of a step whose classification found inverted faces: revert, remove,
// Lawson, reinsert.  Out of line, so k_step's hot loops keep their registers;
// keeps its own counters and returns the next free stamp.
__device__ __noinline__ unsigned repair_step(cg::grid_group g, const KParams P, unsigned stamp, unsigned q0) {
  LocalCounters lc = {0, 0, 0, 0, 0, 0, 0};
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  KParams Q = P;
  Q.move_mode = MOVE_NONE;  // positions were moved by the classification
  const int inverted = ld_i(&P.st->inverted);
  if (gtid == 0) P.st->c[C_INVERTED] += (unsigned long long)inverted;
  const unsigned fs = stamp++;  // revert marks of this launch
  // Edges to pass through Lawson at the end carry the mark mk: the
  // classification's non-Delaunay edges (queued with q0), then every edge a
  // removal or a split touches.  Any other edge is Delaunay: its quad keeps
  // the positions it was classified with (every sent-back vertex is removed,
  // and each edge whose quad held one is a spoke, gone, or a side of its
  // hole, marked).
  unsigned mk = q0;
  // (1) revert until valid
  bool ok = phase_fixpoint(g, Q, lc, fs);
  g.sync();
  timeline(P, 43);
  if (ok) {
    // removal list: reverted vertices that actually moved.  Few: from the
    // list of every vertex sent back (on `hard`); many: by a pass over the
    // vertices, whose id order keeps neighbouring removals in one warp
    // (the mark order scatters them).
    const int stride = gridDim.x * blockDim.x;
    const int nall = ld_i(&P.st->fix_all);
    const bool few = (long long)nall * 64 < (long long)P.V_it;
    if (gtid == 0) { P.st->vl_count[0] = 0; P.st->vl_count[1] = 0; }
    g.sync();
    const int nsb = few ? nall : P.V_it;
    WarpBuf wrev{s_wbuf[0][threadIdx.x >> 5], 0};
    for (int base = (few ? spread_tid() - (int)(threadIdx.x & 31) : blockIdx.x * blockDim.x); base < nsb;
         base += stride) {
      const int vi = base + (few ? (int)(threadIdx.x & 31) : (int)threadIdx.x);
      const int v = vi < nsb ? (few ? ld_i(P.hard + vi) : vert_at(P, vi)) : 0;
      int mine[1];
      int k = 0;
      if (vi < nsb && marked(Q, v, fs) && !P.vfix[v]) {
        const float2 pn = ldpos(Q, v), po = P.pos_old[v];
        if (__float_as_uint(pn.x) != __float_as_uint(po.x) || __float_as_uint(pn.y) != __float_as_uint(po.y)) {
          __stcg(P.target + v, pn);
          __stcg(P.pos + v, po);
          __stcg(P.vlocf + v, 0);  // sub-step level
          mine[k++] = v;
        }
      }
      wb_push(wrev, mine, k, P.vl0, &P.st->vl_count[0], P.V, P.st);
    }
    wb_flush(wrev, P.vl0, &P.st->vl_count[0], P.V, P.st);
    g.sync();
    const int nrev = ld_i(&P.st->vl_count[0]);
    if (gtid == 0) P.st->c[C_REVERTED] += (unsigned long long)nrev;
    if (nrev > 0 && P.substeps > 0) {
      // (1b) Delaunay over every edge with the sent-back vertices at their old
      // positions, then sub-steps toward their targets; the mesh is then
      // Delaunay, so only what removal and reinsertion touch is marked
      if (gtid == 0) { P.st->wl_count[0] = 0; P.st->wl_count[1] = 0; P.st->inverted = 0; P.st->hard_count = 0; }
      g.sync();
      const unsigned qa = stamp++;
      const unsigned sc0 = stamp++;
      phase_classify<false>(g, Q, qa, sc0, lc);
      g.sync();
      phase_classify_hard<false>(g, Q, qa, sc0, lc);
      phase_lawson<false>(g, Q, 0, stamp, lc, sc0);
      g.sync();
      timeline_insert(P, 15, 0);
      phase_substeps(g, Q, stamp, lc);
      timeline_insert(P, 15, 1);
      mk = stamp++;
      // the mesh is Delaunay again: the final Lawson list starts empty
      if (gtid == 0) { P.st->wl_count[0] = 0; P.st->wl_count[1] = 0; }
      g.sync();
    }
    const int nrem = ld_i(&P.st->vl_count[0]);
    // few removals: their marks are appended to a list (no pass over every
    // edge afterwards); many: the list is rebuilt from the marks
    Q.append_marks = (long long)nrem * 64 < (long long)P.E_it ? 1 : 0;
    if (!Q.append_marks && gtid == 0) P.st->mark_ovf = 1;
    if (nrem > 0) {
      // (2) remove what is left, marking each hole's sides and diagonals
      ok = phase_remove(g, Q, stamp, lc, mk);
      g.sync();
      timeline(P, 44);
      // (3) reinsert at the new positions: splits only, their edges marked
      if (gtid == 0) { P.st->vl_count[0] = 0; P.st->vl_count[1] = 0; }
      g.sync();
      // the removed vertices: from the list of every vertex sent back when
      // few (and the sub-steps' classification did not reuse its buffer),
      // else by a pass over the vertices
      const bool from_list = few && !(nrev > 0 && P.substeps > 0);
      const int nscan = from_list ? nall : P.V_it;
      WarpBuf wins{s_wbuf[0][threadIdx.x >> 5], 0};
      for (int base = (from_list ? spread_tid() - (int)(threadIdx.x & 31) : blockIdx.x * blockDim.x); base < nscan;
           base += stride) {
        const int vi = base + (from_list ? (int)(threadIdx.x & 31) : (int)threadIdx.x);
        const int v = vi < nscan ? (from_list ? ld_i(P.hard + vi) : vert_at(P, vi)) : 0;
        int mine[1];
        int k = 0;
        if (vi < nscan && ld_i(P.vhe + v) < 0 && marked(Q, v, fs)) {
          __stcg(P.pos + v, __ldcg(P.target + v));
          mine[k++] = v;
        }
        wb_push(wins, mine, k, P.vl0, &P.st->vl_count[0], P.V, P.st);
      }
      wb_flush(wins, P.vl0, &P.st->vl_count[0], P.V, P.st);
      g.sync();
      if (ok) ok = phase_insert(g, Q, stamp, lc, mk);
      g.sync();
    } else {
      timeline(P, 44);
    }
    timeline(P, 45);
    // (4) one Lawson pass from every marked edge: work-list 0 holds the
    // classification's non-Delaunay edges and the appended marks, repeats
    // included; deduplicated into work-list 1 when short, else rebuilt from
    // the marks over every edge
    if (ok) {
      const int nw = ld_i(&P.st->wl_count[0]);
      const bool rebuild = ld_i(&P.st->mark_ovf) || (long long)nw * 4 >= (long long)P.E_it;
      g.sync();  // every thread has read the count and the flag
      if (rebuild) {
        if (gtid == 0) { P.st->wl_count[0] = 0; P.st->wl_count[1] = 0; }
        g.sync();
        WarpBuf wb{s_wbuf[0][threadIdx.x >> 5], 0};
        for (int base = blockIdx.x * blockDim.x; base < P.E_it; base += stride) {
          const int ei = base + threadIdx.x;
          const int e = ei < P.E_it ? edge_at(P, ei) : -1;
          int mine[1];
          int k = 0;
          if (e >= 0 && (unsigned)ld_i(reinterpret_cast<const int*>(P.qmark) + e) == mk) mine[k++] = e;
          if (__any_sync(kFull, k > 0)) wb_push(wb, mine, k, P.wl0, &P.st->wl_count[0], P.E, P.st);
        }
        wb_flush(wb, P.wl0, &P.st->wl_count[0], P.E, P.st);
        g.sync();
        phase_lawson<false>(g, Q, 0, stamp, lc, 0);
      } else {
        const unsigned du = stamp++;  // first sight of an edge in this pass (cand is free until the flip rounds)
        if (gtid == 0) P.st->wl_count[1] = 0;
        g.sync();
        WarpBuf wb{s_wbuf[0][threadIdx.x >> 5], 0};
        for (int base = spread_tid() - (int)(threadIdx.x & 31); base < nw; base += stride) {
          const int i = base + (int)(threadIdx.x & 31);
          int mine[1];
          int k = 0;
          if (i < nw) {
            const int e = ld_i(P.wl0 + i);
            if (e >= 0 && e < P.E && atomicMax(P.cand + e, du) < du) mine[k++] = e;
          }
          if (__any_sync(kFull, k > 0)) wb_push(wb, mine, k, P.wl1, &P.st->wl_count[1], P.E, P.st);
        }
        wb_flush(wb, P.wl1, &P.st->wl_count[1], P.E, P.st);
        if (gtid == 0) P.st->wl_count[0] = 0;
        g.sync();
        phase_lawson<false>(g, Q, 1, stamp, lc, 0);
      }
      g.sync();
    }
    timeline(P, 46);
  }
  flush_counters(P, lc);
  return stamp;
}

// One kinetic step in one persistent launch: (move +) classify; if a face is
// inverted, repair; then Lawson rounds to the Delaunay triangulation.
__global__ void __launch_bounds__(kThreads, 3) k_step(KParams P) {
  cg::grid_group g = cg::this_grid();
  LocalCounters lc = {0, 0, 0, 0, 0, 0, 0};
  unsigned stamp = ld_i(reinterpret_cast<const int*>(&P.st->epoch));
  timeline(P, 0);
  const unsigned q0 = stamp++;
  const unsigned sc0 = stamp++;
  phase_classify<true>(g, P, q0, sc0, lc);
  g.sync();
  phase_classify_hard<true>(g, P, q0, sc0, lc);
  timeline(P, 1);
  const int inverted = ld_i(&P.st->inverted);
  if (inverted == 0) phase_lawson<true, true>(g, P, 0, stamp, lc, sc0);
  else stamp = repair_step(g, P, stamp, q0);
  flush_counters(P, lc);
  // No closing grid barrier: each block leaves when its own work is done and
  // the last one to leave publishes the launch.  The block barrier orders its
  // threads' counter updates before thread 0's fence, and the fence (which is
  // cumulative) orders them before the block's arrival.
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicMax(&P.st->stamp_max, stamp);
    __threadfence();
    if (atomicAdd(&P.st->arrived, 1u) == gridDim.x - 1) {
      __threadfence();
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      P.st->ts[kTimeline - 1] = t;
      finish_launch(P, __ldcg(&P.st->stamp_max));
      P.st->arrived = 0;
      P.st->stamp_max = 0;
    }
  }
}

// The initial triangulation: parallel insertion rounds from the bounding square.
__global__ void __launch_bounds__(kThreads) k_build(KParams P) {
  cg::grid_group g = cg::this_grid();
  LocalCounters lc = {0, 0, 0, 0, 0, 0, 0};
  unsigned stamp = ld_i(reinterpret_cast<const int*>(&P.st->epoch));
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  phase_insert(g, P, stamp, lc);
  flush_counters(P, lc);
  g.sync();
  if (gtid == 0) finish_launch(P, stamp);
}

// ---------------------------------------------------------------------------
// Host side.
static thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace mcl

void mcl_set_last_error(const std::string& msg) { mcl::g_last_error = msg; }

namespace mcl {

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? MCL_ERR_OUT_OF_MEMORY : MCL_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

void free_mesh(mcl_mesh* m) {
  if (!m) return;
  void* ptrs[] = {m->pos[0], m->pos[1], m->ev, m->en, m->vhe, m->vfix, m->cand, m->win, m->qmark, m->efa, m->hard,
                  m->wl[0], m->wl[1], m->vl[0], m->vl[1], m->vmark, m->claim, m->vfree, m->vhint,
                  m->vaux, m->vloc, m->vlocf, m->target, m->vprev, m->vl2, m->dstage, m->scratch, m->st,
                  m->vcomp, m->vroot, m->cbase, m->table, m->smark, m->smove, m->fnew, m->act_dev,
                  m->bg_cell, m->bg_src, m->bg_perm, m->bg_pos, m->bg_count, m->bg_start, m->bg_cursor,
                  m->bg_tmp, m->bg_par, m->aos_tmp};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (m->dstage2) cudaFree(m->dstage2);
  if (m->stats_dev) cudaFree(m->stats_dev);
  if (m->copy_stream) {
    cudaStreamSynchronize(m->copy_stream);
    cudaStreamDestroy(m->copy_stream);
    for (int i = 0; i < 2; ++i) {
      cudaEventDestroy(m->ev_copied[i]);
      cudaEventDestroy(m->ev_used[i]);
    }
  }
  if (m->st_host) cudaFreeHost(m->st_host);
  if (m->act_host) cudaFreeHost(m->act_host);
  if (m->bg_par_host) cudaFreeHost(m->bg_par_host);
  delete[] m->comp_host;
  delete[] m->act_list;
  delete[] m->dirty;
  delete m;
}

const float2* valid_positions(const mcl_mesh* m) { return m->valid_cur ? m->pos[m->cur] : m->pos[m->cur ^ 1]; }

ActV act_of(const mcl_mesh* m) {
  ActV a;
  a.n = m->nact;
  a.V_it = m->nact ? m->act_V : (int)m->V;
  a.pre = m->nact ? m->act_dev + 2 * m->ncomp + 1 : nullptr;
  a.v0 = m->nact ? m->act_dev + 3 * m->ncomp + 2 : nullptr;
  return a;
}

int alloc_mesh(int64_t V, int64_t E, mcl_mesh** out) {
  if (V < 4 || E < 5 || V > (1ll << 30) || E > (1ll << 29))
    return fail(MCL_ERR_INVALID_ARGUMENT, "mesh size out of range");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  mcl_mesh* m = new mcl_mesh();
  std::memset(m, 0, sizeof(*m));
  m->device = dev;
  m->V = V;
  m->E = E;
  m->T = 2 * (V - 4) + 2;
  m->cur = 0;
  m->valid_cur = true;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  A((void**)&m->pos[0], 8 * V);
  A((void**)&m->pos[1], 8 * V);
  A((void**)&m->ev, 16 * E);
  A((void**)&m->en, 16 * E);
  A((void**)&m->vhe, 4 * V);
  A((void**)&m->vfix, V);
  A((void**)&m->cand, 4 * E);
  A((void**)&m->win, 4 * E);
  A((void**)&m->qmark, 4 * E);
  A((void**)&m->efa, 8 * E);
  A((void**)&m->hard, 4 * E);
  A((void**)&m->wl[0], 4 * E);
  A((void**)&m->wl[1], 4 * E);
  A((void**)&m->vl[0], 4 * V);
  A((void**)&m->vl[1], 4 * V);
  A((void**)&m->vmark, 4 * V);
  A((void**)&m->claim, 8 * 2 * E);
  A((void**)&m->vfree, 12 * V);
  A((void**)&m->vhint, 4 * V);
  A((void**)&m->vaux, 4 * V);
  A((void**)&m->vloc, 4 * V);
  A((void**)&m->vlocf, 4 * V);
  A((void**)&m->target, 8 * V);
  A((void**)&m->dstage, 8 * V);
  A((void**)&m->scratch, 64);
  A((void**)&m->st, sizeof(DevState));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&m->st_host, sizeof(DevState));
  if (e != cudaSuccess) {
    free_mesh(m);
    return cuda_fail(e, "cudaMalloc(mesh)");
  }
  e = cudaMemset(m->cand, 0, 4 * E);
  if (e == cudaSuccess) e = cudaMemset(m->win, 0, 4 * E);
  if (e == cudaSuccess) e = cudaMemset(m->qmark, 0, 4 * E);
  if (e == cudaSuccess) e = cudaMemset(m->claim, 0, 16 * E);
  if (e == cudaSuccess) e = cudaMemset(m->vaux, 0xff, 4 * V);
  if (e == cudaSuccess) e = cudaMemset(m->vhint, 0xff, 4 * V);
  if (e == cudaSuccess) e = cudaMemset(m->vmark, 0, 4 * V);
  DevState s;
  std::memset(&s, 0, sizeof(s));
  s.epoch = 1;
  if (e == cudaSuccess) e = cudaMemcpy(m->st, &s, sizeof(s), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_mesh(m);
    return cuda_fail(e, "mesh init");
  }
  int nsm = 0, per_sm = 0;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int per_sm2 = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step, kThreads, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_build, kThreads, 0);
  if (e != cudaSuccess || per_sm < 1 || per_sm2 < 1) {
    free_mesh(m);
    return cuda_fail(e == cudaSuccess ? cudaErrorInvalidConfiguration : e, "occupancy(k_step, k_build)");
  }
  m->coop_threads = kThreads;
  m->nsm = nsm;
  m->max_blocks_per_sm = per_sm;
  m->tail_items = kTailItems;
  m->substeps = kSubsteps;
  m->ncomp = 1;
  m->coop_blocks = nsm * per_sm;
  m->repair_blocks = nsm * per_sm2;
  *out = m;
  return MCL_OK;
}

// Convert and validate the reference AoS arrays; returns false on malformed input.
static bool aos_to_soa(const mcl_aos_view* a, std::vector<int4>& ev, std::vector<int4>& en, std::vector<int>& vhe,
                       std::string& why) {
  const int64_t V = a->V, HE = a->HE, E = HE / 2;
  if (HE % 2 || V < 4 || E < 5) { why = "bad sizes"; return false; }
  const int32_t* he = a->he;
  ev.assign(E, make_int4(0, 0, 0, 0));
  en.assign(E, make_int4(0, 0, 0, 0));
  std::vector<int> prev(HE, -1);
  for (int64_t h = 0; h < HE; ++h) {
    const int nx = he[4 * h], v = he[4 * h + 1], t = he[4 * h + 2], op = he[4 * h + 3];
    if (nx < 0 || nx >= HE || v < 0 || v >= V) { why = "half-edge index out of range"; return false; }
    if (t >= 0 && (op < 0 || op >= V)) { why = "opposite vertex out of range"; return false; }
    if (prev[nx] != -1) { why = "two half-edges share a next"; return false; }
    prev[nx] = (int)h;
  }
  for (int64_t h = 0; h < HE; ++h) {
    const int nx = he[4 * h];
    // the twin's origin must be this half-edge's destination
    if (he[4 * (h ^ 1) + 1] != he[4 * nx + 1]) { why = "twin/next inconsistent"; return false; }
    if (he[4 * h + 2] >= 0) {
      const int n2 = he[4 * nx], n3 = he[4 * n2];
      if (n3 != h) { why = "inner face is not a triangle"; return false; }
      if (he[4 * h + 3] != he[4 * n2 + 1]) { why = "opposite vertex inconsistent"; return false; }
    }
  }
  for (int64_t e = 0; e < E; ++e) {
    const int32_t* h0 = he + 8 * e;
    const int32_t* h1 = h0 + 4;
    ev[e] = make_int4(h0[1], h1[1], h0[2] >= 0 ? h0[3] : -1, h1[2] >= 0 ? h1[3] : -1);
    en[e] = make_int4(h0[0], prev[2 * e], h1[0], prev[2 * e + 1]);
  }
  vhe.assign(V, -1);
  for (int64_t v = 0; v < V; ++v) {
    const int h = a->v[2 * v + 1];
    if (h < 0 || h >= HE || he[4 * h + 1] != v) { why = "vertex he is not outgoing"; return false; }
    vhe[v] = h;
  }
  return true;
}

static int upload_soa(mcl_mesh* m, const mcl_float2* pos, const std::vector<int4>& ev, const std::vector<int4>& en,
                      const std::vector<int>& vhe) {
  std::vector<unsigned char> fix(m->V, 0);
  for (int i = 0; i < 4 && i < m->V; ++i) fix[i] = 1;
  m->cur = 0;
  m->valid_cur = true;
  CK(cudaMemcpy(m->pos[0], pos, 8 * m->V, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->pos[1], pos, 8 * m->V, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->ev, ev.data(), 16 * m->E, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->en, en.data(), 16 * m->E, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->vhe, vhe.data(), 4 * m->V, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->vfix, fix.data(), m->V, cudaMemcpyHostToDevice));
  return MCL_OK;
}

// transferToHost for the vertices [vb, vb + nv) and edges [eb, eb + ne) of one
// component (the whole mesh, or one mesh of a batch), renumbered from 0.
int download_range(mcl_mesh* m, int64_t vb, int64_t nv, int64_t eb, int64_t ne, int64_t T, mcl_float2* pos,
                   int32_t* v, int32_t* he, int32_t* t) {
  CK(cudaDeviceSynchronize());
  const int64_t V = nv, E = ne, HE = 2 * E;
  if (pos) CK(cudaMemcpy(pos, m->pos[m->cur] + vb, 8 * V, cudaMemcpyDeviceToHost));
  if (!v && !he && !t) return MCL_OK;
  std::vector<int4> ev(E), en(E);
  std::vector<int> vhe(V);
  CK(cudaMemcpy(ev.data(), m->ev + eb, 16 * E, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(en.data(), m->en + eb, 16 * E, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vhe.data(), m->vhe + vb, 4 * V, cudaMemcpyDeviceToHost));
  const int hb = (int)(2 * eb), vbi = (int)vb;
  bool bad = false;
  auto lv = [&](int x) {
    if (x < 0) return -1;
    x -= vbi;
    if (x >= V || x < 0) bad = true;
    return x;
  };
  auto lh = [&](int x) {
    if (x < 0) return -1;
    x -= hb;
    if (x >= HE || x < 0) bad = true;
    return x;
  };
  for (int64_t e = 0; e < E; ++e) {
    ev[e] = make_int4(lv(ev[e].x), lv(ev[e].y), lv(ev[e].z), lv(ev[e].w));
    en[e] = make_int4(lh(en[e].x), lh(en[e].y), lh(en[e].z), lh(en[e].w));
  }
  for (int64_t i = 0; i < V; ++i) vhe[i] = lh(vhe[i]);
  if (bad) return fail(MCL_ERR_DEGENERATE_INPUT, "download: index outside the component");
  auto org = [&](int64_t h) { const int4& q = ev[h >> 1]; return (h & 1) ? q.y : q.x; };
  auto apex = [&](int64_t h) { const int4& q = ev[h >> 1]; return (h & 1) ? q.w : q.z; };
  auto nxt = [&](int64_t h) { const int4& q = en[h >> 1]; return (h & 1) ? q.z : q.x; };
  auto prv = [&](int64_t h) { const int4& q = en[h >> 1]; return (h & 1) ? q.w : q.y; };
  std::vector<int> face(HE, -1);
  int64_t nf = 0;
  std::vector<int> owner;
  owner.reserve(T);
  for (int64_t h = 0; h < HE; ++h) {
    if (apex(h) < 0 || org(h) < 0) continue;
    const int64_t n = nxt(h), p = prv(h);
    if (h < n && h < p) {
      face[h] = (int)nf++;
      owner.push_back((int)h);
    }
  }
  for (int64_t h = 0; h < HE; ++h) {
    if (apex(h) < 0 || org(h) < 0) continue;
    const int64_t n = nxt(h), p = prv(h);
    face[h] = face[std::min(h, std::min(n, p))];
  }
  if (he) {
    for (int64_t h = 0; h < HE; ++h) {
      he[4 * h] = nxt(h);
      he[4 * h + 1] = org(h);
      he[4 * h + 2] = face[h];
      he[4 * h + 3] = apex(h) >= 0 ? apex(h) : -1;
    }
  }
  if (v) {
    for (int64_t i = 0; i < V; ++i) {
      v[2 * i] = (int)i;
      v[2 * i + 1] = vhe[i];
    }
  }
  if (t) {
    for (int64_t i = 0; i < (int64_t)owner.size() && i < T; ++i) t[i] = owner[i];
  }
  if (nf != T) return fail(MCL_ERR_DEGENERATE_INPUT, "face count mismatch on download");
  return MCL_OK;
}

static KParams make_params(mcl_mesh* m, int mode) {
  KParams P;
  std::memset(&P, 0, sizeof(P));
  P.V = (int)m->V;
  P.E = (int)m->E;
  P.ev = m->ev;
  P.en = m->en;
  P.vhe = m->vhe;
  P.vfix = m->vfix;
  P.cand = m->cand;
  P.win = m->win;
  P.qmark = m->qmark;
  P.efa = m->efa;
  P.hard = m->hard;
  P.wl0 = m->wl[0];
  P.wl1 = m->wl[1];
  P.vl0 = m->vl[0];
  P.vl1 = m->vl[1];
  P.vmark = m->vmark;
  P.claim = m->claim;
  P.vfree = m->vfree;
  P.vhint = m->vhint;
  P.vaux = m->vaux;
  P.vloc = m->vloc;
  P.vlocf = m->vlocf;
  P.target = m->target;
  P.vprev = m->vprev;
  P.vl2 = m->vl2;
  P.st = m->st;
  P.mode = mode;
  P.max_rounds = 1 << 16;
  P.walk_cap = 1 << 18;
  P.tail_items = m->tail_items;
  P.rm_tile = m->rm_tile;
  P.substeps = m->vl2 ? m->substeps : 0;  // no scratch, no sub-steps
  P.vroot = m->vroot;
  P.nact = m->nact;
  P.E_it = m->nact ? m->act_E : (int)m->E;
  P.V_it = m->nact ? m->act_V : (int)m->V;
  if (m->nact) {
    const int64_t nc = m->ncomp;
    P.act_epre = m->act_dev;
    P.act_e0 = m->act_dev + nc + 1;
    P.act_vpre = m->act_dev + 2 * nc + 1;
    P.act_v0 = m->act_dev + 3 * nc + 2;
  }
  return P;
}

static int launch_engine(mcl_mesh* m, KParams& P, cudaStream_t s) {
  void* args[] = {&P};
  CK(cudaLaunchCooperativeKernel((void*)k_step, dim3(m->coop_blocks), dim3(m->coop_threads), args, 0, s));
  return MCL_OK;
}

static void fill_stats_from(const unsigned long long* c, int status, int site, mcl_step_stats* o);

static void fill_stats(const DevState& s, mcl_step_stats* o) {
  fill_stats_from(s.last, s.last_status, s.last_site, o);
  o->failed_launches = s.last_status != MCL_OK ? 1 : 0;
}

static void fill_stats_from(const unsigned long long* c, int status, int site, mcl_step_stats* o) {
  struct { const unsigned long long* c; } s{c};
  o->inverted_faces = (int64_t)s.c[C_INVERTED];
  o->reverted_vertices = (int64_t)s.c[C_REVERTED];
  o->removed_vertices = (int64_t)s.c[C_REMOVED];
  o->lawson_flips = (int64_t)s.c[C_LAWSON_FLIPS];
  o->lawson_rounds = (int64_t)s.c[C_LAWSON_ROUNDS];
  o->removal_flips = (int64_t)s.c[C_REMOVAL_FLIPS];
  o->insert_rounds = (int64_t)s.c[C_INSERT_ROUNDS];
  o->incircle_tests = (int64_t)s.c[C_INCIRCLE];
  o->incircle_fp64 = (int64_t)s.c[C_INCIRCLE_FP64];
  o->incircle_exact = (int64_t)s.c[C_INCIRCLE_EXACT];
  o->orient_fp64 = (int64_t)s.c[C_ORIENT_FP64];
  o->orient_exact = (int64_t)s.c[C_ORIENT_EXACT];
  o->sos_decisions = (int64_t)s.c[C_SOS];
  o->substep_vertices = (int64_t)s.c[C_SUBSTEP_DONE];
  o->status = status;
  o->error_site = site;
  o->failed_launches = 0;
}

static int finish(mcl_mesh* m, cudaStream_t s, mcl_step_stats* stats) {
  if (!stats) return MCL_OK;
  CK(cudaMemcpyAsync(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  fill_stats(*m->st_host, stats);
  m->last_status = m->st_host->last_status;
  if (m->st_host->last_status != MCL_OK)
    return fail(m->st_host->last_status,
                std::string("device status: ") + mcl_status_string(m->st_host->last_status));
  return MCL_OK;
}

// Run the engine.  Position buffers: pos[cur] holds the positions the mesh
// must be repaired to; when valid_cur is false (points were moved since the
// last validated state) pos[cur^1] holds the validated positions.  A fused move
// (valid_cur true) reads pos[cur] and writes pos[cur^1].
// stats_mapped (may be NULL): device-visible pinned host record the launch
// itself fills at its end.
static int run_step(mcl_mesh* m, int move_mode, const float2* d, cudaStream_t s, mcl_step_stats* stats,
                    mcl_step_stats* stats_mapped = nullptr) {
  KParams P = make_params(m, ENGINE_STEP);
  P.stats_out = stats_mapped;
  if (move_mode != MOVE_NONE) {
    if (m->dirty) {
      // the launch writes the other position buffer for the active meshes
      // only: the inactive meshes whose buffers differ are brought in step first
      if (m->nact) {
        std::vector<unsigned char> on((size_t)m->ncomp, 0);
        for (int i = 0; i < m->nact; ++i) on[(size_t)m->act_list[i]] = 1;
        int64_t stale = 0;
        for (int64_t c = 0; c < m->ncomp; ++c) stale += (!on[(size_t)c] && m->dirty[c]) ? 1 : 0;
        if (stale > 16) {
          // many small copies cost more than one copy of every position (the
          // launch rewrites the active meshes' part anyway)
          CK(cudaMemcpyAsync(m->pos[m->cur ^ 1], m->pos[m->cur], 8 * m->V, cudaMemcpyDeviceToDevice, s));
          std::memset(m->dirty, 0, (size_t)m->ncomp);
        } else {
          for (int64_t c = 0; c < m->ncomp; ++c) {
            if (on[(size_t)c] || !m->dirty[c]) continue;
            const int64_t v0 = m->comp_host[4 * c], nv = m->comp_host[4 * c + 1];
            CK(cudaMemcpyAsync(m->pos[m->cur ^ 1] + v0, m->pos[m->cur] + v0, 8 * nv, cudaMemcpyDeviceToDevice, s));
            m->dirty[c] = 0;
          }
        }
        for (int i = 0; i < m->nact; ++i) m->dirty[m->act_list[i]] = 1;
      } else {
        std::memset(m->dirty, 1, (size_t)m->ncomp);
      }
    }
    P.pos_old = m->pos[m->cur];
    P.pos = m->pos[m->cur ^ 1];
    P.move_mode = move_mode;
    P.disp = d;
    m->cur ^= 1;
  } else {
    P.pos = m->pos[m->cur];
    P.pos_old = m->valid_cur ? m->pos[m->cur] : m->pos[m->cur ^ 1];
  }
  P.sparse_ok = m->delaunay ? 1 : 0;
  int rc = launch_engine(m, P, s);
  if (rc != MCL_OK) return rc;
  m->valid_cur = true;
  m->delaunay = true;  // a step ends Delaunay (or with an error status)
  return finish(m, s, stats);
}

// Structural invariants of the device mesh (counted per kind):
//  0 next/prev not inverse   1 inner face not a 3-cycle   2 apex != origin(prev)
//  3 origin(next) != origin(twin)   4 vhe not outgoing   5 face not positive
//  6 dead edge   7 index out of range
__global__ void k_validate(KParams P, unsigned long long* bad) {
  LocalCounters lc = {0, 0, 0, 0, 0, 0, 0};
  const int HE = 2 * P.E;
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < HE + P.V; h += gridDim.x * blockDim.x) {
    if (h >= HE) {
      const int v = h - HE;
      const int o = ld_i(P.vhe + v);
      if (o < 0) continue;
      if (bad_h(P, o)) { atomicAdd(bad + 7, 1ull); continue; }
      if (he_origin(P, o) != v) atomicAdd(bad + 4, 1ull);
      continue;
    }
    if (he_origin(P, h) < 0) { atomicAdd(bad + 6, 1ull); continue; }
    const int n = he_next(P, h), p = he_prev(P, h);
    if (bad_h(P, n) || bad_h(P, p)) { atomicAdd(bad + 7, 1ull); continue; }
    if (he_prev(P, n) != h || he_next(P, p) != h) atomicAdd(bad + 0, 1ull);
    if (he_origin(P, n) != he_origin(P, h ^ 1)) atomicAdd(bad + 3, 1ull);
    const int ap = he_apex(P, h);
    if (ap >= 0) {
      if (he_next(P, n) != p) atomicAdd(bad + 1, 1ull);
      if (ap != he_origin(P, p)) atomicAdd(bad + 2, 1ull);
      if (h < n && h < p) {
        const int a = he_origin(P, h), b = he_origin(P, n), c = he_origin(P, p);
        if (bad_v(P, a) || bad_v(P, b) || bad_v(P, c)) { atomicAdd(bad + 7, 1ull); continue; }
        if (orient_v(P, ldpos(P, a), ldpos(P, b), ldpos(P, c), lc) <= 0) atomicAdd(bad + 5, 1ull);
      }
    }
  }
}

}  // namespace mcl

using namespace mcl;

// ---------------------------------------------------------------------------
// Plain move kernels for the API calls that only move (movePoints without a step).
__global__ void k_move_only(int V, const unsigned char* fix, const float2* src, float2* dst, const float2* d,
                            const float* dt, const float2* vel, int mode) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  float2 p = src[v];
  if (!fix[v]) {
    if (mode == MOVE_DISPLACE) {
      p.x = fadd(p.x, d[v].x);
      p.y = fadd(p.y, d[v].y);
    } else {
      p.x = fadd(p.x, fmul(vel[v].x, dt[v]));
      p.y = fadd(p.y, fmul(vel[v].y, dt[v]));
    }
  }
  dst[v] = p;
}

extern "C" {

const char* mcl_status_string(int status) {
  switch (status) {
    case MCL_OK: return "ok";
    case MCL_ERR_INVALID_ARGUMENT: return "invalid argument";
    case MCL_ERR_CUDA: return "CUDA error";
    case MCL_ERR_OUT_OF_MEMORY: return "out of device memory";
    case MCL_ERR_NO_CONVERGENCE: return "iteration cap reached";
    case MCL_ERR_CAPACITY: return "buffer capacity exceeded";
    case MCL_ERR_DEGENERATE_INPUT: return "degenerate input (duplicate point, point outside the bounding square, or invalid mesh)";
    case MCL_ERR_PREDICATE: return "exact predicate capacity exceeded";
    case MCL_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* mcl_last_error(void) { return mcl::g_last_error.c_str(); }
int mcl_version(void) { return 1; }

int mcl_mesh_totals(mcl_mesh* m, mcl_step_stats* totals, int64_t* calls) {
  if (!m || !totals) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  const DevState& t = *m->st_host;
  fill_stats_from(t.tot, t.last_status, t.last_site, totals);
  totals->failed_launches = (int64_t)t.failed;
  if (calls) *calls = (int64_t)t.calls;
  return MCL_OK;
}

int mcl_debug_timeline(mcl_mesh* m, int64_t* out48) {
  if (!m || !out48) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  for (int i = 0; i < kTimeline; ++i) out48[i] = (int64_t)m->st_host->ts[i];
  return MCL_OK;
}

int mcl_debug_insert_timeline(mcl_mesh* m, int64_t* out64) {
  if (!m || !out64) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 64; ++i) out64[i] = (int64_t)m->st_host->ts_insert[i];
  return MCL_OK;
}

int mcl_debug_remove_timeline(mcl_mesh* m, int64_t* out64) {
  if (!m || !out64) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 64; ++i) out64[i] = (int64_t)m->st_host->ts_remove[i];
  for (int i = 0; i < 16; ++i) {
    out64[64 + i] = (int64_t)m->st_host->rm_slow[i];
    out64[80 + i] = (int64_t)m->st_host->rm_uncached[i];
  }
  // the next launches accumulate from zero
  static_assert(offsetof(DevState, rm_uncached) == offsetof(DevState, rm_slow) + 16 * 8, "layout");
  unsigned long long zero[32] = {};
  CK(cudaMemcpy(reinterpret_cast<char*>(m->st) + offsetof(DevState, rm_slow), zero, sizeof(zero),
                cudaMemcpyHostToDevice));
  return MCL_OK;
}

int mcl_debug_counters(mcl_mesh* m, int64_t* out, int n) {
  if (!m || !out || n < 1) return fail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  for (int i = 0; i < n && i < C_COUNT; ++i) out[i] = (int64_t)m->st_host->last[i];
  return C_COUNT;
}

int mcl_debug_state(mcl_mesh* m, int32_t* out68) {
  if (!m || !out68) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  CK(cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 68; ++i) out68[i] = m->st_host->dbg[i];
  return MCL_OK;
}

int mcl_mesh_validate(mcl_mesh* m, int64_t* counts8) {
  if (!m || !counts8) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  KParams P = make_params(m, ENGINE_STEP);
  P.pos = m->pos[m->cur];
  P.pos_old = P.pos;
  CK(cudaMemset(m->scratch, 0, 64));
  k_validate<<<1024, 256>>>(P, m->scratch);
  CK(cudaGetLastError());
  unsigned long long h[8];
  CK(cudaMemcpy(h, m->scratch, 64, cudaMemcpyDeviceToHost));
  for (int i = 0; i < 8; ++i) counts8[i] = (int64_t)h[i];
  return MCL_OK;
}

int mcl_mesh_create_from_aos(const mcl_aos_view* a, mcl_mesh** out) {
  if (!a || !out || !a->pos || !a->v || !a->he) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<int4> ev, en;
  std::vector<int> vhe;
  std::string why;
  if (!aos_to_soa(a, ev, en, vhe, why)) return fail(MCL_ERR_INVALID_ARGUMENT, "malformed mesh: " + why);
  mcl_mesh* m = nullptr;
  int rc = alloc_mesh(a->V, a->HE / 2, &m);
  if (rc != MCL_OK) return rc;
  rc = upload_soa(m, a->pos, ev, en, vhe);
  if (rc != MCL_OK) { free_mesh(m); return rc; }
  m->delaunay = false;  // a caller's mesh: the first step classifies every edge
  *out = m;
  return MCL_OK;
}

int mcl_mesh_upload_aos(mcl_mesh* m, const mcl_aos_view* a) {
  if (!m || !a) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (a->V != m->V || a->HE != 2 * m->E) return fail(MCL_ERR_INVALID_ARGUMENT, "size mismatch");
  std::vector<int4> ev, en;
  std::vector<int> vhe;
  std::string why;
  if (!aos_to_soa(a, ev, en, vhe, why)) return fail(MCL_ERR_INVALID_ARGUMENT, "malformed mesh: " + why);
  m->delaunay = false;
  return upload_soa(m, a->pos, ev, en, vhe);
}

int mcl_mesh_destroy(mcl_mesh* m) {
  if (!m) return MCL_OK;
  cudaDeviceSynchronize();
  free_mesh(m);
  return MCL_OK;
}

int mcl_mesh_sizes(const mcl_mesh* m, int64_t* V, int64_t* HE, int64_t* T) {
  if (!m) return fail(MCL_ERR_INVALID_ARGUMENT, "null mesh");
  if (V) *V = m->V;
  if (HE) *HE = 2 * m->E;
  if (T) *T = m->T;
  return MCL_OK;
}

int mcl_mesh_positions(mcl_mesh* m, mcl_float2** pos_dev) {
  if (!m || !pos_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  *pos_dev = reinterpret_cast<mcl_float2*>(m->pos[m->cur]);
  return MCL_OK;
}

int mcl_mesh_copy_positions(mcl_mesh* m, mcl_float2* dst, int to_host, void* stream) {
  if (!m || !dst) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  CK(cudaMemcpyAsync(dst, m->pos[m->cur], 8 * m->V, to_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                     (cudaStream_t)stream));
  if (to_host) CK(cudaStreamSynchronize((cudaStream_t)stream));
  return MCL_OK;
}

int mcl_mesh_download_aos(mcl_mesh* m, mcl_float2* pos, int32_t* v, int32_t* he, int32_t* t) {
  if (!m) return fail(MCL_ERR_INVALID_ARGUMENT, "null mesh");
  return download_range(m, 0, m->V, 0, m->E, m->T, pos, v, he, t);
}

int mcl_move(mcl_mesh* m, const mcl_float2* d_dev, void* stream) {
  if (!m || !d_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (m->nact) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_move: a subset of the batch is active (use mcl_step)");
  if (m->dirty) std::memset(m->dirty, 1, (size_t)m->ncomp);
  cudaStream_t s = (cudaStream_t)stream;
  const int src = m->cur, dst = m->valid_cur ? m->cur ^ 1 : m->cur;
  k_move_only<<<(unsigned)((m->V + 255) / 256), 256, 0, s>>>((int)m->V, m->vfix, m->pos[src], m->pos[dst],
                                                              (const float2*)d_dev, nullptr, nullptr, MOVE_DISPLACE);
  CK(cudaGetLastError());
  m->cur = dst;
  m->valid_cur = false;
  return MCL_OK;
}

int mcl_integrate(mcl_mesh* m, const float* dt_dev, const mcl_float2* v_dev, void* stream) {
  if (!m || !dt_dev || !v_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (m->nact) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_integrate: a subset of the batch is active (use mcl_step)");
  if (m->dirty) std::memset(m->dirty, 1, (size_t)m->ncomp);
  cudaStream_t s = (cudaStream_t)stream;
  const int src = m->cur, dst = m->valid_cur ? m->cur ^ 1 : m->cur;
  k_move_only<<<(unsigned)((m->V + 255) / 256), 256, 0, s>>>((int)m->V, m->vfix, m->pos[src], m->pos[dst], nullptr,
                                                              dt_dev, (const float2*)v_dev, MOVE_INTEGRATE);
  CK(cudaGetLastError());
  m->cur = dst;
  m->valid_cur = false;
  return MCL_OK;
}

int mcl_untangle(mcl_mesh* m, void* stream, mcl_step_stats* stats) {
  if (!m) return fail(MCL_ERR_INVALID_ARGUMENT, "null mesh");
  return run_step(m, MOVE_NONE, nullptr, (cudaStream_t)stream, stats);
}

int mcl_delaunay_restore(mcl_mesh* m, void* stream, mcl_step_stats* stats) {
  if (!m) return fail(MCL_ERR_INVALID_ARGUMENT, "null mesh");
  return run_step(m, MOVE_NONE, nullptr, (cudaStream_t)stream, stats);
}

int mcl_step(mcl_mesh* m, const mcl_float2* d_dev, void* stream, mcl_step_stats* stats) {
  if (!m || !d_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (!m->valid_cur) {
    int rc = mcl_move(m, d_dev, stream);
    if (rc != MCL_OK) return rc;
    return run_step(m, MOVE_NONE, nullptr, (cudaStream_t)stream, stats);
  }
  return run_step(m, MOVE_DISPLACE, (const float2*)d_dev, (cudaStream_t)stream, stats);
}

int mcl_step_host(mcl_mesh* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats) {
  if (!m || !d_host) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(m->dstage, d_host, 8 * m->V, cudaMemcpyHostToDevice, s));
  return mcl_step(m, reinterpret_cast<const mcl_float2*>(m->dstage), stream, stats);
}

}  // extern "C"

namespace mcl {
// the counters of the last launch as an mcl_step_stats, in device memory
__global__ void k_publish_stats(const DevState* st, mcl_step_stats* out) {
  if (threadIdx.x == 0) publish_stats(st, out);
}
}  // namespace mcl

extern "C" {

int mcl_step_host_async(mcl_mesh* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats_pinned) {
  if (!m || !d_host) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (!m->valid_cur || m->nact) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_step_host_async: needs a validated mesh "
                                                                      "and every mesh of a batch active");
  cudaStream_t s = (cudaStream_t)stream;
  if (!m->copy_stream) {
    CK(cudaMalloc((void**)&m->dstage2, 8 * m->V));
    CK(cudaMalloc((void**)&m->stats_dev, 2 * sizeof(mcl_step_stats)));
    CK(cudaStreamCreateWithFlags(&m->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
      CK(cudaEventCreateWithFlags(&m->ev_copied[i], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&m->ev_used[i], cudaEventDisableTiming));
      CK(cudaEventRecord(m->ev_used[i], m->copy_stream));
    }
  }
  const int k = m->stage_idx;
  m->stage_idx ^= 1;
  float2* buf = k ? m->dstage2 : m->dstage;
  // the copy into buffer k waits for the step that last read it, then runs on
  // the copy stream, overlapping the step in flight on `stream`
  CK(cudaStreamWaitEvent(m->copy_stream, m->ev_used[k], 0));
  CK(cudaMemcpyAsync(buf, d_host, 8 * m->V, cudaMemcpyHostToDevice, m->copy_stream));
  CK(cudaEventRecord(m->ev_copied[k], m->copy_stream));
  CK(cudaStreamWaitEvent(s, m->ev_copied[k], 0));
  // a pinned record the device can address is filled by the step itself
  // (no publishing kernel and copy between steps); otherwise it is copied
  mcl_step_stats* mapped = nullptr;
  if (stats_pinned && cudaHostGetDevicePointer((void**)&mapped, stats_pinned, 0) != cudaSuccess) {
    (void)cudaGetLastError();
    mapped = nullptr;
  }
  const int rc = run_step(m, MOVE_DISPLACE, buf, s, nullptr, mapped);
  if (rc != MCL_OK) return rc;
  CK(cudaEventRecord(m->ev_used[k], s));
  if (stats_pinned && !mapped) {
    k_publish_stats<<<1, 32, 0, s>>>(m->st, m->stats_dev + k);
    CK(cudaMemcpyAsync(stats_pinned, m->stats_dev + k, sizeof(mcl_step_stats), cudaMemcpyDeviceToHost, s));
  }
  return MCL_OK;
}

int mcl_mesh_last_status(mcl_mesh* m, void* stream, mcl_step_stats* stats) {
  if (!m) return fail(MCL_ERR_INVALID_ARGUMENT, "null mesh");
  mcl_step_stats tmp;
  return finish(m, (cudaStream_t)stream, stats ? stats : &tmp);
}

// HostTriangulation::addDelaunayPoints on the GPU: Morton sort on the host with
// the reference's comparator (include/Host_Triangulation.h:287-300, std::sort so
// that ties resolve as in the reference), then parallel insertion rounds.
// libmorton's m2D_e_LUT<uint_fast32_t,uint_fast32_t>(x, y) as the reference
// calls it: each float truncated to an integer (two's complement for negative
// values), the low 32 bits of x in the even bit positions, y in the odd ones.
static uint64_t mcl_morton_key(float x, float y) {
  auto spread = [](uint64_t w) {
    w &= 0xFFFFFFFFull;
    w = (w | (w << 16)) & 0x0000FFFF0000FFFFull;
    w = (w | (w << 8)) & 0x00FF00FF00FF00FFull;
    w = (w | (w << 4)) & 0x0F0F0F0F0F0F0F0Full;
    w = (w | (w << 2)) & 0x3333333333333333ull;
    w = (w | (w << 1)) & 0x5555555555555555ull;
    return w;
  };
  return spread((uint64_t)(int64_t)x) | (spread((uint64_t)(int64_t)y) << 1);
}

int mcl_mesh_build(mcl_float2* pts, int64_t n, mcl_mesh** out) {
  if (!pts || !out || n < 0) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  const float lo = -10000000.0f, hi = 10000000.0f;
  for (int64_t i = 0; i < n; ++i) {
    if (!(pts[i].x > lo && pts[i].x < hi && pts[i].y > lo && pts[i].y < hi))
      return fail(MCL_ERR_DEGENERATE_INPUT, "point outside the bounding square");
  }
  std::sort(pts, pts + n, [](const mcl_float2& a, const mcl_float2& b) {
    return mcl_morton_key(a.x, a.y) < mcl_morton_key(b.x, b.y);
  });
  const int64_t V = n + 4, E = 5 + 3 * n;
  mcl_mesh* m = nullptr;
  int rc = alloc_mesh(V, E, &m);
  if (rc != MCL_OK) return rc;
  // bounding square: the reference's seed (include/Host_Triangulation.h:107-137)
  std::vector<mcl_float2> pos(V);
  pos[0] = {lo, lo}; pos[1] = {hi, lo}; pos[2] = {hi, hi}; pos[3] = {lo, hi};
  for (int64_t i = 0; i < n; ++i) pos[4 + i] = pts[i];
  const int seed_he[10][4] = {{2, 0, 0, 2},  {9, 1, -1, -1}, {4, 1, 0, 0},  {1, 2, -1, -1}, {0, 2, 0, 1},
                              {6, 0, 1, 3},  {8, 2, 1, 0},   {3, 3, -1, -1}, {5, 3, 1, 2},  {7, 0, -1, -1}};
  std::vector<int4> ev(E, make_int4(-1, -1, -1, -1)), en(E, make_int4(-1, -1, -1, -1));
  int prev[10];
  for (int h = 0; h < 10; ++h) prev[seed_he[h][0]] = h;
  for (int e = 0; e < 5; ++e) {
    const int* a = seed_he[2 * e];
    const int* b = seed_he[2 * e + 1];
    ev[e] = make_int4(a[1], b[1], a[2] >= 0 ? a[3] : -1, b[2] >= 0 ? b[3] : -1);
    en[e] = make_int4(a[0], prev[2 * e], b[0], prev[2 * e + 1]);
  }
  std::vector<int> vhe(V, -1);
  vhe[0] = 0; vhe[1] = 2; vhe[2] = 6; vhe[3] = 8;
  rc = upload_soa(m, pos.data(), ev, en, vhe);
  if (rc != MCL_OK) { free_mesh(m); return rc; }
  // pending list and free edge slots: vertex 4+i owns edges 5+3i .. 7+3i
  std::vector<int> vfree(3 * V, -1), list(n), hint(V, 0);
  for (int64_t i = 0; i < n; ++i) {
    list[i] = (int)(4 + i);
    for (int k = 0; k < 3; ++k) vfree[3 * (4 + i) + k] = (int)(5 + 3 * i + k);
  }
  cudaError_t e = cudaMemcpy(m->vfree, vfree.data(), 12 * V, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n) e = cudaMemcpy(m->vl[0], list.data(), 4 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->vhint, hint.data(), 4 * V, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { free_mesh(m); return cuda_fail(e, "build upload"); }
  KParams P = make_params(m, ENGINE_BUILD);
  P.pos = m->pos[0];
  P.pos_old = m->pos[0];
  const int n32 = (int)n;
  e = cudaMemcpy(&m->st->vl_count[0], &n32, sizeof(int), cudaMemcpyHostToDevice);
  void* args[] = {&P};
  if (e == cudaSuccess)
    e = cudaLaunchCooperativeKernel((void*)k_build, dim3(m->repair_blocks), dim3(m->coop_threads), args, 0, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(m->st_host, m->st, sizeof(DevState), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(m->pos[1], m->pos[0], 8 * V, cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) { free_mesh(m); return cuda_fail(e, "build"); }
  if (m->st_host->last_status != MCL_OK) {
    const int st = m->st_host->last_status;
    free_mesh(m);
    return fail(st, std::string("build failed: ") + mcl_status_string(st));
  }
  *out = m;
  return MCL_OK;
}

}  // extern "C"
