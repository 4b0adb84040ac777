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
//   step    one cooperative launch (k_pstep): move + wrap every vertex, the
//           wraps folded into the edge words, then rounds of classify +
//           claim / flip winners over edge work-lists until no edge is
//           non-Delaunay, grid barriers between the phases and every
//           decision taken on the device.  A classification that finds faces
//           turned over sends their moved vertices back (then the fold again)
//           and classifies again; flips start from a mesh whose faces are all
//           positive.  Vertices sent back then follow in up to kSubLevels
//           sub-steps (half of what they still owe, the last all); the few
//           still away (listed in parallel, by ascending id) are removed and
//           reinserted at their targets in claim-based rounds (removal
//           rounds, then insertion rounds; periodic.cuh), and flip rounds
//           from the edges those rewrote restore Delaunay.  The host reads
//           one record at the end.
//   queries one-ring with copy offsets, closest neighbour, mesh FRNN (one
//           launch for the outgoing half-edges, one per query).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
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
namespace cg = cooperative_groups;

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
  // the step's cooperative launch (allocated on the first step)
  PCount* slots;     // three rotating phase counters, clear between launches
  void* out;         // PStepOut (device)
  void* out_host;    // PStepOut (pinned, mapped)
  void* out_map;     // out_host's device address (NULL: copied back instead)
  int* chunk;        // per-block counts of the behind list (grid + 1)
  int* par;          // removal and reinsertion rounds: 8 ints per vertex (state 0 between steps)
  int grid;          // blocks of the launch
};

namespace {

constexpr int kThreads = 256;
constexpr int kMaxRounds = 4096;
constexpr int kMaxRevertPasses = 256;
constexpr int kSubLevels = 5;  // sub-steps for vertices sent back
constexpr int kCenter = 4;  // copy index of the untranslated copy

#define PCK(call)                                       \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return mcl::cuda_fail(_e, #call); \
  } while (0)

// ---------------------------------------------------------------------------
// The step as one cooperative launch: phases over vertices or edges
// (grid-stride) separated by grid barriers, every decision taken on the
// device from the counters of the phase just ended.
//
// Counters: each phase counts into its own PCount slot, three in rotation.
// After the barrier that ends phase p every thread reads slot p % 3 (the same
// values in every thread, so all take the same branch and meet at the same
// barriers); phase p + 1 reads at most the list length of slot p; at the start
// of phase p + 2, one thread adds slot p % 3 to the step's totals and clears
// it (no thread reads it after the barrier ending phase p + 1).  The launch
// ends with every slot cleared, so the next launch needs no reset.
struct PStepOut {
  PCount tot;  // counters of the whole step (error and error_site: the first)
  unsigned long long rounds, inverted_first, incircle_tests, behind_first, behind_sub, behind, reinserted, stamps;
  unsigned long long lq;  // entries of the removal and reinsertion rounds' work-list (wl0)
  int reason;  // kReason*
  int phases;  // grid barriers passed
  // %globaltimer at the launch's start (ts[0]) and after the barrier ending
  // each of its first kPhaseMarks - 1 phases (mcl_periodic_debug_timeline)
  unsigned long long ts[32];
};
constexpr int kPhaseMarks = 32;
__device__ __forceinline__ unsigned long long p_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
enum : int {
  kReasonNone = 0,
  kReasonBody,              // a kernel body flagged an error (tot.error)
  kReasonTurnedAfterFlips,  // a face turned over after flips
  kReasonRevertEndless,     // sending vertices back did not end
  kReasonNoConverge,        // flip rounds did not converge
  kReasonReinsert,          // removal and reinsertion failed (tot.error)
};

__device__ void p_fold(PCount* tot, PCount* slot) {
  constexpr int kWords = (int)(sizeof(PCount) / 8), kErr = (int)(offsetof(PCount, error) / 8),
                kSite = (int)(offsetof(PCount, error_site) / 8);
  unsigned long long* t = reinterpret_cast<unsigned long long*>(tot);
  unsigned long long* x = reinterpret_cast<unsigned long long*>(slot);
  const bool first = t[kErr] == 0 && __ldcg(x + kErr) != 0;
  for (int i = 0; i < kWords; ++i) {
    const unsigned long long v = __ldcg(x + i);
    if (i == kErr || i == kSite) {
      if (first) t[i] = v;
    } else {
      t[i] += v;
    }
    x[i] = 0;
  }
}

struct PCtl {
  cg::grid_group g;
  PView V0;
  PCount* slots;
  PCount* tot;
  unsigned long long* ts;
  int ph;
  long long gt, gs;
  // the thread's id dealt across blocks (thread t of block b: t * blocks + b),
  // for short work-lists: their items spread over every SM instead of filling
  // the first blocks
  __device__ long long gl() const { return (long long)threadIdx.x * gridDim.x + blockIdx.x; }
  // start of a phase: its view (counting into its slot); recycles the slot of
  // the phase before the last
  __device__ PView begin() {
    if (gt == 0) p_fold(tot, slots + (ph + 1) % 3);
    PView V = V0;
    V.cnt = slots + ph % 3;
    return V;
  }
  // end of a phase: the grid barrier, then the phase's counters
  __device__ const PCount* end() {
    g.sync();
    if (gt == 0 && ph + 1 < kPhaseMarks) ts[ph + 1] = p_now();
    return slots + (ph++ % 3);
  }
};
__device__ __forceinline__ bool p_failed(const PCount* c) { return __ldcg(&c->error) != 0; }

// Streaming passes, kU items per thread and iteration with every load of an
// iteration issued before its first store (item j of the iteration at base is
// base + j * (threads of the grid), so each load stays coalesced).
constexpr int kU = 4;

// every vertex: the move by d (and first, at the step's start, the target)
__device__ void p_move_pass(const PCtl& C, const PView& V, const PF2* d, bool target) {
  for (long long base = C.gt; base < V.n; base += C.gs * kU) {
    PF2 p[kU], dv[kU];
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      const long long v = base + j * C.gs;
      if (v < V.n) {
        p[j] = V.pos[v];
        dv[j] = d[v];
      }
    }
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      const long long v = base + j * C.gs;
      if (v < V.n) {
        if (target) mcl::p_target_with(V, (int)v, p[j], dv[j]);
        mcl::p_move_with(V, (int)v, p[j], dv[j]);
      }
    }
  }
}

// every vertex: the displacement it still owes (counting those behind)
__device__ void p_resume_pass(const PCtl& C, const PView& V, PF2* dsub, bool last) {
  for (long long base = C.gt; base < V.n; base += C.gs * kU) {
    PF2 p[kU], t[kU];
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      const long long v = base + j * C.gs;
      if (v < V.n) {
        p[j] = V.pos[v];
        t[j] = V.target[v];
      }
    }
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      const long long v = base + j * C.gs;
      if (v < V.n) mcl::p_resume_with(V, dsub, (int)v, p[j], t[j], last);
    }
  }
}

// every edge (cur < 0), each first folding the wraps of its quad's vertices
// into its offset word (the fold of a move or of vertices sent back, which
// always precedes a classification of every edge), or the first `items`
// entries of work-list cur.  The loop decides each edge with the float32
// filters; an edge they leave open, or with a face turned over, is classified
// after the loop with the full predicates (p_body_classify), two per thread,
// any more listed on `hard` (counted in the slot's `hard`) for a second pass
// after the barrier.  So the loop holds no call of the exact predicates.
__device__ void p_classify_pass(const PCtl& C, const PView& V, int cur, long long items, unsigned stamp, int* hard) {
  constexpr int kU = 2;
  const int* wl = cur == 1 ? V.wl1 : V.wl0;
  int def0 = -1, def1 = -1;
  for (long long base = cur < 0 ? C.gt : C.gl(); base < items; base += C.gs * kU) {
    int e[kU];
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      const long long i = base + j * C.gs;
      e[j] = i < items ? (cur < 0 ? (int)i : __ldcg(wl + i)) : -1;
      if ((unsigned)e[j] >= (unsigned)V.E) e[j] = -1;
    }
    PI4 q[kU];
    unsigned o[kU];
#pragma unroll
    for (int j = 0; j < kU; ++j)
      if (e[j] >= 0) {
        q[j] = V.ev[e[j]];
        o[j] = V.eo[e[j]];
      }
    PF2 pa[kU], pb[kU], pc[kU], pd[kU];
    unsigned char w[kU][4];
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      if (e[j] < 0) continue;
      if (!mcl::p_vertices_ok(V, q[j])) {
        mcl::p_error(V, MCL_ERR_DEGENERATE_INPUT, cur < 0 ? 2 : 3);
        e[j] = -1;
        continue;
      }
      if (cur < 0) {
        w[j][0] = V.wv[q[j].x];
        w[j][1] = V.wv[q[j].y];
        w[j][2] = V.wv[q[j].z];
        w[j][3] = V.wv[q[j].w];
      }
      pa[j] = V.pos[q[j].x];
      pb[j] = V.pos[q[j].y];
      pc[j] = V.pos[q[j].z];
      pd[j] = V.pos[q[j].w];
    }
#pragma unroll
    for (int j = 0; j < kU; ++j) {
      if (e[j] < 0) continue;
      if (cur < 0) {
        mcl::p_wrap_with(V, e[j], w[j][0], w[j][1], w[j][2], w[j][3]);
        o[j] = V.eo[e[j]];
      }
      PF2 qb, qc, qd;
      bool open = !mcl::quad_frame(o[j], pb[j], pc[j], pd[j], V.L, qb, qc, qd);
      if (!open) {
        const int sa = mcl::orient2d_fp32(pa[j].x, pa[j].y, qb.x, qb.y, qc.x, qc.y);
        const int sb = mcl::orient2d_fp32(qb.x, qb.y, pa[j].x, pa[j].y, qd.x, qd.y);
        if (sa == 1 && sb == 1) {
          const int si = mcl::incircle_fp32(pa[j].x, pa[j].y, qb.x, qb.y, qc.x, qc.y, qd.x, qd.y);
          if (si == 1) mcl::p_claim_nd(V, e[j], stamp);
          else open = si != -1;
        } else {
          open = true;  // a face turned over (marks its culprit) or undecided
        }
      }
      if (open) {
        if (def0 < 0) def0 = e[j];
        else if (def1 < 0) def1 = e[j];
        else hard[mcl::p_inc(&V.cnt->hard)] = e[j];
      }
    }
  }
  if (def0 >= 0) mcl::p_body_classify(V, def0, stamp);
  if (def1 >= 0) mcl::p_body_classify(V, def1, stamp);
}

// the control state every thread keeps (the same in all of them)
struct PZ {
  unsigned stamp;
  unsigned long long rounds, inverted_first, incircle_tests, reverted;
  bool classified;
};

// Rounds of classification after a move: faces turned over send their moved
// vertices back (then the fold again), otherwise the winners of the
// non-Delaunay edges flip, until no edge is non-Delaunay.
// Starts from every edge (cur0 < 0) or from the first len0 entries of
// work-list cur0.
__device__ int p_settle(PCtl& C, PZ& z, int cur0 = -1, long long len0 = 0) {
  int revert_passes = 0, cur = cur0;  // the work-list to classify (-1: every edge)
  long long len = len0;               // its length
  bool flipped = false;
  for (int r = 0; r < kMaxRounds; ++r) {
    const unsigned stamp = ++z.stamp;
    const long long items = cur < 0 ? (long long)C.V0.E : len;
    const int next = cur == 0 ? 1 : 0;  // the list the round's flips fill, free until then
    int* hard = next ? C.V0.wl1 : C.V0.wl0;
    p_classify_pass(C, C.begin(), cur, items, stamp, hard);
    const PCount* c = C.end();
    const long long nh = (long long)__ldcg(&c->hard);
    if (nh) {
      // the edges the classification left over, into the same counters
      PView V = C.V0;
      V.cnt = const_cast<PCount*>(c);
      for (long long i = C.gl(); i < nh; i += C.gs) mcl::p_body_classify(V, __ldcg(hard + i), stamp);
      C.g.sync();
    }
    ++z.rounds;
    if (p_failed(c)) return kReasonBody;
    const unsigned long long inverted = __ldcg(&c->inverted), nd = __ldcg(&c->nondelaunay);
    if (!z.classified) {
      z.inverted_first = inverted;
      z.classified = true;
    }
    if (inverted) {
      // flips only start from a mesh whose faces are all positive
      if (flipped) return kReasonTurnedAfterFlips;
      if (revert_passes == kMaxRevertPasses) return kReasonRevertEndless;
      {
        const PView V = C.begin();
        for (long long v = C.gt; v < V.n; v += C.gs) mcl::p_body_revert(V, (int)v);
      }
      const PCount* cr = C.end();
      if (p_failed(cr)) return kReasonBody;
      z.reverted += __ldcg(&cr->reverted);
      ++revert_passes;
      cur = -1;
      continue;
    }
    z.incircle_tests += (unsigned long long)items;
    if (!nd) return kReasonNone;
    {
      const PView V = C.begin();  // a fresh slot: work-list `next` starts empty
      for (long long i = C.gl(); i < (long long)nd; i += C.gs) {
        const int e = __ldcg(V.clist + i);
        if ((unsigned)e < (unsigned)V.E) mcl::p_body_flip(V, e, stamp, next);
      }
    }
    c = C.end();
    if (p_failed(c)) return kReasonBody;
    len = (long long)__ldcg(&c->lcount[next]);
    cur = next;
    flipped = true;
  }
  return kReasonNoConverge;
}

__device__ __forceinline__ bool p_behind(const PView& V, int i) {
  const float2 here = __ldcg(reinterpret_cast<const float2*>(V.pos) + i);
  const PF2 t = V.target[i];
  return !(here.x == t.x && here.y == t.y);
}

// The vertices still away from their targets, listed by ascending id (the
// order the reinsertion takes them in) into V.clist, their number into
// chunk[gridDim.x]: each block counts a contiguous range, block 0 scans the
// counts, each block writes its range in order.  Three phases.
__device__ void p_list_behind(PCtl& C, int* chunk) {
  __shared__ int wsum[kThreads / 32];
  __shared__ int run;
  const long long n = C.V0.n, per = (n + gridDim.x - 1) / gridDim.x;
  const long long lo = min(n, (long long)blockIdx.x * per), hi = min(n, lo + per);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  {
    const PView V = C.begin();
    int k = 0;
    for (long long base = lo; base < hi; base += blockDim.x) {
      const long long i = base + threadIdx.x;
      k += __syncthreads_count(i < hi && p_behind(V, (int)i));
    }
    if (threadIdx.x == 0) chunk[blockIdx.x] = k;
  }
  C.end();
  {
    C.begin();
    if (blockIdx.x == 0) {
      // exclusive scan of chunk[0 .. gridDim.x), the total into chunk[gridDim.x]
      __shared__ int tot[kThreads];
      const int nb = gridDim.x, seg = (nb + kThreads - 1) / kThreads;
      const int a = min(nb, (int)threadIdx.x * seg), b = min(nb, a + seg);
      int x = 0;
      for (int i = a; i < b; ++i) x += __ldcg(chunk + i);
      tot[threadIdx.x] = x;
      __syncthreads();
      for (int o = 1; o < kThreads; o <<= 1) {
        const int y = (int)threadIdx.x >= o ? tot[threadIdx.x - o] : 0;
        __syncthreads();
        tot[threadIdx.x] += y;
        __syncthreads();
      }
      int acc = tot[threadIdx.x] - x;
      for (int i = a; i < b; ++i) {
        const int c = __ldcg(chunk + i);
        chunk[i] = acc;
        acc += c;
      }
      if (threadIdx.x == kThreads - 1) chunk[nb] = tot[kThreads - 1];
    }
  }
  C.end();
  {
    const PView V = C.begin();
    if (threadIdx.x == 0) run = __ldcg(chunk + blockIdx.x);
    __syncthreads();
    for (long long base = lo; base < hi; base += blockDim.x) {
      const long long i = base + threadIdx.x;
      const bool b = i < hi && p_behind(V, (int)i);
      const unsigned bal = __ballot_sync(0xffffffffu, b);
      if (lane == 0) wsum[warp] = __popc(bal);
      __syncthreads();
      int before = run, total = 0;
      for (int w = 0; w < kThreads / 32; ++w) {
        if (w == warp) before += total;
        total += wsum[w];
      }
      if (b) V.clist[before + __popc(bal & ((1u << lane) - 1u))] = (int)i;
      __syncthreads();
      if (threadIdx.x == 0) run += total;
      __syncthreads();
    }
  }
  C.end();
}

// out: the step's record in device memory; host_out (may be NULL): a
// host-mapped copy of it written at the end
// The vertices still away after the sub-steps (nl of them listed in V.clist):
// removal rounds, then insertion rounds (periodic.cuh), each round three
// phases (claims; verification, nothing written; winners' rewrites, losers
// listed for the next round), the rewritten edges queued on wl0 (*lq).
__device__ int p_reinsert_rounds_(PCtl& C, PZ& z, int* vhe, int* par, long long nl, unsigned long long* lq,
                                  unsigned long long& reinserted) {
  const int n = C.V0.n;
  int* pf = par;           // 3 n: free edges
  int* pa = par + 3 * n;   // n: a neighbour that stays (walk start)
  int* loc = par + 4 * n;  // n: face located this round (-1 none, -2 the goal is a corner)
  int* ps = par + 5 * n;   // n: state
  int* la = par + 6 * n;   // n, n: vertex lists
  int* lb = par + 7 * n;
  constexpr int kWon = 16;  // state bit: holds its claims this round
  const unsigned sq = ++z.stamp;  // the queue mark of this work-list
  {
    const PView V = C.begin();
    for (long long i = C.gl(); i < nl; i += C.gs) {
      const int v = V.clist[i];
      ps[v] = mcl::kParPending;
      loc[v] = -1;
      la[i] = v;
    }
  }
  if (p_failed(C.end())) return kReasonReinsert;
  long long na = nl;
  // removal rounds; a vertex left over stays where it is
  for (int r = 0; r < mcl::kParRounds && na > 0; ++r) {
    const unsigned s = ++z.stamp;
    {
      const PView V = C.begin();
      for (long long i = C.gl(); i < na; i += C.gs) mcl::p_body_claim_star(V, vhe, la[i], s);
    }
    if (p_failed(C.end())) return kReasonReinsert;
    {
      const PView V = C.begin();
      for (long long i = C.gl(); i < na; i += C.gs)
        if (mcl::p_body_holds_star(V, vhe, la[i], s)) ps[la[i]] = mcl::kParPending | kWon;
    }
    if (p_failed(C.end())) return kReasonReinsert;
    {
      const PView V = C.begin();
      for (long long i = C.gl(); i < na; i += C.gs) {
        const int v = la[i];
        if (ps[v] == (mcl::kParPending | kWon)) mcl::p_body_remove_par(V, vhe, v, pf, pa, ps, lq, sq);
        else lb[mcl::p_inc(&V.cnt->lcount[1])] = v;
      }
    }
    const PCount* c = C.end();
    if (p_failed(c)) return kReasonReinsert;
    na = (long long)__ldcg(&c->lcount[1]);
    int* t = la;
    la = lb;
    lb = t;
  }
  // insertion rounds over the removed vertices
  {
    const PView V = C.begin();
    for (long long i = C.gl(); i < na; i += C.gs) ps[la[i]] = mcl::kParStays;  // removal rounds ran out
    for (long long i = C.gl(); i < nl; i += C.gs) {
      const int v = V.clist[i];
      if (ps[v] == mcl::kParRemoved) lb[mcl::p_inc(&V.cnt->lcount[1])] = v;
    }
  }
  {
    const PCount* c = C.end();
    if (p_failed(c)) return kReasonReinsert;
    na = (long long)__ldcg(&c->lcount[1]);
    int* t = la;
    la = lb;
    lb = t;
  }
  for (int r = 0; na > 0; ++r) {
    if (r == mcl::kParRounds) {
      {
        const PView V = C.begin();
        if (C.gt == 0) mcl::p_error(V, MCL_ERR_NO_CONVERGENCE, 26);  // vertices would stay out of the mesh
      }
      C.end();
      return kReasonReinsert;
    }
    const unsigned s = ++z.stamp;
    {
      const PView V = C.begin();
      for (long long i = C.gl(); i < na; i += C.gs) mcl::p_body_locate_par(V, vhe, la[i], pa, loc, ps, s);
    }
    if (p_failed(C.end())) return kReasonReinsert;
    {
      const PView V = C.begin();
      for (long long i = C.gl(); i < na; i += C.gs) {
        const int v = la[i];
        if (mcl::p_body_holds_face(V, v, loc, ps, s)) ps[v] |= kWon;
      }
    }
    if (p_failed(C.end())) return kReasonReinsert;
    {
      const PView V = C.begin();
      for (long long i = C.gl(); i < na; i += C.gs) {
        const int v = la[i];
        if (ps[v] & kWon) {
          ps[v] &= ~kWon;
          mcl::p_body_split_par(V, vhe, v, pf, loc, ps, lq, sq);
        } else if (loc[v] == -2) {
          // the goal is taken: back where it was, or (already going back) an error
          if (ps[v] == mcl::kParBack) {
            mcl::p_error(V, MCL_ERR_DEGENERATE_INPUT, 20);
          } else {
            ps[v] = mcl::kParBack;
            loc[v] = -1;
            lb[mcl::p_inc(&V.cnt->lcount[1])] = v;
          }
        } else {
          lb[mcl::p_inc(&V.cnt->lcount[1])] = v;
        }
      }
    }
    const PCount* c = C.end();
    if (p_failed(c)) return kReasonReinsert;
    reinserted += __ldcg(&c->reinserted);
    na = (long long)__ldcg(&c->lcount[1]);
    int* t = la;
    la = lb;
    lb = t;
  }
  return kReasonNone;
}
__device__ int p_reinsert_rounds(PCtl& C, PZ& z, int* vhe, int* par, long long nl, unsigned long long* lq,
                                 unsigned long long& reinserted) {
  const int reason = p_reinsert_rounds_(C, z, vhe, par, nl, lq, reinserted);
  {
    // every listed vertex back to state 0 for the next step (V.clist still
    // holds the list: the rounds keep their lists in par)
    const PView V = C.begin();
    int* ps = par + 5 * C.V0.n;
    for (long long i = C.gl(); i < nl; i += C.gs) ps[V.clist[i]] = 0;
  }
  C.end();
  return reason;
}

// par: the removal and reinsertion rounds' per-vertex arrays (8 n ints: free
// edges, walk start, state, location, two vertex lists); state 0 between steps
__global__ void __launch_bounds__(kThreads, 2) k_pstep(PView V0, const PF2* d, PF2* dsub, PCount* slots, PStepOut* out,
                                                       PStepOut* host_out, int* chunk, int* vhe, int* par,
                                                       unsigned stamp0) {
  PCtl C{cg::this_grid(), V0, slots, &out->tot, out->ts, 0, (long long)blockIdx.x * blockDim.x + threadIdx.x,
         (long long)gridDim.x * blockDim.x};
  if (C.gt == 0) {
    out->ts[0] = p_now();
    out->lq = 0;
    unsigned long long* t = reinterpret_cast<unsigned long long*>(&out->tot);
    for (int i = 0; i < (int)(sizeof(PCount) / 8); ++i) t[i] = 0;
  }
  PZ z{stamp0, 0, 0, 0, 0, false};
  int reason = kReasonNone;
  unsigned long long behind_first = 0, behind = 0, behind_sub = 0, reinserted = 0;
  bool first = true;
  // the step's targets, then the move and wrap of every vertex
  p_move_pass(C, C.begin(), d, true);
  if (p_failed(C.end())) reason = kReasonBody;
  if (!reason) reason = p_settle(C, z);
  // sub-steps: vertices sent back move again by half of what they still owe,
  // the last level by all of it (landing exactly on the target)
  for (int level = 1; !reason; ++level) {
    const bool last = level >= kSubLevels;
    if (first && z.reverted == 0) {
      // nothing was sent back: every vertex stands on its target (computed
      // with the move's own arithmetic), so no vertex is behind
      behind = 0;
    } else {
      p_resume_pass(C, C.begin(), dsub, last);
      behind = __ldcg(&C.end()->behind);
    }
    if (first) behind_first = behind;
    first = false;
    if (behind == 0 || level > kSubLevels) break;
    p_move_pass(C, C.begin(), dsub, false);
    if (p_failed(C.end())) reason = kReasonBody;
    if (!reason) reason = p_settle(C, z);
  }
  behind_sub = behind;
  // the rest: removed and reinserted at their targets, one by one
  if (!reason && behind > 0) {
    {
      const PView V = C.begin();
      for (long long v = C.gt; v < V.n; v += C.gs) vhe[v] = -1;  // the largest candidate wins
    }
    C.end();
    {
      const PView V = C.begin();
      for (long long h = C.gt; h < 2 * (long long)V.E; h += C.gs) mcl::p_body_vhe(V, vhe, (int)h);
    }
    if (p_failed(C.end())) reason = kReasonReinsert;
    if (!reason) {
      p_list_behind(C, chunk);
      reason = p_reinsert_rounds(C, z, vhe, par, __ldcg(chunk + gridDim.x), &out->lq, reinserted);
      if (!reason) reason = p_settle(C, z, 0, (long long)__ldcg(&out->lq));
      p_resume_pass(C, C.begin(), dsub, true);  // counts who is still behind
      behind = __ldcg(&C.end()->behind);
    }
  }
  C.g.sync();  // every thread has read the last phase's counters
  if (C.gt == 0) {
    for (int k = 0; k < 3; ++k) p_fold(&out->tot, slots + k);
    out->rounds = z.rounds;
    out->inverted_first = z.inverted_first;
    out->incircle_tests = z.incircle_tests;
    out->behind_first = behind_first;
    out->behind_sub = behind_sub;
    out->behind = behind;
    out->reinserted = reinserted;
    out->stamps = z.stamp - stamp0;
    out->reason = reason;
    out->phases = C.ph;
    if (host_out) *host_out = *out;
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
  cudaFree(m->slots);
  cudaFree(m->out);
  cudaFree(m->chunk);
  cudaFree(m->par);
  if (m->out_host) cudaFreeHost(m->out_host);
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

// the step's launch state, allocated on the first step: the grid is as many
// blocks as fit on the device at once (a cooperative launch), at most one per
// kThreads edges
int ensure_step(mcl_periodic* m) {
  if (m->slots) return MCL_OK;
  int dev = 0, sms = 0, per_sm = 0;
  PCK(cudaGetDevice(&dev));
  PCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pstep, kThreads, 0));
  if (per_sm < 1) return mcl::fail(MCL_ERR_CUDA, "mcl_periodic_step: the step kernel does not fit on an SM");
  const int64_t want = std::max<int64_t>(1, (m->E + kThreads - 1) / kThreads);
  const int grid = (int)std::min<int64_t>((int64_t)per_sm * sms, want);
  PCK(cudaMalloc((void**)&m->slots, 3 * sizeof(PCount)));
  PCK(cudaMemset(m->slots, 0, 3 * sizeof(PCount)));
  PCK(cudaMalloc(&m->out, sizeof(PStepOut)));
  PCK(cudaHostAlloc(&m->out_host, sizeof(PStepOut), cudaHostAllocMapped));
  if (cudaHostGetDevicePointer(&m->out_map, m->out_host, 0) != cudaSuccess) {
    cudaGetLastError();
    m->out_map = nullptr;
  }
  PCK(cudaMalloc((void**)&m->chunk, sizeof(int) * (size_t)(grid + 1)));
  PCK(cudaMalloc((void**)&m->par, 8 * sizeof(int) * (size_t)m->n));
  PCK(cudaMemset(m->par, 0, 8 * sizeof(int) * (size_t)m->n));
  m->grid = grid;
  return MCL_OK;
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
  const int rc0 = ensure_step(m);
  if (rc0 != MCL_OK) return rc0;
  // a step uses at most (1 + kSubLevels) * kMaxRounds round stamps (+1 for
  // the queue marks of the last): forget every old claim and queue mark
  // before the stamps could wrap
  static_assert((1 + kSubLevels) * kMaxRounds + 2 < (1 << 16), "stamp budget");
  if (m->stamp > 0xFFFFFFFFu - (1u << 16)) {
    PCK(cudaMemsetAsync(m->claim, 0, 16 * (size_t)m->E, s));
    PCK(cudaMemsetAsync(m->cand, 0, 4 * (size_t)m->E, s));
    PCK(cudaMemsetAsync(m->qstamp, 0, 4 * (size_t)m->E, s));
    m->stamp = 0;
  }
  PView V = view(m);
  const PF2* d = reinterpret_cast<const PF2*>(d_dev);
  PStepOut* out = static_cast<PStepOut*>(m->out);
  unsigned stamp0 = m->stamp;
  PStepOut* host_out = static_cast<PStepOut*>(m->out_map);
  void* args[] = {&V, (void*)&d, &m->dsub, &m->slots, &out, &host_out, &m->chunk, &m->vhe, &m->par, &stamp0};
  PCK(cudaLaunchCooperativeKernel((const void*)k_pstep, dim3((unsigned)m->grid), dim3(kThreads), args, 0, s));
  if (!host_out) PCK(cudaMemcpyAsync(m->out_host, m->out, sizeof(PStepOut), cudaMemcpyDeviceToHost, s));
  PCK(cudaStreamSynchronize(s));
  const PStepOut& o = *static_cast<const PStepOut*>(m->out_host);
  const PCount& c = o.tot;
  m->stamp += (unsigned)o.stamps;
  int rc = MCL_OK;
  std::string msg;
  const std::string site = " (site " + std::to_string(c.error_site) + ")";
  switch (o.reason) {
    case kReasonNone:
      break;
    case kReasonBody:
      rc = c.error ? (int)c.error : MCL_ERR_CUDA;
      msg = "mcl_periodic_step: " + std::string(mcl_status_string(rc)) + site;
      break;
    case kReasonTurnedAfterFlips:
      rc = MCL_ERR_DEGENERATE_INPUT;
      msg = "mcl_periodic_step: a face turned over after flips (the mesh was not valid)";
      break;
    case kReasonRevertEndless:
      rc = MCL_ERR_NO_CONVERGENCE;
      msg = "mcl_periodic_step: sending vertices back did not end";
      break;
    case kReasonNoConverge:
      rc = MCL_ERR_NO_CONVERGENCE;
      msg = "mcl_periodic_step: flip rounds did not converge";
      break;
    default:
      rc = c.error ? (int)c.error : MCL_ERR_CUDA;
      msg = "mcl_periodic_step: removal and reinsertion failed" + site;
      break;
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->inverted_faces = (int64_t)((o.inverted_first + 2) / 3);  // each face is seen from its three edges
    stats->reverted_vertices = (int64_t)o.behind;
    stats->removed_vertices = (int64_t)o.reinserted;
    stats->substep_vertices = o.behind_first > o.behind_sub ? (int64_t)(o.behind_first - o.behind_sub) : 0;
    stats->lawson_flips = (int64_t)c.flips;
    stats->lawson_rounds = (int64_t)o.rounds;
    stats->incircle_tests = (int64_t)o.incircle_tests;
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
    msg = "mcl_periodic_step: exact predicate capacity exceeded";
  }
  return rc == MCL_OK ? MCL_OK : mcl::fail(rc, msg);
}

int mcl_periodic_step_host(mcl_periodic* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats,
                           int64_t* wrapped) {
  if (!m || !d_host) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  PCK(cudaMemcpyAsync(m->dstage, d_host, 8 * (size_t)m->n, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return mcl_periodic_step(m, reinterpret_cast<const mcl_float2*>(m->dstage), stream, stats, wrapped);
}

int mcl_periodic_debug_timeline(const mcl_periodic* m, int64_t* out32, int64_t* phases) {
  if (!m || !out32) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (!m->out_host) return mcl::fail(MCL_ERR_INVALID_ARGUMENT, "mcl_periodic_debug_timeline: no step yet");
  const PStepOut& o = *static_cast<const PStepOut*>(m->out_host);
  for (int i = 0; i < kPhaseMarks; ++i) out32[i] = i < o.phases + 1 ? (int64_t)(o.ts[i] - o.ts[0]) : -1;
  if (phases) *phases = o.phases;
  return MCL_OK;
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
