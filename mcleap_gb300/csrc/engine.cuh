// Internal declarations of the GB300 kinetic Delaunay engine.
//
// Device mesh layout (structure of arrays, one record per undirected edge e;
// half-edge ids are 2e and 2e+1 and the twin of half-edge h is h^1, the same
// numbering as the reference's AoS half-edges, include/Common_Triangulation.h:47-53):
//
//   ev[e] : int4 {origin(2e), origin(2e+1), apex(2e), apex(2e+1)}
//           apex(h) = vertex opposite h in the face left of h, -1 = outside
//   en[e] : int4 {next(2e), prev(2e), next(2e+1), prev(2e+1)}
//   vhe[v]: one outgoing half-edge of v (-1 while v is detached)
//   pos   : float2[V], double-buffered (old / new positions of a step)
//
// One edge's quad (a, b, c, d) sits in a single 16-byte load, which is all the
// Delaunay and orientation classification reads besides four positions.  Flips,
// splits and vertex removal rewrite whole records of their own edges and only
// the one-side fields {apex, next, prev} of neighbouring edges, so concurrent
// operations on faces they own never write the same word.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "predicates.cuh"
#include "../../include/mcl_gb300.h"

// Message returned by mcl_last_error() on this host thread.
void mcl_set_last_error(const std::string& msg);

namespace mcl {

// Device-side counters (indices into DevState::c).
enum Counter {
  C_LAWSON_FLIPS = 0,
  C_LAWSON_ROUNDS,
  C_INVERTED,
  C_REVERTED,
  C_REMOVED,
  C_REMOVAL_FLIPS,
  C_INSERT_ROUNDS,
  C_INCIRCLE,
  C_INCIRCLE_FP64,
  C_INCIRCLE_EXACT,
  C_ORIENT_FP64,
  C_ORIENT_EXACT,
  C_SOS,
  C_OVERFLOW,
  C_FIX_PASSES,
  C_REMOVE_ROUNDS,
  C_SUBSTEPS,       // sub-step rounds of the repair
  C_SUBSTEP_DONE,   // sent-back vertices brought to their targets by sub-steps
  C_COUNT
};

constexpr int kTimeline = 48;

struct DevState {
  // working state of the running launch; the launch leaves it cleared
  int wl_count[2];         // edge work-list sizes
  int vl_count[2];         // vertex work-list sizes
  int status;              // MCL_OK or the first error
  int site;                // source line that set `status` (diagnostics)
  int inverted;            // faces with orientation <= 0 found by the last classification
  int hard_count;          // edges the FP32 filters could not classify
  int fix_new[3];          // vertices newly reverted per fixpoint pass (triple-buffered)
  int fix_bad[3];          // non-positive faces seen per fixpoint pass
  int fix_list[3];         // vertices listed for the next fixpoint pass (triple-buffered counts)
  int fix_all;             // vertices sent back by this launch (listed once, on `hard`)
  int mark_ovf;            // the repair's appended marks did not fit, or were not all appended
  int movers_now;          // vertices this launch's move pass moved
  int movers_last;         // ... the last launch's (whether this move pass lists them)
  int sub_count[3];        // repair sub-steps: mover lists (2), vertices left for removal
  int sub_rev[3];          // movers sent back per sub-step pass (triple-buffered)
  unsigned int epoch;      // next unused stamp
  unsigned int tail_stamp; // stamp after a single-block flip tail
  unsigned int arrived;    // blocks of k_step that have finished (the last one publishes)
  unsigned int stamp_max;  // largest next-free stamp over those blocks
  unsigned long long c[C_COUNT];
  // published by the last launch
  int last_status;
  int last_site;
  unsigned long long last[C_COUNT];
  unsigned long long tot[C_COUNT];  // running totals over all launches
  unsigned long long calls;
  unsigned long long failed;       // launches that ended with an error
  int dbg[68];             // first failing vertex star: v, deg, then neighbour ids
  unsigned long long ts[kTimeline];  // %globaltimer at phase boundaries of the last launch
  // insertion round r < 16: [4r] located, [4r+1] won, [4r+2] split, [4r+3] flips done
  unsigned long long ts_insert[64];
  // removal round r < 16: [4r] claimed, [4r+1] winners known, [4r+2] removed;
  // [48 + p]: end of send-back pass p < 16
  unsigned long long ts_remove[64];
  // removal round r < 16: the slowest removal ((SM cycles << 16) | spokes)
  // and how many removals walked their star again (not cached); cleared by
  // mcl_debug_remove_timeline
  unsigned long long rm_slow[16];
  unsigned long long rm_uncached[16];
  // latest block at the move / classification marks of the running launch;
  // published to ts[43..46] by a step without repair (a repair step keeps its
  // own marks there)
  unsigned long long tsmax[4];
  // mcl_settle_moves: [0] last stamp used, [1..3] moves sent back per pass
  // (triple-buffered), [4] sent back by the last call, [5] status of the last call
  unsigned int settle[8];
};

enum MoveMode { MOVE_NONE = 0, MOVE_DISPLACE = 1, MOVE_INTEGRATE = 2 };
enum EngineMode { ENGINE_STEP = 0, ENGINE_BUILD = 1 };

struct KParams {
  int V, E;
  float2* pos;             // positions the mesh is repaired to (new)
  const float2* pos_old;   // positions at which the mesh was last valid
  int4* ev;
  int4* en;
  int* vhe;
  const unsigned char* vfix;  // 1 = fixed vertex (bounding corners)
  unsigned int* cand;      // per edge: stamp of the round in which it is a flip candidate
  unsigned int* win;       // per edge: stamp of the round in which it won
  unsigned int* qmark;     // per edge: stamp of the last work-list it was queued on
  int2* efa;               // per edge: the two faces it claimed in the current round
  int* hard;               // edges left to the full predicate ladder by the classification
  int* wl0;
  int* wl1;
  int* vl0;
  int* vl1;
  int* vmark;              // per vertex: stamp of the launch that reverted it
  unsigned long long* claim;  // per half-edge: face claims {stamp, ~priority}
  int* vfree;              // 3 per vertex: free edge slots for (re)insertion
  int* vhint;              // per vertex: half-edge to start point location from
  int* vaux;               // per vertex: a neighbour at removal time
  int* vloc;               // per vertex: located half-edge (+ on-edge flag in vlocf)
  int* vlocf;
  float2* target;          // per vertex: position to reinsert at
  float2* vprev;           // per vertex: position before the current repair sub-step
  int* vl2;                // 4 x V: repair sub-step lists (movers x2, sent back, left for removal);
                           // vprev and vl2 exist only after mcl_mesh_set_substeps(m, n > 0)
  DevState* st;
  // move inputs
  const float2* disp;
  const float* dt;
  const float2* vel;
  int move_mode;
  int mode;
  int max_rounds;
  int walk_cap;
  int tail_items;          // flip rounds with at most this many queued edges run in one block
  int rm_tile;             // lanes of a warp that take removal-list entries (0: as few as fit one pass)
  int substeps;            // repair sub-steps before removal
  int sparse_ok;           // the mesh is Delaunay at pos_old: a step may classify only its movers' stars
  int append_marks;        // repair: append marked edges to work-list 0 (few removals), else rebuild from the marks
  mcl_step_stats* stats_out;  // device-visible host record the launch fills at its end (or NULL)
  const int* vroot;        // per vertex: a never-freed half-edge of its mesh (batches); NULL = half-edge 0
  // active meshes of a batch (nact == 0: every edge and vertex): the full
  // passes run over index spaces [0, E_it) and [0, V_it) that map to the
  // edges and vertices of the active meshes
  int nact;
  int E_it, V_it;
  const int* act_epre;     // [nact + 1] prefix sums of the active meshes' edge counts
  const int* act_e0;       // [nact] first edge of each active mesh
  const int* act_vpre;     // [nact + 1]
  const int* act_v0;       // [nact]
};

__device__ __forceinline__ int act_map(const int* pre, const int* base, int n, int i) {
  int lo = 0, hi = n - 1;  // largest c with pre[c] <= i
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= i) lo = mid;
    else hi = mid - 1;
  }
  return __ldg(base + lo) + (i - __ldg(pre + lo));
}
// Index space of a pass over the active meshes' vertices (all when n == 0).
struct ActV {
  int n, V_it;
  const int* pre;
  const int* v0;
  __device__ __forceinline__ int at(int i) const { return n ? act_map(pre, v0, n, i) : i; }
};

__device__ __forceinline__ int edge_at(const KParams& P, int i) {
  return P.nact ? act_map(P.act_epre, P.act_e0, P.nact, i) : i;
}
__device__ __forceinline__ int vert_at(const KParams& P, int i) {
  return P.nact ? act_map(P.act_vpre, P.act_v0, P.nact, i) : i;
}

// ---------------------------------------------------------------------------
// Accessors.  Mesh records are mutated by other blocks inside the persistent
// kernels, so they are read with L2-coherent loads (ld.global.cg).
__device__ __forceinline__ int4 ld_ev(const KParams& P, int e) { return __ldcg(P.ev + e); }
__device__ __forceinline__ int4 ld_en(const KParams& P, int e) { return __ldcg(P.en + e); }
__device__ __forceinline__ int ld_i(const int* p) { return __ldcg(p); }

__device__ __forceinline__ int he_origin(const KParams& P, int h) {
  return ld_i(reinterpret_cast<const int*>(P.ev) + 4 * (h >> 1) + (h & 1));
}
__device__ __forceinline__ int he_apex(const KParams& P, int h) {
  return ld_i(reinterpret_cast<const int*>(P.ev) + 4 * (h >> 1) + 2 + (h & 1));
}
__device__ __forceinline__ int he_next(const KParams& P, int h) {
  return ld_i(reinterpret_cast<const int*>(P.en) + 4 * (h >> 1) + 2 * (h & 1));
}
__device__ __forceinline__ int he_prev(const KParams& P, int h) {
  return ld_i(reinterpret_cast<const int*>(P.en) + 4 * (h >> 1) + 2 * (h & 1) + 1);
}
// Rewrite the face-side fields of half-edge h (its origin is unchanged).
__device__ __forceinline__ void he_set_face(const KParams& P, int h, int apex, int next, int prev) {
  int* ev = reinterpret_cast<int*>(P.ev) + 4 * (h >> 1);
  int* en = reinterpret_cast<int*>(P.en) + 4 * (h >> 1);
  __stcg(ev + 2 + (h & 1), apex);
  __stcg(en + 2 * (h & 1), next);
  __stcg(en + 2 * (h & 1) + 1, prev);
}
__device__ __forceinline__ void he_set_origin(const KParams& P, int h, int v) {
  __stcg(reinterpret_cast<int*>(P.ev) + 4 * (h >> 1) + (h & 1), v);
}

__device__ __forceinline__ int face_min(const KParams& P, int h) {
  const int n = he_next(P, h), p = he_prev(P, h);
  return min(h, min(n, p));
}

// 32-bit bijective mixer (murmur3 finaliser); distinct inputs give distinct
// priorities, so flip / claim conflicts never tie.
__device__ __forceinline__ unsigned int mix32(unsigned int x) {
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}

struct LocalCounters {  // per-thread, folded into DevState at the end of a launch
  unsigned orient_fp64, orient_exact, incircle_fp64, incircle_exact, sos;
  unsigned incircle;
  int overflow;
};

__device__ __forceinline__ float2 ldpos(const KParams& P, int v) { return __ldcg(P.pos + v); }
// Positions that stay fixed for the rest of the launch and were not read by
// this SM before they were written may go through L1 (k_step after its move
// pass); positions that change during the launch (k_repair) must not.
template <bool kFixedPos>
__device__ __forceinline__ float2 ldpos_t(const KParams& P, int v) {
  return kFixedPos ? __ldca(P.pos + v) : __ldcg(P.pos + v);
}

__device__ __forceinline__ int orient_v(const KParams& P, float2 a, float2 b, float2 c, LocalCounters& lc) {
  return orient2d(a.x, a.y, b.x, b.y, c.x, c.y, &lc, &lc.overflow);
}

__device__ __forceinline__ bool bad_v(const KParams& P, int v) { return (unsigned)v >= (unsigned)P.V; }
__device__ __forceinline__ bool bad_h(const KParams& P, int h) { return (unsigned)h >= (unsigned)(2 * P.E); }
__device__ __forceinline__ void flag_error_at(const KParams& P, int code, int line) {
  if (atomicCAS(&P.st->status, 0, code) == 0) P.st->site = line;
}
#define flag_error(P, code) flag_error_at(P, code, __LINE__)

// Is edge e locally non-Delaunay (d inside the circle of the left face a,b,c)?
template <bool kFixedPos = false>
__device__ __forceinline__ bool edge_illegal(const KParams& P, const int4 q, LocalCounters& lc) {
  if (q.x < 0 || q.z < 0 || q.w < 0) return false;
  if (bad_v(P, q.x) || bad_v(P, q.y) || bad_v(P, q.z) || bad_v(P, q.w)) {
    flag_error(P, MCL_ERR_DEGENERATE_INPUT);
    return false;
  }
  const float2 a = ldpos_t<kFixedPos>(P, q.x), b = ldpos_t<kFixedPos>(P, q.y), c = ldpos_t<kFixedPos>(P, q.z),
               d = ldpos_t<kFixedPos>(P, q.w);
  lc.incircle++;
  return incircle_sos(a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, q.x, q.y, q.z, q.w, &lc, &lc.overflow) > 0;
}

// Edge flip of e = (a,b,c,d): the diagonal a-b becomes d-c.  Faces after the
// flip: (d,c,a) left of 2e and (c,d,b) left of 2e+1.  Only e's own records and
// the facing-side fields of its four wing half-edges are written.
// flip_edge with e's records (q = ev[e], w = en[e]) and the one-ring anchors
// of its endpoints (vha = vhe[a], vhb = vhe[b]) already loaded: valid when no
// other thread writes them meanwhile, as for a flip-round winner.
__device__ __forceinline__ bool flip_edge_with(const KParams& P, int e, int4 q, int4 w, int vha, int vhb) {
  const int a = q.x, b = q.y, c = q.z, d = q.w;
  const int n0 = w.x, p0 = w.y, n1 = w.z, p1 = w.w;
  if (bad_v(P, a) || bad_v(P, b) || bad_v(P, c) || bad_v(P, d) || bad_h(P, n0) || bad_h(P, p0) ||
      bad_h(P, n1) || bad_h(P, p1)) {
    flag_error(P, MCL_ERR_DEGENERATE_INPUT);
    return false;
  }
  const int h0 = 2 * e, h1 = 2 * e + 1;
  __stcg(P.ev + e, make_int4(d, c, a, b));
  __stcg(P.en + e, make_int4(p0, n1, p1, n0));
  he_set_face(P, p0, d, n1, h0);
  he_set_face(P, n1, c, h0, p0);
  he_set_face(P, p1, c, n0, h1);
  he_set_face(P, n0, d, h1, p1);
  if (vha == h0) __stcg(P.vhe + a, n1);
  if (vhb == h1) __stcg(P.vhe + b, n0);
  return true;
}

__device__ __forceinline__ bool flip_edge(const KParams& P, int e) {
  const int4 q = ld_ev(P, e);
  const int4 w = ld_en(P, e);
  const int a = q.x, b = q.y, c = q.z, d = q.w;
  const int n0 = w.x, p0 = w.y, n1 = w.z, p1 = w.w;
  if (bad_v(P, a) || bad_v(P, b) || bad_v(P, c) || bad_v(P, d) || bad_h(P, n0) || bad_h(P, p0) ||
      bad_h(P, n1) || bad_h(P, p1)) {
    flag_error(P, MCL_ERR_DEGENERATE_INPUT);
    return false;
  }
  const int h0 = 2 * e, h1 = 2 * e + 1;
  __stcg(P.ev + e, make_int4(d, c, a, b));
  __stcg(P.en + e, make_int4(p0, n1, p1, n0));
  he_set_face(P, p0, d, n1, h0);
  he_set_face(P, n1, c, h0, p0);
  he_set_face(P, p1, c, n0, h1);
  he_set_face(P, n0, d, h1, p1);
  if (ld_i(P.vhe + a) == h0) __stcg(P.vhe + a, n1);
  if (ld_i(P.vhe + b) == h1) __stcg(P.vhe + b, n0);
  return true;
}

}  // namespace mcl

struct mcl_mesh {
  int device;
  int64_t V, E, T;
  int cur;                 // index of the current position buffer
  bool valid_cur;          // pos[cur] is the last validated state
  float2* pos[2];
  int4* ev;
  int4* en;
  int* vhe;
  unsigned char* vfix;
  unsigned int* cand;
  unsigned int* win;
  unsigned int* qmark;
  int2* efa;
  int* hard;
  int* wl[2];
  int* vl[2];
  int* vmark;
  unsigned long long* claim;
  int* vfree;
  int* vhint;
  int* vaux;
  int* vloc;
  int* vlocf;
  float2* target;
  float2* vprev;
  int* vl2;
  float2* dstage;          // device staging buffer for host displacements
  // mcl_step_host_async: a second staging buffer, a copy stream, and events
  float2* dstage2;
  cudaStream_t copy_stream;
  cudaEvent_t ev_copied[2], ev_used[2];
  mcl_step_stats* stats_dev;  // [2] published counters of the pipelined steps
  int stage_idx;
  unsigned long long* scratch;  // small device scratch for query counters
  mcl::DevState* st;
  mcl::DevState* st_host;  // pinned mirror
  int coop_blocks;         // k_step grid
  int repair_blocks;       // k_repair grid
  int coop_threads;
  int last_status;
  // tuning (mcl_mesh_set_tuning)
  int nsm;                 // SMs of the device
  int max_blocks_per_sm;   // k_step occupancy limit
  int tail_items;          // single-block flip-round threshold
  int rm_tile;             // removal tile (mcl_mesh_set_removal_tile; 0 = automatic)
  int substeps;            // repair sub-steps before removal (mcl_mesh_set_substeps)
  bool delaunay;           // the last launch left the mesh Delaunay (set when a step or build is launched)
  // batches: a mesh made of independent components (mcl_batch_create)
  int64_t ncomp;           // 1 for a plain mesh
  int64_t* comp_host;      // [4 * ncomp]: first vertex, vertices, first edge, edges
  int* vcomp;              // per vertex: component (NULL for a plain mesh)
  int* vroot;              // per vertex: half-edge 0 of its component (NULL for a plain mesh)
  int* cbase;              // per component: first vertex (NULL for a plain mesh)
  // mcl_settle_moves
  unsigned long long* table;  // hash table of positions, stamped entries
  int64_t table_size;
  int* smark;              // per vertex: stamp of the settle pass that found it coincident
  unsigned* smove;         // per mesh: stamp of the settle call that found a mover in it
  int settle_blocks;       // k_settle grid (cooperative)
  unsigned char* fnew;     // per vertex: newly frozen flags of mcl_dla_freeze
  // mcl_batch_frnn_grid: one uniform grid per mesh, cells of all meshes in one table
  int* bg_cell;            // per vertex: its cell (-1: bounding corner)
  int* bg_src;             // per sorted slot: vertex
  int* bg_perm;            // per vertex: sorted slot
  float2* bg_pos;          // per sorted slot: position
  int* bg_count;           // per cell
  int* bg_start;
  int* bg_cursor;
  int* bg_tmp;             // scan scratch
  int4* bg_par;            // per mesh: {cell size bits, cells per side, first cell, 0}
  int4* bg_par_host;       // pinned copy of the uploaded grid parameters
  int64_t bg_cap;          // cells the tables hold
  int64_t bg_cells;        // cells of the uploaded parameters (0: none yet)
  // active meshes (mcl_batch_set_active)
  int nact;                // 0 = all
  int act_E, act_V;
  int* act_dev;            // device: epre[ncomp+1], e0[ncomp], vpre[ncomp+1], v0[ncomp], ids[ncomp]
  int* act_host;           // pinned staging of the same
  int* act_list;           // host: the active mesh ids
  unsigned char* dirty;    // host, per mesh: its two position buffers differ
  // mcl_mesh_export_aos: per half-edge face-owner flags and their prefix sums
  int* aos_tmp;
  int64_t aos_cap;         // ints aos_tmp holds
};

// Host-side helpers shared by the translation units of the library.
namespace mcl {
int alloc_mesh(int64_t V, int64_t E, mcl_mesh** out);
void free_mesh(mcl_mesh* m);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
int download_range(mcl_mesh* m, int64_t vb, int64_t nv, int64_t eb, int64_t ne, int64_t T, mcl_float2* pos,
                   int32_t* v, int32_t* he, int32_t* t);
const float2* valid_positions(const mcl_mesh* m);
ActV act_of(const mcl_mesh* m);
}  // namespace mcl
