/*
 * mcl_gb300.h - C ABI of the GB300 kinetic 2D Delaunay engine (libmcl_gb300.so).
 *
 * Plain C: opaque handles, POD structs, pointers and sizes, int status codes.
 * CUDA streams are passed as `void*` (a cudaStream_t; NULL = the legacy
 * default stream) so this header needs no CUDA include.
 *
 * The reference (hporro/mcleap) has no FFI: its call surface is the header-only
 * C++ structs HostTriangulation, DeviceTriangulation and GridCount2d.  Each entry
 * point below names the reference member it replaces (file:line in the
 * reference); the C++ drop-in headers in include/mcleap/ keep those class and
 * method names and forward to these functions.
 *
 * Mesh interchange format (the reference's AoS layout,
 * include/Common_Triangulation.h:42-57): positions float2[V]; vertices
 * int2[V] = {pos_index, he}; half-edges int4[HE] = {next, v, t, op} with the
 * twin of half-edge i at i^1; triangles int[T] = {he}.  Vertex ids 0..3 are the
 * corners of the +-1e7 bounding square and never move.
 *
 * Device pointers: arguments named *_dev are device memory, *_host host memory.
 */
#ifndef MCL_GB300_H
#define MCL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  MCL_OK = 0,
  MCL_ERR_INVALID_ARGUMENT = 1,
  MCL_ERR_CUDA = 2,               /* a CUDA runtime call failed */
  MCL_ERR_OUT_OF_MEMORY = 3,
  MCL_ERR_NO_CONVERGENCE = 4,     /* an iteration cap was reached (flip rounds, walks) */
  MCL_ERR_CAPACITY = 5,           /* an output or work buffer was too small */
  MCL_ERR_DEGENERATE_INPUT = 6,   /* duplicate point, point outside or on the bounding square,
                                     or a mesh that was not valid before the step */
  MCL_ERR_PREDICATE = 7,          /* exact predicate expansion capacity exceeded */
  MCL_ERR_NO_DEVICE = 8           /* no usable CUDA device */
};

/* Layouts of fixed-capacity neighbour tables (include/Device_Triangulation.h:196-218):
 * COLUMN: out[i] = count, out[(k+1)*n + i] = k-th neighbour of i
 * ROW:    out[i*M] = count, out[i*M + k + 1] = k-th neighbour of i              */
enum { MCL_LAYOUT_COLUMN = 0, MCL_LAYOUT_ROW = 1 };

typedef struct { float x, y; } mcl_float2;

typedef struct {
  const mcl_float2* pos; /* [V] */
  const int32_t* v;      /* [2*V] {pos_index, he} */
  const int32_t* he;     /* [4*HE] {next, v, t, op} */
  const int32_t* t;      /* [T] {he} */
  int64_t V, HE, T;
} mcl_aos_view;

/* Counters of one call (zeroed at the start of each call that fills them). */
typedef struct {
  int64_t inverted_faces;        /* faces with orientation <= 0 after the move */
  int64_t reverted_vertices;     /* vertices moved back while untangling */
  int64_t removed_vertices;      /* vertices removed and reinserted */
  int64_t lawson_flips;          /* Delaunay edge flips */
  int64_t lawson_rounds;         /* parallel flip rounds */
  int64_t removal_flips;         /* flips made while removing vertices */
  int64_t insert_rounds;         /* parallel insertion rounds */
  int64_t incircle_tests;        /* incircle evaluations */
  int64_t incircle_fp64;         /* ... that the FP32 filter could not decide */
  int64_t incircle_exact;        /* ... that the FP64 filter could not decide */
  int64_t orient_fp64;           /* orientation tests past the FP32 filter */
  int64_t orient_exact;          /* ... past the FP64 filter */
  int64_t sos_decisions;         /* exactly cocircular quads decided by perturbation */
  int64_t status;                /* MCL_OK or an error code */
  int64_t error_site;            /* engine source location that reported `status` */
  int64_t failed_launches;       /* launches that ended with an error (totals: since creation) */
  int64_t substep_vertices;      /* sent-back vertices brought to their targets by repair sub-steps
                                    (without removal) */
} mcl_step_stats;

/* ---- library ------------------------------------------------------------ */
const char* mcl_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char* mcl_last_error(void);
int mcl_version(void);

/* ---- meshes --------------------------------------------------------------- */
typedef struct mcl_mesh mcl_mesh;

/* DeviceTriangulation(HostTriangulation*) = allocateMemory + transferToDevice
 * (include/Device_Triangulation.h:232-236, :255-285). */
int mcl_mesh_create_from_aos(const mcl_aos_view* aos_host, mcl_mesh** out);

/* HostTriangulation::addDelaunayPoints (include/Host_Triangulation.h:287-300):
 * sorts pts_host IN PLACE into the reference's Morton order (vertex id =
 * 4 + sorted index) and builds the Delaunay triangulation of the bounding
 * square plus the points on the GPU. */
int mcl_mesh_build(mcl_float2* pts_host, int64_t n, mcl_mesh** out);

/* ~DeviceTriangulation / freeMemory (include/Device_Triangulation.h:238-241, :287-306). */
int mcl_mesh_destroy(mcl_mesh* m);

/* m_pos_size, m_v_size, m_he_size, m_t_size (include/Device_Triangulation.h:134-137). */
int mcl_mesh_sizes(const mcl_mesh* m, int64_t* V, int64_t* HE, int64_t* T);

/* transferToHost (include/Device_Triangulation.h:245-253): any pointer may be NULL.
 * Triangle ids are assigned canonically (by the smallest half-edge of each face). */
int mcl_mesh_download_aos(mcl_mesh* m, mcl_float2* pos_host, int32_t* v_host, int32_t* he_host,
                          int32_t* t_host);

/* transferToDevice (include/Device_Triangulation.h:255-263) with new host arrays of
 * the same sizes. */
int mcl_mesh_upload_aos(mcl_mesh* m, const mcl_aos_view* aos_host);
/* DeviceTriangulation's public device arrays m_v / m_he / m_t
 * (include/Device_Triangulation.h:139-142): the reference's AoS records
 * (Vertex {id, he}, HalfEdge {next, v, t, op}, Triangle {he}) written into
 * caller-owned device buffers of V, 2E and T records, with the face numbering
 * of mcl_mesh_download_aos.  Any pointer may be NULL.  Asynchronous on
 * `stream`; the first call allocates the conversion scratch. */
int mcl_mesh_export_aos(mcl_mesh* m, int32_t* v_dev, int32_t* he_dev, int32_t* t_dev, void* stream);

/* m_pos: the device position array (float2[V]).  The pointer changes after every
 * call that moves points (positions are double-buffered); fetch it again. */
int mcl_mesh_positions(mcl_mesh* m, mcl_float2** pos_dev);

/* Copy the current positions (float2[V]) to device (to_host = 0) or host memory
 * (to_host = 1, synchronous); the experiments copy dt.m_pos this way
 * (experiments/moving_device_mesh.cu:106, :125). */
int mcl_mesh_copy_positions(mcl_mesh* m, mcl_float2* dst, int to_host, void* stream);

/* movePoints (include/Device_Triangulation.h:395-402): pos[i] += d[i] for i >= 4. */
int mcl_move(mcl_mesh* m, const mcl_float2* d_dev, void* stream);
/* integrateMovePoints (include/Device_Triangulation.h:403-410): pos[i] += v[i]*dt[i], i >= 4. */
int mcl_integrate(mcl_mesh* m, const float* dt_dev, const mcl_float2* v_dev, void* stream);

/* untangle / untangle2 (include/Device_Triangulation.h:422-495).  Unlike the
 * reference (which only handles its B and C cases), this always returns a valid
 * triangulation: vertices of inverted faces are moved back, removed and
 * reinserted at their new positions, and the result is Delaunay. */
int mcl_untangle(mcl_mesh* m, void* stream, mcl_step_stats* stats_host);

/* delonize / delonize2 (include/Device_Triangulation.h:324-390): Lawson flips to the
 * Delaunay triangulation (untangling first if any face is inverted). */
int mcl_delaunay_restore(mcl_mesh* m, void* stream, mcl_step_stats* stats_host);

/* One kinetic step: movePoints(d) + untangle + delonize in one persistent launch.
 * stats_host may be NULL (then the call does not synchronise the stream). */
int mcl_step(mcl_mesh* m, const mcl_float2* d_dev, void* stream, mcl_step_stats* stats_host);

/* Same step with the displacement in host memory (copied in on `stream`). */
int mcl_step_host(mcl_mesh* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats_host);

/* Pipelined form of mcl_step_host: returns at once.  The host-to-device copy of
 * d_host (pinned memory, kept unchanged until the copy is done) runs on a copy
 * stream of the mesh into one of two staging buffers, overlapping the step in
 * flight; the step runs on `stream` after its copy, and its counters land in
 * *stats_pinned (pinned host memory, may be NULL): written by the step's last
 * block when the device can address the record (cudaHostGetDevicePointer),
 * else copied on `stream`.  Synchronise `stream` (or an event recorded on it)
 * before reading them.  No counterpart in the reference. */
int mcl_step_host_async(mcl_mesh* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats_pinned);

/* Counters summed over every call on this mesh since creation (synchronises
 * the device); *calls_host (may be NULL) = number of engine launches.  Check
 * failed_launches after a run of asynchronous steps: status reports only the
 * last launch. */
int mcl_mesh_totals(mcl_mesh* m, mcl_step_stats* totals_host, int64_t* calls_host);

/* Status of the last asynchronous step on this mesh (synchronises the stream). */
int mcl_mesh_last_status(mcl_mesh* m, void* stream, mcl_step_stats* stats_host);

/* oneRing<M> / oneRing2<M> (include/Device_Triangulation.h:499-517): neighbour ids
 * around every vertex, in the layout given; at most M-1 neighbours are stored
 * (the reference's truncation, include/kernels.cuh:68).  Order: clockwise
 * (the reference's PREV_OUTGOING walk), starting at the smallest neighbour id.
 * *truncated_host (may be NULL) receives the number of truncated vertices. */
int mcl_one_ring(mcl_mesh* m, int layout, int max_ring, int32_t* ring_dev, void* stream,
                 int64_t* truncated_host);

/* closestNeighbors<M> / closestNeighbors2<M> (include/Device_Triangulation.h:519-547):
 * nearest ring neighbour of every vertex (ties: smallest id). */
int mcl_closest_neighbors(mcl_mesh* m, int layout, int max_ring, const int32_t* ring_dev,
                          int32_t* closest_dev, void* stream);

/* getFRNN<M,F> / getFRNN2<M,F> (include/Device_Triangulation.h:529-557): all
 * vertices j != i with fl(fl(dx*dx) + fl(dy*dy)) <= fl(r*r) (dx = p_i - p_j in
 * float), found by a walk over the mesh; at most F-1 per vertex, sorted
 * ascending.  *overflow_host (may be NULL) receives the number of vertices
 * whose list was truncated. */
int mcl_mesh_frnn(mcl_mesh* m, float r, int layout, int max_frnn, int32_t* out_dev, void* stream,
                  int64_t* overflow_host);

/* ---- uniform-grid fixed-radius neighbours (include/gridCount2d.h) ---------- */
typedef struct mcl_grid mcl_grid;

enum { MCL_GRID_PERIODIC = 1 };

/* GridCount2d(numP, min, cell_size, num_cells) (include/gridCount2d.h:50-71).
 * flags: MCL_GRID_PERIODIC wraps the cells and uses minimum-image distances on
 * a torus of size cell_size*num_cells. */
int mcl_grid_create(int64_t num_points, float min_x, float min_y, float cell_x, float cell_y,
                    int32_t cells_x, int32_t cells_y, int flags, mcl_grid** out);
int mcl_grid_destroy(mcl_grid* g);

/* GridCount2d::update(pos[, vel]) (include/gridCount2d.h:119-135, :174-260): sorts
 * the points by cell (cells row-major like the reference's hash y*nx + x,
 * points inside a cell by their previous index) and permutes pos_dev (and
 * vel_dev when not NULL) in place. */
int mcl_grid_update(mcl_grid* g, mcl_float2* pos_dev, mcl_float2* vel_dev, void* stream);

/* d_ind: perm_dev[i] = sorted position of the point that was at index i before
 * the last update; cell tables for header-side functors (apply_f_frnn). */
int mcl_grid_tables(mcl_grid* g, const int32_t** perm_dev, const int32_t** cell_start_dev,
                    const int32_t** cell_count_dev, int32_t* cells_x, int32_t* cells_y);

/* Everything a header-side functor loop (apply_f_frnn) needs to visit cells:
 * the cell of a point is (x, y) = floor((p - min) / cell), wrapped when
 * periodic, else clamped to [0, cells); its table index is
 * morton ? interleave(x, y) (x in the even bits) : y * cells_x + x. */
typedef struct {
  float min_x, min_y, cell_x, cell_y;
  int32_t cells_x, cells_y, morton, periodic;
  int64_t table_size, num_points;
  const int32_t* perm_dev;        /* d_ind */
  const int32_t* cell_start_dev;  /* first sorted index of each cell */
  const int32_t* cell_count_dev;  /* points in each cell */
} mcl_grid_desc;
int mcl_grid_describe(mcl_grid* g, mcl_grid_desc* desc_host);

/* apply_f_frnn with the reference tests' SaveNeighborsFunctor
 * (tests/grid2d_frnn.cu:26-60): for every sorted point i, the sorted indices j != i
 * with fl(fl(dx*dx)+fl(dy*dy)) <= fl(r*r), in the reference's stencil order
 * (cell rows bottom to top, cells left to right, points of a cell in sorted
 * order; gridCount2d.h:263-296); ROW layout without the
 * count slot: counts_dev[i], ids_dev[i*max_nb + k].  *overflow_host may be NULL. */
int mcl_grid_frnn(mcl_grid* g, const mcl_float2* pos_dev, float r, int max_nb, int32_t* counts_dev,
                  int32_t* ids_dev, void* stream, int64_t* overflow_host);

/* GridCount2d::update without the in-place permutation (the tables of
 * include/gridCount2d.h:174-260 for positions the caller must keep in order,
 * e.g. a mesh's vertex positions): builds the cell tables and keeps the sorted
 * copy inside the grid; pos_dev is only read. */
int mcl_grid_build(mcl_grid* g, const mcl_float2* pos_dev, void* stream);

/* mcl_grid_frnn over the positions of the last mcl_grid_build / mcl_grid_update,
 * in INPUT index space: counts_dev[i] and ids_dev[i*max_nb + k] for input point
 * i, neighbour input indices in stencil order (the SaveNeighborsFunctor result of
 * tests/grid2d_frnn.cu:26-60 mapped back through d_ind). */
int mcl_grid_frnn_ids(mcl_grid* g, float r, int max_nb, int32_t* counts_dev, int32_t* ids_dev, void* stream,
                      int64_t* overflow_host);

/* mean_num_particle_in_cell (include/gridCount2d.h:314-334). */
int mcl_grid_mean_occupancy(mcl_grid* g, float* mean_host);

/* Grid fixed-radius neighbours for callers that cannot allocate device memory
 * (frameworks that own all GPU memory, loops that must not block in an
 * allocator).  No counterpart in the reference: it does what mcl_grid_create +
 * mcl_grid_update + mcl_grid_frnn do, but allocates nothing and leaves pos_dev
 * untouched.  Its scratch is one fixed array in the library's device image
 * (5.3 MB held on every GPU that loads the library until exit); limits: n <=
 * 262144 points and at most 262144 cell-table entries, else MCL_ERR_CAPACITY.
 * Outputs (caller-owned device buffers): sorted_pos_dev[n] = positions in cell
 * order, perm_dev[n] = sorted slot of input point i, counts_dev[n] and
 * ids_dev[n*max_nb] = neighbours in sorted index space, as mcl_grid_frnn.
 * The first call on a device looks up the array's device address (do it before
 * any stream capture).  All calls share the array, so calls that overlap on the
 * GPU race; serialise them (one stream, or events). */
int mcl_grid_frnn_noalloc(const mcl_float2* pos_dev, int64_t n, float min_x, float min_y, float cell_x,
                          float cell_y, int32_t cells_x, int32_t cells_y, int flags, float r, int max_nb,
                          mcl_float2* sorted_pos_dev, int32_t* perm_dev, int32_t* counts_dev, int32_t* ids_dev,
                          void* stream, int64_t* overflow_host);

/* ---- batches of meshes ---------------------------------------------------------
 * No counterpart in the reference, which steps one DeviceTriangulation at a
 * time.  A batch is an mcl_mesh whose connected components are independent
 * meshes (each with its own bounding square): every mesh call above
 * (mcl_step, mcl_one_ring, mcl_mesh_validate, ...) works on it and processes
 * all meshes in one launch.  Vertex and edge ids are global in the batch;
 * mcl_batch_range gives each mesh's slice. */

/* Copy `count` meshes (their validated state) into a new batch; the inputs are
 * unchanged and may be destroyed.  At most 2^30 vertices and 2^29 edges. */
int mcl_batch_create(mcl_mesh* const* meshes, int64_t count, mcl_mesh** out);
/* Number of meshes in a batch (1 for a plain mesh). */
int mcl_batch_count(const mcl_mesh* m, int64_t* count);
/* Mesh i of the batch: vertices [v0, v0 + nv), edges [e0, e0 + ne). */
int mcl_batch_range(const mcl_mesh* m, int64_t i, int64_t* v0, int64_t* nv, int64_t* e0, int64_t* ne);
/* Per vertex: index of its mesh (int32[V], device; NULL for a plain mesh). */
int mcl_batch_vertex_mesh(const mcl_mesh* m, const int32_t** vcomp_dev);
/* transferToHost for mesh i alone, renumbered from 0 (same layout as
 * mcl_mesh_download_aos). */
int mcl_batch_download_aos(mcl_mesh* m, int64_t i, mcl_float2* pos_host, int32_t* v_host, int32_t* he_host,
                           int32_t* t_host);
/* getFRNN (include/Device_Triangulation.h:529-557) with one radius per mesh:
 * r_dev[i] for the vertices of mesh i (a plain mesh reads r_dev[0]). */
int mcl_batch_frnn(mcl_mesh* m, const float* r_dev, int layout, int max_frnn, int32_t* out_dev, void* stream,
                   int64_t* overflow_host);
/* mcl_batch_frnn (ROW layout) over per-mesh uniform grids instead of mesh
 * walks: mesh c gets a grid over [lo, hi)^2 with cells of its radius r_host[c]
 * (r_dev holds the same radii on the device); one counting sort of every
 * point, one query kernel.  Same rows as mcl_batch_frnn (ascending vertex
 * ids); max_frnn <= 49; every mesh of the batch (no active subset). */
int mcl_batch_frnn_grid(mcl_mesh* m, const float* r_host, const float* r_dev, float lo, float hi, int max_frnn,
                        int32_t* out_dev, void* stream, int64_t* overflow_host);
/* Mesh FRNN (getFRNN semantics) for a list of query vertices: row q of out_dev
 * (n rows, COLUMN or ROW layout with the count slot) holds the neighbours of
 * verts_dev[q] within r_dev[its mesh], ascending. */
int mcl_batch_frnn_list(mcl_mesh* m, const float* r_dev, const int32_t* verts_dev, int64_t n, int layout,
                        int max_frnn, int32_t* out_dev, void* stream, int64_t* overflow_host);
/* oneRing (include/Device_Triangulation.h:499-517) for a list of query vertices. */
int mcl_one_ring_list(mcl_mesh* m, const int32_t* verts_dev, int64_t n, int layout, int max_ring, int32_t* out_dev,
                      void* stream, int64_t* truncated_host);
/* Restrict the following mcl_step, mcl_untangle, mcl_delaunay_restore,
 * mcl_walk, mcl_settle_moves and mcl_dla_freeze calls to the listed meshes of
 * a batch (n == 0: every mesh again).  The other meshes are left exactly as
 * they are, and a launch costs only what the listed meshes hold.
 * Synchronises `stream` (the list is staged through one pinned buffer);
 * mcl_move and mcl_integrate refuse to run while a subset is active. */
int mcl_batch_set_active(mcl_mesh* m, const int32_t* meshes_host, int64_t n, void* stream);
/* A copy of a mesh or batch at its validated state (for snapshots and tuning). */
int mcl_mesh_clone(const mcl_mesh* src, mcl_mesh** out);

/* Launch shape of the kinetic step: blocks_per_sm in [1, max] (0 = max), and
 * the work-list size at or below which one block finishes the flip rounds
 * (0 = 2048).  Results do not depend on either. */
int mcl_mesh_set_tuning(mcl_mesh* m, int blocks_per_sm, int tail_items);
/* Work-list tile of the repair's removal rounds: how many lanes of each warp
 * take entries of the vertex list (1..32; 0 = automatic, as few as let one
 * pass over the grid take the list).  A removal is a long divergent chain,
 * so fewer lanes per warp run faster when the grid has warps to spare.
 * Results do not depend on it.  No reference counterpart. */
int mcl_mesh_set_removal_tile(mcl_mesh* m, int tile);
int mcl_mesh_get_removal_tile(const mcl_mesh* m, int* tile);

/* Repair sub-steps per kinetic step (default 0: every vertex sent back while
 * untangling is removed and reinserted at its target).  A sub-step moves the
 * sent-back vertices toward their targets as far as their stars allow and
 * restores the Delaunay property around them; those still short of their
 * targets after the last sub-step are removed and reinserted.  The resulting
 * mesh is the same Delaunay triangulation either way. */
int mcl_mesh_set_substeps(mcl_mesh* m, int substeps);
int mcl_mesh_get_tuning(const mcl_mesh* m, int* blocks_per_sm, int* tail_items, int* max_blocks_per_sm);

/* ---- motion models ----------------------------------------------------------- */
/* Gaussian random walk, the motion of the reference's diffusion-limited
 * aggregation experiment (experiments/diffusion_limited_aggregation.cu:51-60,
 * :263-268): d_dev[v] = clamp(pos + sigma * N(0, I), lo, hi) - pos with
 * sigma = sigma_dev[mesh of v], zero for the bounding corners and for vertices
 * with frozen_dev[v] != 0 (frozen_dev may be NULL).  counter_dev holds one
 * step counter per mesh (uint64[meshes]).  The normal draws of vertex v of
 * mesh c are a function of (seed + c, counter_dev[c], the id of v within
 * mesh c) only (a counter-based generator), so a mesh draws the same numbers
 * alone (with seed + c) as inside a batch, whatever else runs; the counters
 * of the walked meshes are incremented on the device after the draw, so a
 * captured CUDA graph replays new steps. */
int mcl_walk(mcl_mesh* m, const float* sigma_dev, const uint8_t* frozen_dev, uint64_t seed, uint64_t* counter_dev,
             float lo, float hi, mcl_float2* d_dev, void* stream);
/* mcl_walk with the generator key of mesh c taken from seeds_dev[c]
 * (uint64[meshes]) instead of seed + c, so a mesh keeps its own draws when it
 * moves to another batch or position in a batch (the serving layer regroups
 * meshes as they arrive and leave).  No reference counterpart. */
int mcl_walk_seeded(mcl_mesh* m, const float* sigma_dev, const uint8_t* frozen_dev, const uint64_t* seeds_dev,
                    uint64_t* counter_dev, float lo, float hi, mcl_float2* d_dev, void* stream);
/* Refuse moves that would put two vertices of one mesh at the same point: while
 * two vertices sit at one point, each of them that moves is sent back (its
 * displacement zeroed).  The result does not depend on thread order; vertices
 * that do not move never yield.  No counterpart in the reference (duplicate
 * points make its triangulation undefined).  *sent_back_host (may be NULL: no
 * synchronisation) = displacements zeroed. */
int mcl_settle_moves(mcl_mesh* m, mcl_float2* d_dev, void* stream, int64_t* sent_back_host);
/* check_if_close_diffusion (experiments/diffusion_limited_aggregation.cu:51-60),
 * in place: a free vertex v becomes frozen when a vertex that was frozen before
 * the call lies within r_dev[mesh of v] (fl(dx*dx + dy*dy) <= fl(r*r)).  The
 * decisions read the state before the call only, so the result does not
 * depend on thread order.  *newly_frozen_host may be NULL. */
int mcl_dla_freeze(mcl_mesh* m, const float* r_dev, uint8_t* frozen_dev, void* stream, int64_t* newly_frozen_host);

/* ---- diagnostics ------------------------------------------------------------ */
/* Structural invariants of the device mesh; counts8[k] = violations of kind k:
 * 0 next/prev not inverse, 1 inner face not a 3-cycle, 2 apex != origin(prev),
 * 3 origin(next) != origin(twin), 4 vertex half-edge not outgoing,
 * 5 face orientation <= 0 (exact), 6 dead edge, 7 index out of range.
 * All zero for a valid triangulation. */
int mcl_mesh_validate(mcl_mesh* m, int64_t* counts8);
/* Device diagnostics record of the last call: out68[0] = 1 + id of the first
 * vertex whose removal failed (0 if none), out68[1] = its degree, then its
 * neighbour ids in counter-clockwise order. */
int mcl_debug_state(mcl_mesh* m, int32_t* out68);
/* Device timestamps (ns, %globaltimer) of the last engine launch: [0] start,
 * [1] after the classification barrier, [2 + r] end of flip round r (r < 40),
 * [47] end; unused slots keep older values. */
int mcl_debug_timeline(mcl_mesh* m, int64_t* out48);
/* All counters of the last launch (engine order: flips, flip rounds, inverted
 * faces, reverted, removed, removal flips, insertion rounds, incircle tests and
 * stages, orientation stages, perturbation decisions, expansion overflows,
 * fixpoint passes, removal
 * rounds); returns how many exist. */
int mcl_debug_counters(mcl_mesh* m, int64_t* out, int n);
/* %globaltimer marks of the reinsertion rounds r < 16 of the last launch:
 * [4r] located, [4r+1] winners known, [4r+2] split, [4r+3] flips done. */
int mcl_debug_insert_timeline(mcl_mesh* m, int64_t* out64);
/* %globaltimer marks of the repair's removal rounds r < 16 of the last launch:
 * [4r] stars claimed, [4r+1] winners known, [4r+2] removed; [48 + p] end of
 * send-back pass p < 16; [64 + r] the slowest removal of round r since the
 * last call, (SM cycles << 16) | spokes; [80 + r] removals of round r that
 * walked their star again.  Diagnostics only (no reference counterpart). */
int mcl_debug_remove_timeline(mcl_mesh* m, int64_t* out96);

/* The device predicate ladder evaluated on the host CPU (same source as the
 * device code), for testing without a GPU.  kind 0 = orient2d on n records of
 * 6 floats, 1 = incircle on n records of 8 floats, 2 = incircle with symbolic
 * perturbation (ids: n records of 4 ints).  stage_out (may be NULL) receives
 * the stage that decided each record (0 fp32, 1 fp64, 2 exact, 3 perturbation). */
int mcl_debug_predicates_host(int kind, const float* pts, const int32_t* ids, int64_t n,
                              int32_t* sign_out, int32_t* stage_out);
/* The same on the GPU (device pointers). */
int mcl_debug_predicates_device(int kind, const float* pts_dev, const int32_t* ids_dev, int64_t n,
                                int32_t* sign_dev, int32_t* stage_dev, void* stream);

/* ---- periodic (flat torus) meshes ------------------------------------------
 * The reference's periodic triangulation is a stub
 * (include/Host_PeriodicTriangulation.h: the constructor at :101-104 keeps a
 * CGAL periodic domain, commented out; the rest is the bounding-square code).
 * Here: n points on the torus [2L, 3L)^2, L a power of two (so every
 * translate by one period is an exact float), point ids 0..n-1 in the
 * caller's order, 3n edges, 2n faces, no bounding square.  Edge e holds
 * ev[e] = (a, b, c, d) and en[e] = (next h0, prev h0, next h1, prev h1) as in
 * the planar engine (h0 = 2e: a -> b with apex c; h1 = 2e + 1: b -> a with apex
 * d) and one offset word eo[e]: bytes 0, 1, 2 hold, in periods, the copy of b
 * relative to a, of c relative to a, and of d relative to b, a nibble per
 * component biased by 8 (x low, y high). */
typedef struct mcl_periodic mcl_periodic;

/* Exact periodic Delaunay triangulation of pts_host (n points in
 * [2L, 3L)^2, in general position), built on the GPU as the planar
 * triangulation of the points and their copies within a band around the
 * domain, restricted to the torus.  Fails with MCL_ERR_DEGENERATE_INPUT when
 * the points are too sparse for the period (a face would use two copies of
 * one point). */
int mcl_periodic_build(const mcl_float2* pts_host, int64_t n, float L, mcl_periodic** out);

/* A periodic mesh from host arrays in the layout above (validated). */
int mcl_periodic_create(const mcl_float2* pos_host, int64_t n, float L, const int32_t* ev_host,
                        const int32_t* en_host, const uint32_t* eo_host, mcl_periodic** out);
int mcl_periodic_destroy(mcl_periodic* m);
int mcl_periodic_sizes(const mcl_periodic* m, int64_t* n, int64_t* E, float* L);
/* Any pointer may be NULL. */
int mcl_periodic_download(mcl_periodic* m, mcl_float2* pos_host, int32_t* ev_host, int32_t* en_host,
                          uint32_t* eo_host);
/* The device positions (float2[n], canonical, in [2L, 3L)^2). */
int mcl_periodic_positions(mcl_periodic* m, mcl_float2** pos_dev);

/* One kinetic step on the torus: every point moves by d_dev[i] (device,
 * float2[n]; shorter than a period) and wraps into the domain, then parallel
 * Lawson flip rounds restore the periodic Delaunay triangulation.  Moves that
 * would turn faces over are refused vertex by vertex: the farthest-moved
 * vertex of every turned face goes back to where it was (repeatedly, until no
 * face is turned) before any flip; then up to five sub-steps move
 * the vertices still owing part of their displacement by half of it (the last
 * by all of it, landing exactly on the target), each with the same refusal
 * and flips; the vertices still away after that are removed and reinserted
 * at their targets in claim-based rounds (removal rounds, then insertion
 * rounds; a point whose target is taken by an earlier one, by smallest id,
 * goes back where it was), then flips from the edges those rewrote.  The
 * whole step is one cooperative kernel launch; the call returns after reading
 * its result record (it synchronizes `stream`).  The result is the periodic
 * Delaunay triangulation of the moved points.  stats (may be NULL): inverted_faces (turned by the move),
 * substep_vertices (sent back, then brought to their target by sub-steps),
 * removed_vertices (removed and reinserted), reverted_vertices (not at their
 * target at the end), lawson_flips, lawson_rounds, the predicate counters,
 * status; wrapped (may be NULL): wraps across a side (a vertex may wrap in
 * more than one sub-step). */
int mcl_periodic_step(mcl_periodic* m, const mcl_float2* d_dev, void* stream, mcl_step_stats* stats,
                      int64_t* wrapped);
/* The same step with the displacements in host memory (copied in on `stream`). */
int mcl_periodic_step_host(mcl_periodic* m, const mcl_float2* d_host, void* stream, mcl_step_stats* stats,
                           int64_t* wrapped);
/* Diagnostics of the last step: out32[0] = 0, out32[k] = ns from the launch's
 * start to the grid barrier ending its k-th phase (-1 past the last; 31
 * phases at most); phases (may be NULL) = grid barriers the launch passed. */
int mcl_periodic_debug_timeline(const mcl_periodic* m, int64_t* out32, int64_t* phases);

/* oneRing<M> / oneRing2<M> (include/Device_Triangulation.h:500-517) on a
 * periodic mesh: each vertex's neighbours clockwise, starting at the smallest
 * (id, offset), at most max_ring - 1 of them, slot 0 the count; layout
 * MCL_LAYOUT_COLUMN (ring[(k+1) n + i]) or MCL_LAYOUT_ROW (ring[i max_ring + k]).
 * offs_dev (may be NULL; same layout, one byte per slot) receives each
 * neighbour's copy offset relative to the vertex (an offset byte as in eo).
 * truncated (may be NULL): vertices with more than max_ring - 1 neighbours. */
int mcl_periodic_one_ring(mcl_periodic* m, int max_ring, int layout, int32_t* ring_dev, uint8_t* offs_dev,
                          void* stream, int64_t* truncated);

/* closestNeighbors<M> (include/Device_Triangulation.h:520-528) on a periodic
 * mesh, from a ring table and its offsets: the neighbour nearest on the torus
 * (the reference's float squared distance; smallest id among equals). */
int mcl_periodic_closest(mcl_periodic* m, int max_ring, int layout, const int32_t* ring_dev,
                         const uint8_t* offs_dev, int32_t* closest_dev, void* stream);

/* getFRNN<M,F> (include/Device_Triangulation.h:530-538) on a periodic mesh:
 * for each vertex, every other vertex with a copy within r (r < L/2), found by
 * a search over the mesh; ascending ids, slot 0 the count, at most
 * max_frnn - 1 (layouts as for the ring).  offs_dev (may be NULL) receives
 * each one's copy offset byte.  truncated (may be NULL): vertices with more. */
int mcl_periodic_frnn(mcl_periodic* m, float r, int max_frnn, int layout, int32_t* out_dev, uint8_t* offs_dev,
                      void* stream, int64_t* truncated);

/* Host conversion behind mcl_periodic_build, for meshes built elsewhere: the
 * periodic mesh that a planar triangulation of a cover of the torus stands
 * for.  vertex_point[v] / vertex_copy[v] give, for each vertex of the planar
 * AoS mesh, the point id it is a copy of and the copy k = 3 (oy + 1) + (ox + 1)
 * of its translate (ox, oy) periods (-1 for vertices that are no copy, like
 * the bounding corners).  A face stands for its torus face when the copy of its
 * smallest point id is the untranslated one (k = 4).  Output: ev, en (int32[3n][4])
 * and eo (uint32[3n]), edges numbered by (u, v, offset) in ascending order.
 * No device work. */
int mcl_periodic_from_planar(const mcl_aos_view* planar_host, const int32_t* vertex_point,
                             const int32_t* vertex_copy, int64_t n, int32_t* ev_host, int32_t* en_host,
                             uint32_t* eo_host);

#ifdef __cplusplus
}
#endif

#endif /* MCL_GB300_H */
