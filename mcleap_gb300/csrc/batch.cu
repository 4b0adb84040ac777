// Batches of independent meshes, motion models and settling of coincident moves.
//
// A batch is one mcl_mesh whose connected components are the meshes: their
// vertex and edge records are concatenated (ids offset), each keeps its own
// bounding square, and nothing links two components.  Every kernel of the
// engine walks the topology, so it never leaves a component; the one place
// that needs a starting half-edge by id (point location after a removal) falls
// back to the component's own half-edge 0 (vroot).  One cooperative launch of
// the kinetic step therefore steps every mesh of the batch.
//
// Motion:
//   mcl_walk           Gaussian random walk with a per-mesh sigma, clamped to
//                      a box, optionally only for unfrozen walkers (the
//                      diffusion-limited-aggregation motion of
//                      experiments/diffusion_limited_aggregation.cu:51-60,
//                      263-268 in the reference).
//   mcl_settle_moves   refuses moves that would make two vertices of one mesh
//                      coincide (the triangulation of coincident points is
//                      undefined); see the rule below.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace cg = cooperative_groups;
using namespace mcl;

namespace {

#define BCK(call)                                    \
  do {                                               \
    cudaError_t _e = (call);                         \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

// ---------------------------------------------------------------------------
// Batch assembly: copy one mesh's records into the batch with offset ids.
__global__ void k_append(int V, int E, const float2* pos, const int4* ev, const int4* en, const int* vhe,
                         const unsigned char* vfix, int vb, int eb, int comp, float2* pos0, float2* pos1, int4* ev_o,
                         int4* en_o, int* vhe_o, unsigned char* vfix_o, int* vcomp, int* vroot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int hb = 2 * eb;
  if (i < E) {
    const int4 q = ev[i];
    ev_o[eb + i] = make_int4(q.x < 0 ? -1 : q.x + vb, q.y < 0 ? -1 : q.y + vb, q.z < 0 ? -1 : q.z + vb,
                             q.w < 0 ? -1 : q.w + vb);
    const int4 n = en[i];
    en_o[eb + i] = make_int4(n.x < 0 ? -1 : n.x + hb, n.y < 0 ? -1 : n.y + hb, n.z < 0 ? -1 : n.z + hb,
                             n.w < 0 ? -1 : n.w + hb);
  }
  if (i < V) {
    const float2 p = pos[i];
    pos0[vb + i] = p;
    pos1[vb + i] = p;
    const int h = vhe[i];
    vhe_o[vb + i] = h < 0 ? -1 : h + hb;
    vfix_o[vb + i] = vfix[i];
    vcomp[vb + i] = comp;
    vroot[vb + i] = hb;
  }
}

// ---------------------------------------------------------------------------
// Counter-based random numbers: SplitMix64's finaliser (Steele, Lea and Flood,
// "Fast splittable pseudorandom number generators", 2014) over
// (seed, step, vertex, draw); uniforms in (0, 1] from the top 24 bits; normal
// pairs by the Box-Muller transform.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float2 normal2(unsigned long long seed, unsigned long long step, int v) {
  const unsigned long long a = mix64(seed ^ mix64(step * 0x100000001B3ull + (unsigned long long)v));
  const float u1 = ((unsigned)(a >> 40) + 1u) * (1.0f / 16777216.0f);  // (0, 1]
  const float u2 = ((unsigned)(a >> 16) & 0xFFFFFFu) * (1.0f / 16777216.0f);
  const float rad = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  return make_float2(rad * c, rad * s);
}

// d[v] = clamp(pos + sigma * N(0, I), lo, hi) - pos for free, unfrozen vertices;
// a displacement whose rounded sum would leave [lo, hi] is dropped.
// The draws of vertex v of mesh c are keyed by (seed + c, local id of v), so a
// mesh draws the same numbers alone (with seed + c) and inside a batch.
__global__ void k_walk(ActV A, const float2* __restrict__ pos, const unsigned char* __restrict__ vfix,
                       const int* __restrict__ vcomp, const int* __restrict__ cbase, const float* __restrict__ sigma,
                       const unsigned char* __restrict__ frozen, unsigned long long seed,
                       const unsigned long long* __restrict__ seeds,
                       const unsigned long long* __restrict__ counter, float lo, float hi, float2* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.V_it) return;
  const int v = A.at(i);
  float2 out = make_float2(0.f, 0.f);
  if (!vfix[v] && !(frozen && frozen[v])) {
    const int c = vcomp ? vcomp[v] : 0;
    const float sg = sigma[c];
    const float2 z = normal2(seeds ? seeds[c] : seed + (unsigned long long)c, counter[c], cbase ? v - cbase[c] : v);
    const float2 p = pos[v];
    const float tx = fminf(fmaxf(__fadd_rn(p.x, __fmul_rn(sg, z.x)), lo), hi);
    const float ty = fminf(fmaxf(__fadd_rn(p.y, __fmul_rn(sg, z.y)), lo), hi);
    out = make_float2(__fsub_rn(tx, p.x), __fsub_rn(ty, p.y));
    const float nx = __fadd_rn(p.x, out.x), ny = __fadd_rn(p.y, out.y);
    if (!(nx >= lo && nx <= hi)) out.x = 0.f;
    if (!(ny >= lo && ny <= hi)) out.y = 0.f;
  }
  d[v] = out;
}

// counter[c] += 1 for every active mesh c (every mesh when n == 0)
__global__ void k_advance(unsigned long long* counter, int n, const int* act, int ncomp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (n ? i < n : i < ncomp) counter[n ? act[i] : i] += 1;
}

// ---------------------------------------------------------------------------
// Settling coincident moves.
//
// Rule (a least fixed point, independent of thread order): start with every
// vertex at pos + d; while two vertices of one mesh sit at the same point,
// every MOVING vertex among them (d != 0) is sent back to pos (its d zeroed).
// Old positions are distinct, so the loop ends with distinct positions; a
// vertex that did not move never yields.
//
// Each pass inserts every vertex's candidate position into an open-addressing
// table keyed by (mesh, x, y) (entries stamped with the pass, so the table is
// never cleared); a vertex whose key is already present marks itself and the
// holder.  Marked movers are sent back, and passes repeat until none is.  A
// first pass flags the meshes that have a mover: the others cannot hold a
// coincident pair (their positions are distinct), so their vertices are not
// inserted (with an aggregation most meshes have no walker left).
__device__ __forceinline__ unsigned fbits(float x) { return x == 0.f ? 0u : __float_as_uint(x); }

__device__ __forceinline__ float2 cand_pos(const float2* pos, const float2* d, const unsigned char* vfix, int v) {
  const float2 p = pos[v];
  if (vfix[v]) return p;
  const float2 q = d[v];
  return make_float2(__fadd_rn(p.x, q.x), __fadd_rn(p.y, q.y));
}

struct SettleArgs {
  ActV A;
  const float2* pos;
  float2* d;
  const unsigned char* vfix;
  const int* vcomp;
  unsigned long long* table;
  unsigned long long mask;
  int* smark;
  unsigned* smove;         // per mesh: stamp of the call that found a mover in it
  DevState* st;
  int max_passes;
};

__global__ void k_settle(SettleArgs A) {
  cg::grid_group g = cg::this_grid();
  const int stride = gridDim.x * blockDim.x;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned* words = A.st->settle;
  const unsigned base = (unsigned)ld_i(reinterpret_cast<const int*>(words));
  const unsigned long long probe_cap = 2 * (A.mask + 1) + 1024;
  int pass = 0;
  bool lost = false;
  // meshes with a mover (stamp `base`, unique to this call)
  for (int vi = gtid; vi < A.A.V_it; vi += stride) {
    const int v = A.A.at(vi);
    if (A.vfix[v]) continue;
    const float2 q = A.d[v];
    if (q.x != 0.f || q.y != 0.f) {
      const int comp = A.vcomp ? A.vcomp[v] : 0;
      if (__ldcg(A.smove + comp) != base) atomicExch(A.smove + comp, base);
    }
  }
  g.sync();
  for (; pass < A.max_passes; ++pass) {
    const unsigned stamp = base + 1 + (unsigned)pass;
    const int slot = 1 + pass % 3;
    if (gtid == 0) words[1 + (pass + 1) % 3] = 0;
    for (int vi = gtid; vi < A.A.V_it; vi += stride) {
      const int v = A.A.at(vi);
      const int comp = A.vcomp ? A.vcomp[v] : 0;
      if (__ldcg(A.smove + comp) != base) continue;  // no mover in this mesh
      const float2 p = cand_pos(A.pos, A.d, A.vfix, v);
      const unsigned long long key = ((unsigned long long)fbits(p.x) << 32) | fbits(p.y);
      unsigned long long h = mix64(key ^ ((unsigned long long)comp * 0x9E3779B97F4A7C15ull)) & A.mask;
      bool placed = false;
      for (unsigned long long it = 0; it < probe_cap; ++it) {
        unsigned long long* slotp = A.table + h;
        const unsigned long long cur = __ldcg(slotp);
        if ((unsigned)(cur >> 32) != stamp) {
          const unsigned long long mine = ((unsigned long long)stamp << 32) | (unsigned)v;
          if (atomicCAS(slotp, cur, mine) == cur) { placed = true; break; }
          continue;  // lost the slot to another vertex: look at it again
        }
        const int u = (int)(unsigned)cur;
        const float2 q = cand_pos(A.pos, A.d, A.vfix, u);
        const int cu = A.vcomp ? A.vcomp[u] : 0;
        if (cu == comp && fbits(q.x) == fbits(p.x) && fbits(q.y) == fbits(p.y)) {
          atomicExch(A.smark + v, (int)stamp);
          atomicExch(A.smark + u, (int)stamp);
          placed = true;
          break;
        }
        h = (h + 1) & A.mask;
      }
      if (!placed) lost = true;
    }
    g.sync();
    int sent = 0;
    for (int vi = gtid; vi < A.A.V_it; vi += stride) {
      const int v = A.A.at(vi);
      if ((unsigned)__ldcg(A.smark + v) != stamp || A.vfix[v]) continue;
      const float2 q = A.d[v];
      if (q.x != 0.f || q.y != 0.f) {
        A.d[v] = make_float2(0.f, 0.f);
        ++sent;
      }
    }
    if (sent) {
      atomicAdd(words + slot, (unsigned)sent);
      atomicAdd(words + 4, (unsigned)sent);
    }
    if (lost) atomicOr(words + 5, 2u);
    g.sync();
    if (ld_i(reinterpret_cast<const int*>(words + slot)) == 0 || ld_i(reinterpret_cast<const int*>(words + 5))) break;
  }
  if (gtid == 0) {
    words[0] = base + 1 + (unsigned)A.max_passes;  // the next call's stamps are fresh
    if (pass >= A.max_passes) words[5] |= 1u;
  }
}

int ensure_settle_scratch(mcl_mesh* m) {
  if (m->table) return MCL_OK;
  int64_t size = 1;
  while (size < 2 * m->V) size <<= 1;
  BCK(cudaMalloc((void**)&m->table, 8 * size));
  BCK(cudaMalloc((void**)&m->smark, 4 * m->V));
  BCK(cudaMalloc((void**)&m->smove, 4 * std::max<int64_t>(1, m->ncomp)));
  BCK(cudaMemset(m->table, 0, 8 * size));
  BCK(cudaMemset(m->smark, 0, 4 * m->V));
  BCK(cudaMemset(m->smove, 0xFF, 4 * std::max<int64_t>(1, m->ncomp)));
  m->table_size = size;
  int per_sm = 0;
  BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_settle, 256, 0));
  if (per_sm < 1) return fail(MCL_ERR_CUDA, "k_settle cannot be resident");
  m->settle_blocks = m->nsm * std::min(per_sm, 4);
  return MCL_OK;
}

}  // namespace

extern "C" {

int mcl_batch_create(mcl_mesh* const* meshes, int64_t count, mcl_mesh** out) {
  if (!meshes || !out || count < 1) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_create: no meshes");
  int64_t V = 0, E = 0;
  for (int64_t i = 0; i < count; ++i) {
    if (!meshes[i]) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_create: null mesh");
    if (meshes[i]->ncomp != 1) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_create: nested batch");
    V += meshes[i]->V;
    E += meshes[i]->E;
  }
  if (V > (1ll << 30) || E > (1ll << 29))
    return fail(MCL_ERR_CAPACITY, "mcl_batch_create: more than 2^30 vertices or 2^29 edges in one batch");
  mcl_mesh* b = nullptr;
  int rc = alloc_mesh(V, E, &b);
  if (rc != MCL_OK) return rc;
  auto bail = [&](int code) {
    free_mesh(b);
    return code;
  };
  if (cudaMalloc((void**)&b->vcomp, 4 * V) != cudaSuccess || cudaMalloc((void**)&b->vroot, 4 * V) != cudaSuccess ||
      cudaMalloc((void**)&b->cbase, 4 * count) != cudaSuccess)
    return bail(fail(MCL_ERR_OUT_OF_MEMORY, "mcl_batch_create: component tables"));
  b->ncomp = count;
  b->comp_host = new int64_t[4 * count];
  std::vector<int> base((size_t)count);
  b->T = 0;
  int64_t vb = 0, eb = 0;
  for (int64_t i = 0; i < count; ++i) {
    mcl_mesh* m = meshes[i];
    b->comp_host[4 * i] = vb;
    base[(size_t)i] = (int)vb;
    b->comp_host[4 * i + 1] = m->V;
    b->comp_host[4 * i + 2] = eb;
    b->comp_host[4 * i + 3] = m->E;
    const int n = (int)std::max(m->V, m->E);
    k_append<<<(n + 255) / 256, 256>>>((int)m->V, (int)m->E, valid_positions(m), m->ev, m->en, m->vhe, m->vfix,
                                       (int)vb, (int)eb, (int)i, b->pos[0], b->pos[1], b->ev, b->en, b->vhe, b->vfix,
                                       b->vcomp, b->vroot);
    if (cudaGetLastError() != cudaSuccess) return bail(fail(MCL_ERR_CUDA, "mcl_batch_create: append"));
    b->T += m->T;
    vb += m->V;
    eb += m->E;
  }
  if (cudaMemcpy(b->cbase, base.data(), 4 * count, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess)
    return bail(fail(MCL_ERR_CUDA, "mcl_batch_create: sync"));
  b->dirty = new unsigned char[(size_t)count]();
  b->act_list = new int[(size_t)count];
  if (cudaMalloc((void**)&b->act_dev, 4 * (5 * count + 2)) != cudaSuccess ||
      cudaMallocHost((void**)&b->act_host, 4 * (5 * count + 2)) != cudaSuccess)
    return bail(fail(MCL_ERR_OUT_OF_MEMORY, "mcl_batch_create: active tables"));
  b->cur = 0;
  b->valid_cur = true;
  *out = b;
  return MCL_OK;
}

int mcl_batch_count(const mcl_mesh* m, int64_t* count) {
  if (!m || !count) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  *count = m->ncomp;
  return MCL_OK;
}

int mcl_batch_range(const mcl_mesh* m, int64_t i, int64_t* v0, int64_t* nv, int64_t* e0, int64_t* ne) {
  if (!m || i < 0 || i >= m->ncomp) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_range: bad mesh index");
  const int64_t* c = m->comp_host ? m->comp_host + 4 * i : nullptr;
  if (v0) *v0 = c ? c[0] : 0;
  if (nv) *nv = c ? c[1] : m->V;
  if (e0) *e0 = c ? c[2] : 0;
  if (ne) *ne = c ? c[3] : m->E;
  return MCL_OK;
}

int mcl_batch_vertex_mesh(const mcl_mesh* m, const int32_t** vcomp_dev) {
  if (!m || !vcomp_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  *vcomp_dev = m->vcomp;
  return MCL_OK;
}

int mcl_batch_download_aos(mcl_mesh* m, int64_t i, mcl_float2* pos, int32_t* v, int32_t* he, int32_t* t) {
  int64_t v0 = 0, nv = 0, e0 = 0, ne = 0;
  const int rc = mcl_batch_range(m, i, &v0, &nv, &e0, &ne);
  if (rc != MCL_OK) return rc;
  return download_range(m, v0, nv, e0, ne, 2 * (nv - 4) + 2, pos, v, he, t);
}

int mcl_mesh_clone(const mcl_mesh* src, mcl_mesh** out) {
  if (!src || !out) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  mcl_mesh* m = nullptr;
  int rc = alloc_mesh(src->V, src->E, &m);
  if (rc != MCL_OK) return rc;
  const int64_t V = src->V, E = src->E;
  cudaError_t e = cudaMemcpy(m->pos[0], valid_positions(src), 8 * V, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->pos[1], valid_positions(src), 8 * V, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->ev, src->ev, 16 * E, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->en, src->en, 16 * E, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->vhe, src->vhe, 4 * V, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->vfix, src->vfix, V, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess && src->vcomp) {
    e = cudaMalloc((void**)&m->vcomp, 4 * V);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->vroot, 4 * V);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->cbase, 4 * src->ncomp);
    if (e == cudaSuccess) e = cudaMemcpy(m->vcomp, src->vcomp, 4 * V, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(m->vroot, src->vroot, 4 * V, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(m->cbase, src->cbase, 4 * src->ncomp, cudaMemcpyDeviceToDevice);
  }
  if (e != cudaSuccess) {
    free_mesh(m);
    return cuda_fail(e, "mcl_mesh_clone");
  }
  m->T = src->T;
  m->ncomp = src->ncomp;
  if (src->comp_host) {
    m->comp_host = new int64_t[4 * src->ncomp];
    std::memcpy(m->comp_host, src->comp_host, sizeof(int64_t) * 4 * src->ncomp);
  }
  m->tail_items = src->tail_items;
  m->rm_tile = src->rm_tile;
  m->coop_blocks = src->coop_blocks;
  if (src->substeps > 0 && (rc = mcl_mesh_set_substeps(m, src->substeps)) != MCL_OK) {
    free_mesh(m);
    return rc;
  }
  if (src->dirty) {
    const int64_t nc = src->ncomp;
    m->dirty = new unsigned char[(size_t)nc]();
    m->act_list = new int[(size_t)nc];
    if (cudaMalloc((void**)&m->act_dev, 4 * (5 * nc + 2)) != cudaSuccess ||
        cudaMallocHost((void**)&m->act_host, 4 * (5 * nc + 2)) != cudaSuccess) {
      free_mesh(m);
      return fail(MCL_ERR_OUT_OF_MEMORY, "mcl_mesh_clone: active tables");
    }
  }
  *out = m;
  return MCL_OK;
}

int mcl_batch_set_active(mcl_mesh* m, const int32_t* meshes_host, int64_t n, void* stream) {
  if (!m || n < 0 || (n > 0 && !meshes_host)) return fail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  if (n == 0) {
    m->nact = 0;
    return MCL_OK;
  }
  if (!m->dirty) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_set_active: not a batch");
  if (n > m->ncomp) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_set_active: more meshes than the batch has");
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<unsigned char> seen((size_t)m->ncomp, 0);
  // the staging buffer may still feed the previous call's copy
  BCK(cudaStreamSynchronize(s));
  const int64_t nc = m->ncomp;
  int* epre = m->act_host;
  int* e0 = epre + nc + 1;
  int* vpre = e0 + nc;
  int* v0 = vpre + nc + 1;
  int* ids = v0 + nc;
  int64_t E = 0, V = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int c = meshes_host[i];
    if (c < 0 || c >= nc || seen[(size_t)c])
      return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_batch_set_active: mesh index out of range or repeated");
    seen[(size_t)c] = 1;
    m->act_list[i] = c;
    ids[i] = c;
    epre[i] = (int)E;
    e0[i] = (int)m->comp_host[4 * c + 2];
    vpre[i] = (int)V;
    v0[i] = (int)m->comp_host[4 * c];
    E += m->comp_host[4 * c + 3];
    V += m->comp_host[4 * c + 1];
  }
  epre[n] = (int)E;
  vpre[n] = (int)V;
  BCK(cudaMemcpyAsync(m->act_dev, m->act_host, 4 * (5 * nc + 2), cudaMemcpyHostToDevice, s));
  m->nact = (int)n;
  m->act_E = (int)E;
  m->act_V = (int)V;
  return MCL_OK;
}

int mcl_mesh_set_tuning(mcl_mesh* m, int blocks_per_sm, int tail_items) {
  if (!m || blocks_per_sm < 0 || tail_items < 0) return fail(MCL_ERR_INVALID_ARGUMENT, "bad tuning");
  const int bps = blocks_per_sm == 0 ? m->max_blocks_per_sm : blocks_per_sm;
  if (bps > m->max_blocks_per_sm)
    return fail(MCL_ERR_INVALID_ARGUMENT, "blocks per SM above the kernel's co-resident limit");
  m->coop_blocks = m->nsm * bps;
  m->tail_items = tail_items == 0 ? 2048 : tail_items;
  return MCL_OK;
}

int mcl_mesh_set_removal_tile(mcl_mesh* m, int tile) {
  if (!m || tile < 0 || tile > 32) return fail(MCL_ERR_INVALID_ARGUMENT, "removal tile must be in [0, 32]");
  m->rm_tile = tile;
  return MCL_OK;
}

int mcl_mesh_get_removal_tile(const mcl_mesh* m, int* tile) {
  if (!m || !tile) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  *tile = m->rm_tile;
  return MCL_OK;
}

int mcl_mesh_set_substeps(mcl_mesh* m, int substeps) {
  if (!m || substeps < 0 || substeps > 64) return fail(MCL_ERR_INVALID_ARGUMENT, "substeps must be in [0, 64]");
  if (substeps > 0 && !m->vl2) {
    // the sub-step scratch (24 B per vertex) exists only for meshes that use it
    BCK(cudaMalloc((void**)&m->vprev, 8 * m->V));
    const cudaError_t e = cudaMalloc((void**)&m->vl2, 16 * m->V);
    if (e != cudaSuccess) {
      cudaFree(m->vprev);
      m->vprev = nullptr;
      return cuda_fail(e, "cudaMalloc(sub-step scratch)");
    }
  }
  m->substeps = substeps;
  return MCL_OK;
}

int mcl_mesh_get_tuning(const mcl_mesh* m, int* blocks_per_sm, int* tail_items, int* max_blocks_per_sm) {
  if (!m) return fail(MCL_ERR_INVALID_ARGUMENT, "null mesh");
  if (blocks_per_sm) *blocks_per_sm = m->coop_blocks / std::max(1, m->nsm);
  if (tail_items) *tail_items = m->tail_items;
  if (max_blocks_per_sm) *max_blocks_per_sm = m->max_blocks_per_sm;
  return MCL_OK;
}

static int walk(mcl_mesh* m, const float* sigma_dev, const uint8_t* frozen_dev, uint64_t seed,
                const uint64_t* seeds_dev, uint64_t* counter_dev, float lo, float hi, mcl_float2* d_dev,
                void* stream) {
  if (!m || !sigma_dev || !counter_dev || !d_dev || !(lo <= hi)) return fail(MCL_ERR_INVALID_ARGUMENT, "bad args");
  cudaStream_t s = (cudaStream_t)stream;
  const int V = (int)m->V;
  const ActV A = act_of(m);
  (void)V;
  if (A.V_it > 0)
    k_walk<<<(A.V_it + 255) / 256, 256, 0, s>>>(A, m->pos[m->cur], m->vfix, m->vcomp, m->cbase, sigma_dev, frozen_dev,
                                                seed, reinterpret_cast<const unsigned long long*>(seeds_dev),
                                                reinterpret_cast<const unsigned long long*>(counter_dev), lo, hi,
                                                reinterpret_cast<float2*>(d_dev));
  const int na = m->nact ? m->nact : (int)m->ncomp;
  k_advance<<<(na + 255) / 256, 256, 0, s>>>(reinterpret_cast<unsigned long long*>(counter_dev), m->nact,
                                             m->nact ? m->act_dev + 4 * m->ncomp + 2 : nullptr,
                                             (int)m->ncomp);
  BCK(cudaGetLastError());
  return MCL_OK;
}

int mcl_walk(mcl_mesh* m, const float* sigma_dev, const uint8_t* frozen_dev, uint64_t seed,
             uint64_t* counter_dev, float lo, float hi, mcl_float2* d_dev, void* stream) {
  return walk(m, sigma_dev, frozen_dev, seed, nullptr, counter_dev, lo, hi, d_dev, stream);
}

int mcl_walk_seeded(mcl_mesh* m, const float* sigma_dev, const uint8_t* frozen_dev, const uint64_t* seeds_dev,
                    uint64_t* counter_dev, float lo, float hi, mcl_float2* d_dev, void* stream) {
  if (!seeds_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_walk_seeded: null seed table");
  return walk(m, sigma_dev, frozen_dev, 0, seeds_dev, counter_dev, lo, hi, d_dev, stream);
}

int mcl_settle_moves(mcl_mesh* m, mcl_float2* d_dev, void* stream, int64_t* sent_back_host) {
  if (!m || !d_dev) return fail(MCL_ERR_INVALID_ARGUMENT, "null argument");
  if (!m->valid_cur) return fail(MCL_ERR_INVALID_ARGUMENT, "mcl_settle_moves: points were moved without a step");
  int rc = ensure_settle_scratch(m);
  if (rc != MCL_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  SettleArgs A;
  A.A = act_of(m);
  A.pos = m->pos[m->cur];
  A.d = reinterpret_cast<float2*>(d_dev);
  A.vfix = m->vfix;
  A.vcomp = m->vcomp;
  A.table = m->table;
  A.mask = (unsigned long long)(m->table_size - 1);
  A.smark = m->smark;
  A.smove = m->smove;
  A.st = m->st;
  A.max_passes = 64;
  void* args[] = {&A};
  // words 1..5 (pass counters, total, status) start at zero; the stamp (word 0) persists
  BCK(cudaMemsetAsync(m->st->settle + 1, 0, 5 * sizeof(unsigned), s));
  BCK(cudaLaunchCooperativeKernel((void*)k_settle, dim3(m->settle_blocks), dim3(256), args, 0, s));
  if (sent_back_host) {
    unsigned h[6];
    BCK(cudaMemcpyAsync(h, m->st->settle, sizeof(h), cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    if (h[5] & 2u) return fail(MCL_ERR_CAPACITY, "mcl_settle_moves: position table full");
    if (h[5]) return fail(MCL_ERR_NO_CONVERGENCE, "mcl_settle_moves: pass limit reached");
    *sent_back_host = h[4];
  }
  return MCL_OK;
}

}  // extern "C"
