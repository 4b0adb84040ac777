// Serial run, on the CPU, of the periodic step's kernel bodies
// (mcleap_gb300/csrc/periodic.cuh) in the order of the GPU step's phases: move +
// wrap every vertex, fold the wraps into every edge word, then rounds of
// classify-all and either (faces turned over) send their moved vertices back
// and fold again, or flip the winners, until no edge is non-Delaunay.  (The GPU
// folds each edge's wraps just before classifying it, in the same pass; an
// edge's fold touches only its own word, so the order is equivalent.)  A serial
// run of one phase gives the GPU's result (claims are max-reductions, one
// round's flips write disjoint fields), so this checks the device code's logic
// and indexing without a GPU.
//
//   periodic_step IN OUT
//   IN : int32 n, int32 E, float L, float r (FRNN radius), float pos[n][2], float d[n][2],
//        int32 ev[E][4], int32 en[E][4], uint32 eo[E]
//   OUT: int32 status, int32 flips, int32 wrapped, int32 inverted, int32 rounds,
//        int32 nonpositive_after, int32 truncated, int32 reverted, int32 revert_passes,
//        int32 behind (not at the target at the end), int32 substep_arrivals,
//        int32 classified (edge classifications over all rounds), int32 reinserted,
//        float pos[n][2], int32 ev[E][4],
//        int32 en[E][4], uint32 eo[E], then the queries on the final mesh:
//        int32 ring[kRing][n] and uint8 offs[kRing][n] (column layout), int32 closest[n],
//        int32 frnn[kFrnn][n] and uint8 frnn_offs[kFrnn][n], int32 frnn_truncated
// status: an MCL_* code from the bodies (0 ok), 100 + an I/O failure.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "periodic.cuh"
#include "periodic_rounds.h"

using mcl::PF2;
using mcl::PI4;

namespace {

template <typename T>
bool rd(FILE* f, T* p, size_t k) { return fread(p, sizeof(T), k, f) == k; }
template <typename T>
void wr(FILE* f, const T* p, size_t k) { fwrite(p, sizeof(T), k, f); }

constexpr int kRing = 8;  // small enough that some rings are truncated
constexpr int kFrnn = 64;
constexpr int kMaxRevertPasses = 256;
constexpr int kSubLevels = 5;

struct NoCount {
  int incircle_fp64, incircle_exact, orient_fp64, orient_exact, sos;
};

// orientation of the face of half-edge h, in its origin's frame
int face_sign(const mcl::PView& V, int h) {
  const int e = h >> 1, s = h & 1;
  const PI4 q = V.ev[e];
  const int o = s ? q.y : q.x, t = s ? q.x : q.y, x = s ? q.w : q.z;
  const PF2 pt = mcl::off_translate(V.pos[t], mcl::eo_target(V.eo[e], s), V.L);
  const PF2 px = mcl::off_translate(V.pos[x], mcl::eo_apex(V.eo[e], s), V.L);
  int overflow = 0;
  return mcl::orient2d(V.pos[o].x, V.pos[o].y, pt.x, pt.y, px.x, px.y, (NoCount*)nullptr, &overflow);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) return 1;
  int n = 0, E = 0;
  float L = 0, r = 0;
  FILE* in = fopen(argv[1], "rb");
  if (!in || !rd(in, &n, 1) || !rd(in, &E, 1) || !rd(in, &L, 1) || !rd(in, &r, 1)) return 2;
  std::vector<PF2> pos(n), d(n);
  std::vector<PI4> ev(E), en(E);
  std::vector<uint32_t> eo(E), cand(E, 0);
  std::vector<unsigned char> wv(n, 0x88), wt(n, 0x88), mark(n, 0);
  std::vector<PF2> pos_old(n);
  std::vector<unsigned long long> claim(2 * (size_t)E, 0);
  if (!rd(in, pos.data(), n) || !rd(in, d.data(), n) || !rd(in, ev.data(), E) || !rd(in, en.data(), E) ||
      !rd(in, eo.data(), E))
    return 3;
  fclose(in);

  mcl::PCount cnt{};
  std::vector<PF2> target(n), dsub(n);
  std::vector<int> clist(E), wl0(E), wl1(E);
  std::vector<unsigned> qstamp(E, 0);
  mcl::PView V{n,           E,           L,           2.0f * L,       pos.data(),    ev.data(),   en.data(),
               eo.data(),   wv.data(),   wt.data(),   mark.data(),    pos_old.data(), target.data(), cand.data(),
               claim.data(), &cnt,       clist.data(), wl0.data(),    wl1.data(),    qstamp.data()};
  long long classified = 0;
  int rounds = 0, revert_passes = 0;
  unsigned stamp = 0;
  long long inverted = -1;
  // the phases of mcl_periodic_step's launch, one after another; starts from
  // every edge (cur0 < 0) or from work-list cur0 (cnt.lcount[cur0] entries)
  auto settle = [&](int cur0) {
    bool flipped = false;
    int passes = 0, cur = cur0;  // the work-list to classify (-1: every edge)
    for (int r = 0; r < 4096; ++r) {
      ++stamp;
      cnt.nondelaunay = 0;
      cnt.inverted = 0;
      const long long items = cur < 0 ? E : (long long)cnt.lcount[cur];
      const int* wl = cur == 1 ? wl1.data() : wl0.data();
      for (long long i = 0; i < items; ++i) mcl::p_body_classify(V, cur < 0 ? (int)i : wl[i], stamp);
      classified += items;
      ++rounds;
      if (cnt.error) return;
      if (inverted < 0) inverted = (long long)cnt.inverted;
      if (cnt.inverted) {
        if (flipped || passes == kMaxRevertPasses) {
          cnt.error = flipped ? MCL_ERR_DEGENERATE_INPUT : MCL_ERR_NO_CONVERGENCE;
          return;
        }
        for (int v = 0; v < n; ++v) mcl::p_body_revert(V, v);
        for (int e = 0; e < E; ++e) mcl::p_body_wrap(V, e);
        ++passes;
        ++revert_passes;
        cur = -1;
        continue;
      }
      if (!cnt.nondelaunay) return;
      const int next = cur == 0 ? 1 : 0;
      cnt.lcount[next] = 0;
      for (unsigned long long i = 0; i < cnt.nondelaunay; ++i) mcl::p_body_flip(V, clist[i], stamp, next);
      cur = next;
      flipped = true;
    }
    cnt.error = MCL_ERR_NO_CONVERGENCE;
  };
  for (int v = 0; v < n; ++v) mcl::p_body_target(V, d.data(), v);
  for (int v = 0; v < n; ++v) mcl::p_body_move(V, d.data(), v);
  if (!cnt.error)
    for (int e = 0; e < E; ++e) mcl::p_body_wrap(V, e);
  if (!cnt.error) settle(-1);
  long long behind_first = -1, behind = 0;
  for (int level = 1; !cnt.error; ++level) {
    const bool last = level >= kSubLevels;
    cnt.behind = 0;
    for (int v = 0; v < n; ++v) mcl::p_body_resume(V, dsub.data(), v, last);
    behind = (long long)cnt.behind;
    if (behind_first < 0) behind_first = behind;
    if (behind == 0 || level > kSubLevels) break;
    for (int v = 0; v < n; ++v) mcl::p_body_move(V, dsub.data(), v);
    for (int e = 0; e < E; ++e) mcl::p_body_wrap(V, e);
    settle(-1);
  }
  // the rest: removed and reinserted in the launch's claim-based rounds
  // (each round's claims, then its verification, then its winners, as the
  // launch's phases), then flip rounds from the edges those rewrote
  long long substep_arrivals = behind_first > behind ? behind_first - behind : 0;
  if (!cnt.error && behind > 0) {
    std::vector<int> vh(n, -1);
    for (int h = 0; h < 2 * E; ++h) mcl::p_body_vhe(V, vh.data(), h);
    std::vector<int> list;
    for (int v = 0; v < n; ++v)
      if (pos[v].x != target[v].x || pos[v].y != target[v].y) list.push_back(v);
    unsigned long long lq = 0;
    periodic_par_rounds(V, vh.data(), list, stamp, &lq);
    if (!cnt.error) {
      cnt.lcount[0] = lq;
      settle(0);
    }
    behind = 0;
    for (int v = 0; v < n; ++v) behind += pos[v].x != target[v].x || pos[v].y != target[v].y;
  }
  int after = 0;
  if (!cnt.error)
    for (int h = 0; h < 2 * E; ++h) after += face_sign(V, h) <= 0;

  // queries, in launch order: outgoing half-edges, rings, closest neighbours
  std::vector<int> vhe(n, -1), ring((size_t)kRing * n, -1), closest(n, -2);
  std::vector<unsigned char> offs((size_t)kRing * n, 0);
  if (!cnt.error) {
    for (int h = 0; h < 2 * E; ++h) mcl::p_body_vhe(V, vhe.data(), h);
    for (int v = 0; v < n && !cnt.error; ++v) mcl::p_body_ring(V, vhe.data(), v, true, kRing, ring.data(), offs.data());
    for (int v = 0; v < n && !cnt.error; ++v)
      mcl::p_body_closest(V, v, true, kRing, ring.data(), offs.data(), closest.data());
  }
  std::vector<int> frnn((size_t)kFrnn * n, -1);
  std::vector<unsigned char> foffs((size_t)kFrnn * n, 0);
  const unsigned long long trunc_rings = cnt.truncated;
  if (!cnt.error)
    for (int v = 0; v < n && !cnt.error; ++v)
      mcl::p_body_frnn(V, vhe.data(), v, r * r, true, kFrnn, frnn.data(), foffs.data());
  const int32_t frnn_truncated = (int32_t)(cnt.truncated - trunc_rings);

  FILE* out = fopen(argv[2], "wb");
  if (!out) return 4;
  const int32_t head[13] = {(int32_t)cnt.error,     (int32_t)cnt.flips,    (int32_t)cnt.wrapped,
                            (int32_t)inverted,      rounds,                after,
                            (int32_t)trunc_rings,   (int32_t)cnt.reverted, revert_passes,
                            (int32_t)behind,        (int32_t)substep_arrivals,
                            (int32_t)classified,    (int32_t)cnt.reinserted};
  wr(out, head, 13);
  wr(out, pos.data(), n);
  wr(out, ev.data(), E);
  wr(out, en.data(), E);
  wr(out, eo.data(), E);
  wr(out, ring.data(), ring.size());
  wr(out, offs.data(), offs.size());
  wr(out, closest.data(), closest.size());
  wr(out, frnn.data(), frnn.size());
  wr(out, foffs.data(), foffs.size());
  wr(out, &frnn_truncated, 1);
  fclose(out);
  return 0;
}
