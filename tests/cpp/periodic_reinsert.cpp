// The removal and reinsertion of the periodic step run on the CPU for chosen
// vertices and targets, so that the rare branches (a target on an edge, a
// target already taken, a refused removal) can be driven directly: the
// one-thread pass (mcleap_gb300/csrc/periodic.cuh: p_body_reinsert), or with
// a third argument "rounds" the GPU launch's claim-based rounds
// (periodic_rounds.h) followed by flip rounds from the edges they rewrote
// ("rounds:S": every phase in a pseudo-random order drawn from seed S).
//
//   periodic_reinsert IN OUT [rounds[:S]]
//   IN : int32 n, int32 E, float L, int32 k, float pos[n][2], int32 ev[E][4],
//        int32 en[E][4], uint32 eo[E], int32 vert[k], float target[k][2]
//   OUT: int32 status, int32 reinserted, float pos[n][2], int32 ev[E][4],
//        int32 en[E][4], uint32 eo[E]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "periodic.cuh"
#include "periodic_rounds.h"

using mcl::PF2;
using mcl::PI4;

template <typename T>
static bool rd(FILE* f, T* p, size_t k) { return fread(p, sizeof(T), k, f) == k; }
template <typename T>
static void wr(FILE* f, const T* p, size_t k) { fwrite(p, sizeof(T), k, f); }

int main(int argc, char** argv) {
  if (argc != 3 && argc != 4) return 1;
  const bool rounds = argc == 4;
  const unsigned shuffle = rounds && argv[3][6] == ':' ? (unsigned)atoi(argv[3] + 7) : 0u;
  int n = 0, E = 0, k = 0;
  float L = 0;
  FILE* in = fopen(argv[1], "rb");
  if (!in || !rd(in, &n, 1) || !rd(in, &E, 1) || !rd(in, &L, 1) || !rd(in, &k, 1)) return 2;
  std::vector<PF2> pos(n), target, tv(k), pos_old(n);
  std::vector<PI4> ev(E), en(E);
  std::vector<uint32_t> eo(E), cand(E, 0), qstamp(E, 0);
  std::vector<int> vert(k), clist(E), wl0(E), wl1(E), vhe(n, -1);
  std::vector<unsigned char> wv(n, 0x88), wt(n, 0x88), mark(n, 0);
  std::vector<unsigned long long> claim(2 * (size_t)E, 0);
  if (!rd(in, pos.data(), n) || !rd(in, ev.data(), E) || !rd(in, en.data(), E) || !rd(in, eo.data(), E) ||
      !rd(in, vert.data(), k) || !rd(in, tv.data(), k))
    return 3;
  fclose(in);
  target = pos;
  for (int i = 0; i < k; ++i) target[vert[i]] = tv[i];
  mcl::PCount cnt{};
  mcl::PView V{n,           E,           L,           2.0f * L,       pos.data(),    ev.data(),   en.data(),
               eo.data(),   wv.data(),   wt.data(),   mark.data(),    pos_old.data(), target.data(), cand.data(),
               claim.data(), &cnt,       clist.data(), wl0.data(),    wl1.data(),    qstamp.data()};
  for (int h = 0; h < 2 * E; ++h) mcl::p_body_vhe(V, vhe.data(), h);
  if (!rounds) {
    mcl::p_body_reinsert(V, vhe.data(), vert.data(), k, 1 << 16);
  } else {
    unsigned stamp = 0;
    unsigned long long lq = 0;
    periodic_par_rounds(V, vhe.data(), vert, stamp, &lq, shuffle);
    // flip rounds from the rounds' work-list (wl0), as the launch's settle
    // from a list: classify the list, flip the winners, classify their wings
    int cur = 0;
    unsigned long long len = lq;
    for (int r = 0; r < 4096 && !cnt.error && len > 0; ++r) {
      ++stamp;
      cnt.nondelaunay = 0;
      cnt.inverted = 0;
      const int* wl = cur == 1 ? wl1.data() : wl0.data();
      for (unsigned long long i = 0; i < len; ++i) mcl::p_body_classify(V, wl[i], stamp);
      if (cnt.error) break;
      if (cnt.inverted) {
        cnt.error = MCL_ERR_DEGENERATE_INPUT;  // the rounds leave every face positive
        break;
      }
      if (!cnt.nondelaunay) break;
      const int next = cur == 0 ? 1 : 0;
      cnt.lcount[next] = 0;
      for (unsigned long long i = 0; i < cnt.nondelaunay; ++i) mcl::p_body_flip(V, clist[i], stamp, next);
      cur = next;
      len = cnt.lcount[next];
    }
  }
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 4;
  const int32_t head[2] = {(int32_t)cnt.error, (int32_t)cnt.reinserted};
  wr(out, head, 2);
  wr(out, pos.data(), n);
  wr(out, ev.data(), E);
  wr(out, en.data(), E);
  wr(out, eo.data(), E);
  fclose(out);
  return 0;
}
