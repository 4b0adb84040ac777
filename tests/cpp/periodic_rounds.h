// The periodic step's removal and reinsertion rounds (the p_body_*_par bodies
// of mcleap_gb300/csrc/periodic.cuh), run on the CPU one phase after another
// as the GPU launch runs them: each round's claims for every listed vertex,
// then its verification, then its winners and the next round's list.  The
// edges the rounds rewrote end up on V.wl0 (*lq of them), queued with stamp
// sq; the caller runs the flip rounds from there.  With shuffle != 0 every
// phase takes its vertices in a fresh pseudo-random order (the GPU runs them
// in any order: the result must not depend on it).
#pragma once

#include <algorithm>
#include <random>
#include <vector>

#include "periodic.cuh"

inline void periodic_par_rounds(const mcl::PView& V, int* vh, const std::vector<int>& list, unsigned& stamp,
                                unsigned long long* lq, unsigned shuffle = 0) {
  std::mt19937 rng(shuffle);
  // the order a phase takes the vertices of `l` in
  auto order = [&](const std::vector<int>& l) {
    std::vector<int> o = l;
    if (shuffle) std::shuffle(o.begin(), o.end(), rng);
    return o;
  };
  const int n = V.n;
  std::vector<int> par((size_t)8 * n, 0);
  int* pf = par.data();
  int* pa = pf + 3 * n;
  int* loc = pf + 4 * n;
  int* ps = pf + 5 * n;
  constexpr int kWon = 16;
  for (const int v : list) {
    ps[v] = mcl::kParPending;
    loc[v] = -1;
  }
  const unsigned sq = ++stamp;
  std::vector<int> la = list, lb;
  for (int r = 0; r < mcl::kParRounds && !la.empty() && !V.cnt->error; ++r) {
    const unsigned s = ++stamp;
    for (const int v : order(la)) mcl::p_body_claim_star(V, vh, v, s);
    for (const int v : order(la))
      if (mcl::p_body_holds_star(V, vh, v, s)) ps[v] = mcl::kParPending | kWon;
    lb.clear();
    for (const int v : order(la)) {
      if (ps[v] == (mcl::kParPending | kWon)) mcl::p_body_remove_par(V, vh, v, pf, pa, ps, lq, sq);
      else lb.push_back(v);
    }
    la.swap(lb);
  }
  for (const int v : la) ps[v] = mcl::kParStays;
  la.clear();
  for (const int v : list)
    if (ps[v] == mcl::kParRemoved) la.push_back(v);
  for (int r = 0; !la.empty() && !V.cnt->error; ++r) {
    if (r == mcl::kParRounds) {
      mcl::p_error(V, MCL_ERR_NO_CONVERGENCE, 26);
      break;
    }
    const unsigned s = ++stamp;
    for (const int v : order(la)) mcl::p_body_locate_par(V, vh, v, pa, loc, ps, s);
    for (const int v : order(la))
      if (mcl::p_body_holds_face(V, v, loc, ps, s)) ps[v] |= kWon;
    lb.clear();
    for (const int v : order(la)) {
      if (ps[v] & kWon) {
        ps[v] &= ~kWon;
        mcl::p_body_split_par(V, vh, v, pf, loc, ps, lq, sq);
      } else if (loc[v] == -2) {
        if (ps[v] == mcl::kParBack) {
          mcl::p_error(V, MCL_ERR_DEGENERATE_INPUT, 20);
        } else {
          ps[v] = mcl::kParBack;
          loc[v] = -1;
          lb.push_back(v);
        }
      } else {
        lb.push_back(v);
      }
    }
    la.swap(lb);
  }
}
