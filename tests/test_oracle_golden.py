"""The oracle against the golden vectors generated from the reference itself.

The fixtures in tests/golden/ come from the reference's own HostTriangulation
and Shewchuk's predicates.c (tests/golden/make_golden.py).  These tests pin the
CPU restatement in oracle/ before the GPU engine is compared with it.
"""
import hashlib
import os
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, name))


def test_exact_predicates_match_shewchuk():
    g = load("predicates.npz")
    assert np.array_equal(O.orient2d(g["orient_pts"], 1), g["orient_exact"])
    assert np.array_equal(O.incircle(g["incircle_pts"], 1), g["incircle_exact"])
    # the set exercises exact zeros and one-ulp perturbations
    assert (g["orient_exact"] == 0).sum() > 100 and (g["incircle_exact"] == 0).sum() > 100


def test_reference_fp64_predicates_restated():
    g = load("predicates.npz")
    assert np.array_equal(O.orient2d(g["orient_pts"], 0), g["orient_ref_fp64"])
    assert np.array_equal(O.incircle(g["incircle_pts"], 0), g["incircle_ref_fp64"])


def _det4(rows):
    # rows: 4 x (x, y, z, 1) as Fractions
    import itertools
    det = Fraction(0)
    for perm in itertools.permutations(range(4)):
        sgn = 1
        p = list(perm)
        for i in range(4):
            for j in range(i + 1, 4):
                if p[i] > p[j]:
                    sgn = -sgn
        term = Fraction(sgn)
        for i in range(4):
            term *= rows[i][p[i]]
        det += term
    return det


def test_sos_incircle_is_the_lifted_perturbation():
    """Symbolic perturbation equals a tiny explicit lift, checked exactly."""
    rng = np.random.default_rng(3)
    cases = 0
    for _ in range(40):
        base = rng.integers(0, 50, 2).astype(np.float32) * 4
        sq = np.array([base, base + [4, 0], base + [4, 4], base + [0, 4]], np.float32)
        perm = rng.permutation(4)
        pts = sq[perm]
        ids = rng.choice(100, 4, replace=False).astype(np.int32)
        s = O.incircle(pts.reshape(1, 8), 2, ids.reshape(1, 4))[0]
        # explicit perturbation: z_i += eps^(rank_i + 1), rank by ascending id
        eps = Fraction(1, 10 ** 12)
        rank = np.argsort(np.argsort(ids))
        rows = []
        for k in range(4):
            x, y = Fraction(float(pts[k, 0])), Fraction(float(pts[k, 1]))
            rows.append([x, y, x * x + y * y + eps ** (int(rank[k]) + 1), Fraction(1)])
        d = _det4(rows)
        assert s == (1 if d > 0 else -1)
        cases += 1
    assert cases == 40


def test_morton_order_matches_reference():
    g = load("test_frnn_1000.npz")
    assert np.array_equal(O.morton_sort(g["points"]), g["sorted_points"])


def test_build_restatement_is_bit_identical():
    g = load("test_frnn_1000.npz")
    m = O.Mesh.build(g["sorted_points"], exact=False)
    pos, v, he, t = m.aos()
    assert np.array_equal(pos, g["pos"]) and np.array_equal(v, g["v"])
    assert np.array_equal(he, g["he"]) and np.array_equal(t, g["t"])


def test_exact_dt_equals_reference_build():
    g = load("test_frnn_1000.npz")
    m = O.Mesh.build(g["sorted_points"], exact=True)
    assert np.array_equal(m.edges(), g["edges"])
    assert m.check(exact=True) == dict(non_delaunay=0, creased=0, inverted_faces=0, zero_faces=0)


def test_one_ring_and_frnn_restated():
    g = load("test_frnn_1000.npz")
    m = O.Mesh.build(g["sorted_points"], exact=False)
    V = len(g["pos"])
    offs = np.concatenate([[0], np.cumsum(g["ring_counts"])])
    for vi in range(V):
        assert np.array_equal(m.one_ring_ref(vi), g["ring_ids"][offs[vi]:offs[vi + 1]])
    for r in (5, 10, 20, 30, 40, 50):
        c, ids = m.frnn_ref_all(float(r))
        assert np.array_equal(c, g[f"frnn_counts_r{r}"])
        assert np.array_equal(ids, g[f"frnn_ids_r{r}"])


@pytest.mark.parametrize("r", [5, 10, 20, 30, 40, 50])
def test_frnn_brute_matches_reference_counts(r):
    # tests/test_frnn.cu:59-94 asserts mesh FRNN counts == brute-force counts
    g = load("test_frnn_1000.npz")
    c, ids = O.frnn_brute(g["pos"], float(r))
    assert np.array_equal(c, g[f"frnn_counts_r{r}"])
    assert np.array_equal(ids, g[f"frnn_ids_r{r}"])


def test_kinetic_restatement_and_dt():
    g = load("kinetic_2000.npz")
    m = O.Mesh.build(g["sorted_points"], exact=False)
    assert np.array_equal(m.edges(), g["edges_step0"])
    for step in (1, 2, 3):
        d = g[f"disp_step{step}"]
        m.move(d)
        k = 0
        while m.untangle_pass() and k < 64:
            k += 1
        m.delonize()
        assert k == int(g[f"ref_untangle_passes_step{step}"])
        h = hashlib.sha256()
        for a in m.aos():
            h.update(np.ascontiguousarray(a).tobytes())
        assert h.hexdigest() == str(g[f"ref_kinetic_digest_step{step}"])
        exact = O.Mesh.build(m.positions()[4:], exact=True)
        assert np.array_equal(exact.edges(), g[f"dt_edges_step{step}"])
