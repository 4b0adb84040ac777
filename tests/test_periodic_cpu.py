"""The engine's periodic (torus) offset algebra (mcleap_gb300/csrc/periodic.cuh)
on the CPU: a sequential Lawson harness built from the engine's own headers
moves points of a periodic Delaunay mesh, wraps them into the domain, flips,
and must land on the oracle's periodic Delaunay triangulation of the new
positions, edge offsets included."""
import os
import subprocess

import numpy as np
import pytest

from oracle import periodic as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
L = 8192.0


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("periodic") / "periodic_lawson")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "mcleap_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "periodic_lawson.cpp"), "-o", exe], check=True)
    return exe


def torus_points(n, seed):
    rng = np.random.default_rng(seed)
    x0 = P.domain_origin(L)
    p = (x0 + rng.random((n, 2)) * L).astype(np.float32)
    p[p >= x0 + L] = np.nextafter(np.float32(x0 + L), np.float32(0))
    return p


def wrap_rule(q):
    """The engine's wrap of a moved coordinate into [2L, 3L) (float32 steps)."""
    lo, hi = np.float32(2 * L), np.float32(3 * L)
    q = q.astype(np.float32).copy()
    up = q >= hi
    q[up] = q[up] - np.float32(L)
    dn = q < lo
    r = (q[dn] + np.float32(L)).astype(np.float32)
    r[r >= hi] = lo
    q[dn] = r
    return q


def run(harness, tmp_path, moved, ev, en, eo):
    n, E = len(moved), len(ev)
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(src, "wb") as f:
        f.write(np.array([n, E], np.int32).tobytes() + np.float32(L).tobytes())
        for a in (moved.astype(np.float32), ev.astype(np.int32), en.astype(np.int32), eo.astype(np.uint32)):
            f.write(np.ascontiguousarray(a).tobytes())
    subprocess.run([harness, src, dst], check=True)
    raw = open(dst, "rb").read()
    head = np.frombuffer(raw[:20], np.int32)
    o = 20
    pos = np.frombuffer(raw[o:o + 8 * n], np.float32).reshape(n, 2)
    o += 8 * n
    ev2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    en2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    eo2 = np.frombuffer(raw[o:o + 4 * E], np.uint32)
    status, flips, wrapped, before, after = (int(x) for x in head)
    return dict(status=status, flips=flips, wrapped=wrapped, before=before, after=after), pos, ev2, en2, eo2


def settle(xy, d, ev, eo, drift):
    """Reset to the common drift the moves of the vertices of faces the move
    would turn (or nearly turn) over, until none would: the harness only
    flips, it does not untangle."""
    B, C, X1 = P.eo_unpack(eo)
    D = B + X1
    a, b, c, dd = (ev[:, k] for k in range(4))
    d = d.copy()

    def orient(p, q, r):
        return (q[:, 0] - p[:, 0]) * (r[:, 1] - p[:, 1]) - (q[:, 1] - p[:, 1]) * (r[:, 0] - p[:, 0])

    tol = 1e-6 * L * L / len(xy)
    for _ in range(100):
        p = (xy + d).astype(np.float32).astype(np.float64)
        pa, pb, pc, pd = p[a], p[b] + B * L, p[c] + C * L, p[dd] + D * L
        bad = (orient(pa, pb, pc) <= tol) | (orient(pb, pa, pd) <= tol)
        if not bad.any():
            return d
        d[np.unique(ev[bad])] = drift
    raise RuntimeError("settle did not converge")


def face_offsets_consistent(ev, en, eo):
    """t(h) + t(next h) + t(prev h) = 0 around every face, x(h) = t(h) + t(next h)."""
    B, C, X1 = P.eo_unpack(eo)
    h = np.arange(2 * len(ev))
    e, s = h // 2, h % 2

    def t_of(hh):
        return np.where((hh % 2 == 1)[:, None], -B[hh // 2], B[hh // 2])

    nx = np.where(s == 0, en[e, 0], en[e, 2])
    pv = np.where(s == 0, en[e, 1], en[e, 3])
    x = np.where((s == 0)[:, None], C[e], X1[e])
    return (t_of(h) + t_of(nx) + t_of(pv) == 0).all() and (x == t_of(h) + t_of(nx)).all()


@pytest.mark.parametrize("n,sigma,shift,seed", [
    (3000, 0.05, (0.0, 0.0), 1),      # jitter: a few flips, a few wraps at the sides
    (3000, 0.05, (0.37, -0.61), 2),   # plus a drift: every point near a side wraps
    (5000, 0.12, (-0.9, 0.45), 3),
])
def test_lawson_with_wraps_matches_oracle(harness, tmp_path, n, sigma, shift, seed):
    xy = torus_points(n, seed)
    ev, en, eo = P.periodic_mesh(xy, L)
    h = L / np.sqrt(n)
    rng = np.random.default_rng(100 + seed)
    drift = (np.array(shift) * h).astype(np.float32)
    d = (rng.normal(0, sigma * h, (n, 2)) + drift).astype(np.float32)
    d = settle(xy, d, ev, eo, drift)
    assert (d != drift).any(1).mean() > 0.7
    moved = (xy + d).astype(np.float32)
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, moved, ev, en, eo)
    assert st["status"] == 0, st
    assert st["before"] == 0 and st["after"] == 0, st
    assert np.array_equal(pos, wrap_rule(moved))
    assert st["wrapped"] > 0 and st["flips"] > 0
    assert face_offsets_consistent(ev2, en2, eo2)
    assert np.array_equal(P.mesh_edges(ev2, eo2), P.periodic_edges(pos, L))


def test_identity_step_changes_nothing(harness, tmp_path):
    xy = torus_points(2000, 9)
    ev, en, eo = P.periodic_mesh(xy, L)
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, ev, en, eo)
    assert st == dict(status=0, flips=0, wrapped=0, before=0, after=0)
    assert np.array_equal(ev2, ev) and np.array_equal(en2, en) and np.array_equal(eo2, eo)


def test_whole_period_translation_is_a_relabelling(harness, tmp_path):
    """Moving every point by exactly one period wraps all of them back: the
    positions and the mesh come back unchanged, through n wraps."""
    xy = torus_points(2000, 11)
    ev, en, eo = P.periodic_mesh(xy, L)
    moved = (xy.astype(np.float64) + np.array([L, 0.0])).astype(np.float32)
    assert np.array_equal(moved.astype(np.float64), xy.astype(np.float64) + np.array([L, 0.0]))
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, moved, ev, en, eo)
    assert st["status"] == 0 and st["wrapped"] == 2000 and st["flips"] == 0
    assert np.array_equal(pos, xy) and np.array_equal(eo2, eo)
