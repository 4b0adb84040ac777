"""The periodic (torus) step's kernel bodies (mcleap_gb300/csrc/periodic.cuh)
run serially on the CPU, in the GPU's launch order: points of a periodic
Delaunay mesh move, wrap into the domain, and the flip rounds must land on the
oracle's periodic Delaunay triangulation of the new positions, offsets
included."""
import os
import subprocess

import numpy as np
import pytest

from helpers import TORUS_L as L
from helpers import torus_faces_consistent, torus_points, torus_settle, torus_wrap
from oracle import periodic as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("periodic") / "periodic_step")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "mcleap_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "periodic_step.cpp"), "-o", exe], check=True)
    return exe


def run(harness, tmp_path, pos, d, ev, en, eo):
    n, E = len(pos), len(ev)
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(src, "wb") as f:
        f.write(np.array([n, E], np.int32).tobytes() + np.float32(L).tobytes())
        for a in (pos.astype(np.float32), d.astype(np.float32), ev.astype(np.int32), en.astype(np.int32),
                  eo.astype(np.uint32)):
            f.write(np.ascontiguousarray(a).tobytes())
    subprocess.run([harness, src, dst], check=True)
    raw = open(dst, "rb").read()
    head = [int(x) for x in np.frombuffer(raw[:24], np.int32)]
    o = 24
    pos2 = np.frombuffer(raw[o:o + 8 * n], np.float32).reshape(n, 2)
    o += 8 * n
    ev2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    en2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    eo2 = np.frombuffer(raw[o:o + 4 * E], np.uint32)
    st = dict(zip(["status", "flips", "wrapped", "inverted", "rounds", "nonpositive_after"], head))
    return st, pos2, ev2, en2, eo2


def test_oracle_mesh_is_consistent():
    xy = torus_points(2000, 3)
    ev, en, eo = P.periodic_mesh(xy, L)
    assert ev.shape == (6000, 4) and torus_faces_consistent(ev, en, eo)
    assert np.array_equal(P.mesh_edges(ev, eo), P.periodic_edges(xy, L))


@pytest.mark.parametrize("n,sigma,shift,seed", [
    (3000, 0.05, (0.0, 0.0), 1),      # jitter: flips, and a few wraps at the sides
    (3000, 0.05, (0.37, -0.61), 2),   # plus a drift: every point near a side wraps
    (5000, 0.12, (-0.9, 0.45), 3),
])
def test_step_with_wraps_matches_oracle(harness, tmp_path, n, sigma, shift, seed):
    xy = torus_points(n, seed)
    ev, en, eo = P.periodic_mesh(xy, L)
    h = L / np.sqrt(n)
    rng = np.random.default_rng(100 + seed)
    drift = (np.array(shift) * h).astype(np.float32)
    d = (rng.normal(0, sigma * h, (n, 2)) + drift).astype(np.float32)
    d = torus_settle(xy, d, ev, eo, drift)
    assert (d != drift).any(1).mean() > 0.7
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, d, ev, en, eo)
    assert st["status"] == 0 and st["inverted"] == 0 and st["nonpositive_after"] == 0, st
    assert np.array_equal(pos, torus_wrap(xy + d))
    assert st["wrapped"] > 0 and st["flips"] > 0 and st["rounds"] >= 2
    assert torus_faces_consistent(ev2, en2, eo2)
    assert np.array_equal(P.mesh_edges(ev2, eo2), P.periodic_edges(pos, L))


def test_identity_step_changes_nothing(harness, tmp_path):
    xy = torus_points(2000, 9)
    ev, en, eo = P.periodic_mesh(xy, L)
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, np.zeros_like(xy), ev, en, eo)
    assert st == dict(status=0, flips=0, wrapped=0, inverted=0, rounds=1, nonpositive_after=0)
    assert np.array_equal(ev2, ev) and np.array_equal(en2, en) and np.array_equal(eo2, eo)


def test_whole_period_move_is_a_relabelling(harness, tmp_path):
    """Moving every point by exactly one period wraps all of them back: the
    positions and the mesh come back unchanged, through n wraps."""
    xy = torus_points(2000, 11)
    ev, en, eo = P.periodic_mesh(xy, L)
    d = np.zeros_like(xy)
    d[:, 0] = -L
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, d, ev, en, eo)
    assert st["status"] == 0 and st["wrapped"] == 2000 and st["flips"] == 0
    assert np.array_equal(pos, xy) and np.array_equal(eo2, eo)


def test_a_face_turned_over_is_reported(harness, tmp_path):
    """The periodic step restores Delaunay by flips only: a move that turns a
    face over stops after the first classification, with the count."""
    xy = torus_points(2000, 12)
    ev, en, eo = P.periodic_mesh(xy, L)
    a, b = ev[0, 0], ev[0, 1]
    d = np.zeros_like(xy)
    d[a] = 2.0 * (xy[b] - xy[a] + eo_b_vec(eo[0]) * L)   # a jumps across b
    st, *_ = run(harness, tmp_path, xy, d, ev, en, eo)
    assert st["status"] == 0 and st["inverted"] > 0 and st["flips"] == 0 and st["rounds"] == 1


def eo_b_vec(w):
    w = int(w)
    return np.array([(w & 15) - 8, ((w >> 4) & 15) - 8], np.float32)
