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
from oracle import oracle as O
from oracle import periodic as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RING = 8  # ring slots of the harness (kRing)
FRNN = 64  # FRNN slots of the harness (kFrnn)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("periodic") / "periodic_step")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "mcleap_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "periodic_step.cpp"), "-o", exe], check=True)
    return exe


def run(harness, tmp_path, pos, d, ev, en, eo, r=None):
    n, E = len(pos), len(ev)
    r = 2.5 * L / np.sqrt(n) if r is None else r
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(src, "wb") as f:
        f.write(np.array([n, E], np.int32).tobytes() + np.float32(L).tobytes() + np.float32(r).tobytes())
        for a in (pos.astype(np.float32), d.astype(np.float32), ev.astype(np.int32), en.astype(np.int32),
                  eo.astype(np.uint32)):
            f.write(np.ascontiguousarray(a).tobytes())
    subprocess.run([harness, src, dst], check=True)
    raw = open(dst, "rb").read()
    head = [int(x) for x in np.frombuffer(raw[:52], np.int32)]
    o = 52
    pos2 = np.frombuffer(raw[o:o + 8 * n], np.float32).reshape(n, 2)
    o += 8 * n
    ev2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    en2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    eo2 = np.frombuffer(raw[o:o + 4 * E], np.uint32)
    o += 4 * E
    ring = np.frombuffer(raw[o:o + 4 * RING * n], np.int32).reshape(RING, n)
    o += 4 * RING * n
    offs = np.frombuffer(raw[o:o + RING * n], np.uint8).reshape(RING, n)
    o += RING * n
    closest = np.frombuffer(raw[o:o + 4 * n], np.int32)
    o += 4 * n
    frnn = np.frombuffer(raw[o:o + 4 * FRNN * n], np.int32).reshape(FRNN, n)
    o += 4 * FRNN * n
    foffs = np.frombuffer(raw[o:o + FRNN * n], np.uint8).reshape(FRNN, n)
    o += FRNN * n
    frnn_truncated = int(np.frombuffer(raw[o:o + 4], np.int32)[0])
    run.queries = (ring, offs, closest)
    run.frnn = (frnn, foffs, frnn_truncated, np.float32(r))
    st = dict(zip(["status", "flips", "wrapped", "inverted", "rounds", "nonpositive_after", "truncated", "reverted",
                   "revert_passes", "behind", "substep_arrivals", "classified", "reinserted"], head))
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
    assert st["reverted"] == 0 and st["revert_passes"] == 0 and st["behind"] == 0
    assert np.array_equal(pos, torus_wrap(xy + d))
    assert st["wrapped"] > 0 and st["flips"] > 0 and st["rounds"] >= 2
    # rounds after the first classify only the edges around the last flips
    assert st["classified"] < len(ev) + 5 * st["flips"]
    assert torus_faces_consistent(ev2, en2, eo2)
    assert np.array_equal(P.mesh_edges(ev2, eo2), P.periodic_edges(pos, L))


def test_identity_step_changes_nothing(harness, tmp_path):
    xy = torus_points(2000, 9)
    ev, en, eo = P.periodic_mesh(xy, L)
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, np.zeros_like(xy), ev, en, eo)
    assert {k: st[k] for k in ("status", "flips", "wrapped", "inverted", "rounds", "nonpositive_after")} == dict(
        status=0, flips=0, wrapped=0, inverted=0, rounds=1, nonpositive_after=0)
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


def check_step(st, xy, d, pos, ev, en, eo):
    """Every point at its target or counted behind; the mesh valid and the
    periodic Delaunay triangulation of where the points are."""
    assert st["status"] == 0 and st["nonpositive_after"] == 0, st
    at = (pos == torus_wrap(xy + d)).all(1)
    assert (~at).sum() == st["behind"]
    assert torus_faces_consistent(ev, en, eo)
    assert np.array_equal(P.mesh_edges(ev, eo), P.periodic_edges(pos, L))


def test_a_face_turned_over_is_refused_then_resumed(harness, tmp_path):
    """A vertex jumping across its neighbour is sent back; sub-steps (half of
    what it still owes, the last one all of it) or, failing those, removal and
    reinsertion take it to its target."""
    xy = torus_points(2000, 12)
    ev, en, eo = P.periodic_mesh(xy, L)
    a, b = ev[0, 0], ev[0, 1]
    d = np.zeros_like(xy)
    d[a] = 2.0 * (xy[b] - xy[a] + eo_b_vec(eo[0]) * L)   # a jumps across b
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, d, ev, en, eo)
    assert st["inverted"] > 0 and st["reverted"] >= 1, st
    check_step(st, xy, d, pos, ev2, en2, eo2)
    assert st["behind"] == 0 and st["substep_arrivals"] + st["reinserted"] == 1


@pytest.mark.parametrize("sigma,shift,seed", [(0.1, (0.0, 0.0), 51), (0.2, (0.4, -0.3), 52), (0.3, (0.0, 0.0), 53),
                                              (1.0, (0.3, 0.3), 55)])
def test_tangling_moves_all_arrive(harness, tmp_path, sigma, shift, seed):
    """Unsettled random moves: the farthest-moved vertex of each turned face
    goes back (repeatedly, until no face is turned), sub-steps bring most of
    them to their targets, and the rest are removed and reinserted there; the
    result is the periodic Delaunay triangulation of the moved points."""
    n = 4000
    xy = torus_points(n, seed)
    ev, en, eo = P.periodic_mesh(xy, L)
    h = L / np.sqrt(n)
    d = (np.random.default_rng(seed).normal(0, sigma * h, (n, 2)) + np.array(shift) * h).astype(np.float32)
    st, pos, ev2, en2, eo2 = run(harness, tmp_path, xy, d, ev, en, eo)
    assert st["inverted"] > 0 and st["reverted"] > 0 and st["revert_passes"] >= 2, st
    check_step(st, xy, d, pos, ev2, en2, eo2)
    assert st["substep_arrivals"] > 0 and st["reinserted"] > 0 and st["behind"] == 0


def eo_b_vec(w):
    w = int(w)
    return np.array([(w & 15) - 8, ((w >> 4) & 15) - 8], np.float32)


# -- the library's host side of the periodic meshes (no device work) -------------------

@pytest.fixture(scope="module")
def lib():
    from mcleap_gb300 import _lib
    from mcleap_gb300 import build as B

    B.build()
    return _lib


def test_from_planar_equals_the_oracle_mesh(lib):
    """The host conversion behind mcl_periodic_build, fed the oracle's planar
    triangulation of the 3 x 3 cover, gives the oracle's periodic mesh, edge
    numbering included."""
    from mcleap_gb300 import periodic as MP

    n = 2500
    xy = torus_points(n, 21)
    pos, v, he, t = O.Mesh.build(P.cover(xy, L), exact=True).aos()
    row = np.arange(len(pos)) - 4
    vpoint = np.where(row >= 0, row % n, -1).astype(np.int32)
    vcopy = np.where(row >= 0, row // n, -1).astype(np.int32)
    keep = [np.ascontiguousarray(a) for a in (pos, v, he, t)]
    view = lib.AosView(*(lib.ptr(a) for a in keep), len(pos), len(he), len(t))
    ev, en, eo = MP.from_planar(view, vpoint, vcopy, n)
    ev0, en0, eo0 = P.periodic_mesh(xy, L)
    assert np.array_equal(ev, ev0) and np.array_equal(en, en0) and np.array_equal(eo, eo0)
    assert np.array_equal(MP.canonical_edges(ev, eo), P.periodic_edges(xy, L))


def test_from_planar_refuses_a_sparse_cover(lib):
    """Too few points for the period: some face would use two copies of one point."""
    from mcleap_gb300 import periodic as MP

    n = 3
    xy = torus_points(n, 5)
    pos, v, he, t = O.Mesh.build(P.cover(xy, L), exact=True).aos()
    row = np.arange(len(pos)) - 4
    keep = [np.ascontiguousarray(a) for a in (pos, v, he, t)]
    view = lib.AosView(*(lib.ptr(a) for a in keep), len(pos), len(he), len(t))
    with pytest.raises(lib.McleapError) as err:
        MP.from_planar(view, np.where(row >= 0, row % n, -1), np.where(row >= 0, row // n, -1), n)
    assert err.value.code == lib.MCL_ERR_DEGENERATE_INPUT


def test_periodic_arguments_are_checked_before_device_work(lib):
    import ctypes as C

    h = C.c_void_p()
    pts = torus_points(100, 1)
    L_ = lib.lib()
    assert L_.mcl_periodic_build(lib.ptr(pts), 100, 1000.0, C.byref(h)) == lib.MCL_ERR_INVALID_ARGUMENT
    bad = pts.copy()
    bad[7] = (1.0, 1.0)
    assert L_.mcl_periodic_build(lib.ptr(bad), 100, L, C.byref(h)) == lib.MCL_ERR_DEGENERATE_INPUT
    ev = np.zeros((300, 4), np.int32)
    en = np.zeros((300, 4), np.int32)
    eo = np.full(300, 0x888888, np.uint32)
    ev[5, 2] = 100  # a vertex id out of range
    rc = L_.mcl_periodic_create(lib.ptr(pts), 100, L, lib.ptr(ev), lib.ptr(en), lib.ptr(eo), C.byref(h))
    assert rc == lib.MCL_ERR_INVALID_ARGUMENT and b"ev out of range" in L_.mcl_last_error()
    ev[5, 2] = 0
    eo[9] = 0x8A8888  # an offset of +2
    rc = L_.mcl_periodic_create(lib.ptr(pts), 100, L, lib.ptr(ev), lib.ptr(en), lib.ptr(eo), C.byref(h))
    assert rc == lib.MCL_ERR_INVALID_ARGUMENT and b"eo out of range" in L_.mcl_last_error()
    for name in ("mcl_periodic_destroy",):
        assert getattr(L_, name)(None) == lib.MCL_OK
    st = lib.StepStats()
    assert L_.mcl_periodic_step(None, None, None, C.byref(st), None) == lib.MCL_ERR_INVALID_ARGUMENT
    assert L_.mcl_periodic_one_ring(None, 8, 0, None, None, None, None) == lib.MCL_ERR_INVALID_ARGUMENT
    assert L_.mcl_periodic_closest(None, 8, 0, None, None, None, None) == lib.MCL_ERR_INVALID_ARGUMENT
    assert L_.mcl_periodic_frnn(None, 1.0, 8, 0, None, None, None, None) == lib.MCL_ERR_INVALID_ARGUMENT


def band_cover(xy, band):
    """The cover mcl_periodic_build triangulates: the points (copy 4), then
    their translates within `band` of the domain, copies 0..3 and 5..8."""
    lo, hi = 2 * L, 3 * L
    pts, point, copy = [], [], []
    for k in [4, 0, 1, 2, 3, 5, 6, 7, 8]:
        ox, oy = k % 3 - 1, k // 3 - 1
        q = (xy.astype(np.float64) + np.array([ox * L, oy * L])).astype(np.float32)
        inside = ((q >= lo - band) & (q < hi + band)).all(1)
        pts.append(q[inside])
        point.append(np.nonzero(inside)[0])
        copy.append(np.full(inside.sum(), k))
    return np.concatenate(pts), np.concatenate(point), np.concatenate(copy)


@pytest.mark.parametrize("n,seed", [(500, 1), (800, 31), (6000, 32)])
def test_band_cover_build_equals_the_oracle_mesh(lib, n, seed):
    """mcl_periodic_build's host logic with the oracle's exact builder standing
    in for the GPU build (equal edge sets, shown by the GPU parity tests): the
    quarter-period band cover, Morton-sorted like mcl_mesh_build, ids recovered
    by position, converted by the library, gives the oracle's periodic mesh."""
    from mcleap_gb300 import periodic as MP

    xy = torus_points(n, seed)
    cp, cpoint, ccopy = band_cover(xy, 0.25 * L)
    assert len(cp) < 2.5 * n
    srt = O.morton_sort(cp)
    pos, v, he, t = O.Mesh.build(srt, exact=True).aos()
    where = {(a.tobytes()): i for i, a in enumerate(cp)}
    idx = np.array([where[p.tobytes()] for p in pos[4:]])
    vpoint = np.concatenate([[-1] * 4, cpoint[idx]]).astype(np.int32)
    vcopy = np.concatenate([[-1] * 4, ccopy[idx]]).astype(np.int32)
    keep = [np.ascontiguousarray(a) for a in (pos, v, he, t)]
    view = lib.AosView(*(lib.ptr(a) for a in keep), len(pos), len(he), len(t))
    ev, en, eo = MP.from_planar(view, vpoint, vcopy, n)
    ev0, en0, eo0 = P.periodic_mesh(xy, L)
    assert np.array_equal(ev, ev0) and np.array_equal(en, en0) and np.array_equal(eo, eo0)


def ring_reference(edges, n):
    """Directed (neighbour, ox, oy) sets of every vertex from canonical edges."""
    out = [set() for _ in range(n)]
    for u, v, ox, oy in edges:
        out[u].add((v, ox, oy))
        out[v].add((u, -ox, -oy))
    return out


def test_ring_and_closest_on_a_stepped_mesh(harness, tmp_path):
    """One-ring (clockwise from the smallest neighbour, truncated at RING - 1)
    and closest neighbour on the torus, by the query bodies, after a step."""
    n = 3000
    xy = torus_points(n, 41)
    ev, en, eo = P.periodic_mesh(xy, L)
    h = L / np.sqrt(n)
    drift = np.float32([0.45 * h, -0.2 * h])
    d = (np.random.default_rng(4).normal(0, 0.05 * h, (n, 2)) + drift).astype(np.float32)
    d = torus_settle(xy, d, ev, eo, drift)
    st, pos, ev2, _, eo2 = run(harness, tmp_path, xy, d, ev, en, eo)
    assert st["status"] == 0 and st["wrapped"] > 0
    ring, offs, closest = run.queries
    want = ring_reference(P.periodic_edges(pos, L), n)
    deg = np.array([len(w) for w in want])
    assert st["truncated"] == int((deg > RING - 1).sum()) > 0
    p64 = pos.astype(np.float64)
    for v in range(n):
        cnt = ring[0, v]
        assert cnt == min(deg[v], RING - 1)
        nb = ring[1:cnt + 1, v]
        ob = offs[1:cnt + 1, v].astype(np.int64)
        o = np.stack([(ob & 15) - 8, ((ob >> 4) & 15) - 8], 1)
        got = {(int(a), int(b), int(c)) for a, (b, c) in zip(nb, o)}
        assert got <= want[v] and (cnt < deg[v] or got == want[v])
        # starts at the smallest (id, offset) of the whole ring, turns clockwise
        if cnt == deg[v]:
            assert (nb[0], ob[0]) == min(zip(nb, ob))
        q = p64[nb] + o * L - p64[v]
        ang = np.arctan2(q[:, 1], q[:, 0])
        turn = np.mod(ang[1:] - ang[:-1], 2 * np.pi)
        assert (turn > np.pi).all()  # each step turns clockwise by less than pi
        # closest among the ring, by the float formula, smallest id among equals
        dx = (pos[v, 0] - (pos[nb, 0] + (o[:, 0] * L).astype(np.float32))).astype(np.float32)
        dy = (pos[v, 1] - (pos[nb, 1] + (o[:, 1] * L).astype(np.float32))).astype(np.float32)
        dd = (dx * dx + dy * dy).astype(np.float32)
        best = nb[np.lexsort((nb, dd))[0]]
        assert closest[v] == best


def frnn_brute(pos, r):
    """(neighbour, ox, oy) sets within r on the torus by the reference's float
    squared distance, over the nine copies of every point."""
    n = len(pos)
    r2 = np.float32(r) * np.float32(r)
    out = [set() for _ in range(n)]
    for oy in (-1, 0, 1):
        for ox in (-1, 0, 1):
            q = (pos + np.float32([ox * L, oy * L])).astype(np.float32)
            for a in range(0, n, 500):
                dx = (pos[a:a + 500, None, 0] - q[None, :, 0]).astype(np.float32)
                dy = (pos[a:a + 500, None, 1] - q[None, :, 1]).astype(np.float32)
                d2 = (dx * dx + dy * dy).astype(np.float32)
                ii, jj = np.nonzero(d2 <= r2)
                for i, j in zip(ii + a, jj):
                    if i != j:
                        out[i].add((int(j), ox, oy))
    return out


@pytest.mark.parametrize("rf", [1.5, 3.0])
def test_frnn_on_a_stepped_mesh(harness, tmp_path, rf):
    """getFRNN on the torus by the query body: every other point with a copy
    within r, ascending ids, with the copy offsets; equal to brute force."""
    n = 3000
    xy = torus_points(n, 61)
    ev, en, eo = P.periodic_mesh(xy, L)
    h = L / np.sqrt(n)
    drift = np.float32([-0.3 * h, 0.55 * h])
    d = (np.random.default_rng(6).normal(0, 0.05 * h, (n, 2)) + drift).astype(np.float32)
    st, pos, *_ = run(harness, tmp_path, xy, d, ev, en, eo, r=rf * h)
    assert st["status"] == 0 and st["wrapped"] > 0
    frnn, foffs, trunc, r = run.frnn
    assert trunc == 0
    want = frnn_brute(pos, r)
    for i in range(n):
        cnt = frnn[0, i]
        ids = frnn[1:cnt + 1, i]
        ob = foffs[1:cnt + 1, i].astype(np.int64)
        assert (np.diff(ids) > 0).all()
        got = {(int(a), int((b & 15) - 8), int(((b >> 4) & 15) - 8)) for a, b in zip(ids, ob)}
        assert got == want[i], i


def test_many_steps_of_advection_with_drift(harness, tmp_path):
    """Twenty steps of Taylor-Green advection plus a drift on the torus (the
    periodic benchmark's motion): points cross the sides every step, and after
    every step the mesh is the oracle's periodic triangulation of the moved points."""
    n = 3000
    pos = torus_points(n, 71)
    ev, en, eo = P.periodic_mesh(pos, L)
    h = L / np.sqrt(n)
    wrapped = 0
    for k in range(20):
        q = (pos.astype(np.float64) - 2 * L) / L
        u = np.sin(2 * np.pi * q[:, 0]) * np.cos(2 * np.pi * q[:, 1]) + 0.3
        v = -np.cos(2 * np.pi * q[:, 0]) * np.sin(2 * np.pi * q[:, 1]) + 0.2
        d = (np.stack([u, v], 1) * 0.5 * h).astype(np.float32)
        st, pos2, ev, en, eo = run(harness, tmp_path, pos, d, ev, en, eo)
        assert st["status"] == 0 and st["behind"] == 0 and st["nonpositive_after"] == 0, (k, st)
        assert np.array_equal(pos2, torus_wrap(pos + d))
        assert np.array_equal(P.mesh_edges(ev, eo), P.periodic_edges(pos2, L)), k
        wrapped += st["wrapped"]
        pos = pos2.copy()
        ev, en, eo = ev.copy(), en.copy(), eo.copy()
    assert wrapped > 20 * 10
    assert torus_faces_consistent(ev, en, eo)
    assert np.array_equal(P.mesh_edges(ev, eo), P.periodic_edges(pos, L))


@pytest.fixture(scope="module")
def reinsert_harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("reinsert") / "periodic_reinsert")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "mcleap_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "periodic_reinsert.cpp"), "-o", exe], check=True)
    return exe


def run_reinsert(exe, tmp_path, pos, ev, en, eo, verts, targets, rounds=False):
    n, E, k = len(pos), len(ev), len(verts)
    src, dst = str(tmp_path / "rin.bin"), str(tmp_path / "rout.bin")
    with open(src, "wb") as f:
        f.write(np.array([n, E], np.int32).tobytes() + np.float32(L).tobytes() + np.int32(k).tobytes())
        for a in (pos.astype(np.float32), ev.astype(np.int32), en.astype(np.int32), eo.astype(np.uint32),
                  np.asarray(verts, np.int32), np.asarray(targets, np.float32)):
            f.write(np.ascontiguousarray(a).tobytes())
    mode = [] if not rounds else (["rounds"] if rounds is True else [f"rounds:{int(rounds)}"])
    subprocess.run([exe, src, dst] + mode, check=True)
    raw = open(dst, "rb").read()
    status, reinserted = (int(x) for x in np.frombuffer(raw[:8], np.int32))
    o = 8
    pos2 = np.frombuffer(raw[o:o + 8 * n], np.float32).reshape(n, 2)
    o += 8 * n
    ev2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    en2 = np.frombuffer(raw[o:o + 16 * E], np.int32).reshape(E, 4)
    o += 16 * E
    eo2 = np.frombuffer(raw[o:o + 4 * E], np.uint32)
    return status, reinserted, pos2, ev2, en2, eo2


@pytest.mark.parametrize("rounds", [False, True], ids=["one-thread", "rounds"])
def test_reinsertion_inside_a_face_on_an_edge_and_onto_a_taken_spot(reinsert_harness, tmp_path, rounds):
    """Removal and reinsertion, by the one-thread pass and by the launch's
    claim-based rounds (then flips from the edges they rewrote): a target
    inside a face (1 -> 3 split), a target exactly on an edge (2 -> 4 split,
    three collinear points afterwards) and a target that another point
    occupies (the vertex goes back where it was); the mesh is the oracle's
    triangulation afterwards."""
    n = 2000
    xy = torus_points(n, 81)
    h = L / np.sqrt(n)
    X = Y = np.float32(2.5 * L)
    dl = np.float32(np.round(0.25 * h))
    xy[0] = (X, Y)
    xy[1] = (X + 2 * dl, Y)
    ev, en, eo = P.periodic_mesh(xy, L)
    edges = P.periodic_edges(xy, L)
    assert ((edges[:, 0] == 0) & (edges[:, 1] == 1)).any()
    mid = np.float32([X + dl, Y])
    far = np.argsort(((xy - mid) ** 2).sum(1))[::-1]
    v_edge, v_taken, v_face = int(far[0]), int(far[1]), int(far[2])
    t_face = np.float32([2.25 * L + 0.123, 2.75 * L - 0.456])
    targets = [mid, xy[5], t_face]
    st, re, pos, ev2, en2, eo2 = run_reinsert(reinsert_harness, tmp_path, xy, ev, en, eo,
                                              [v_edge, v_taken, v_face], targets, rounds)
    assert st == 0 and re == 2
    assert (pos[v_edge] == mid).all() and (pos[v_taken] == xy[v_taken]).all() and (pos[v_face] == t_face).all()
    assert torus_faces_consistent(ev2, en2, eo2)
    got = P.mesh_edges(ev2, eo2)
    assert np.array_equal(got, P.periodic_edges(pos, L))
    # the split edge: 0 - v - 1 on one line
    assert not ((got[:, 0] == 0) & (got[:, 1] == 1)).any()
    assert ((got[:, 0] == min(0, v_edge)) & (got[:, 1] == max(0, v_edge))).any()
    assert ((got[:, 0] == min(1, v_edge)) & (got[:, 1] == max(1, v_edge))).any()


@pytest.mark.parametrize("rounds", [False, True], ids=["one-thread", "rounds"])
def test_refused_removal_leaves_the_torus_delaunay(reinsert_harness, tmp_path, rounds):
    """Tiny tori, where a vertex's star can hold two copies of one neighbour:
    the removal (one-thread pass or the launch's rounds) then refuses (the
    vertex stays where it was), some of them after spoke flips.  Whatever happens, a call that returns OK leaves
    the oracle's triangulation of the final positions (a refusal is counted,
    never a silently non-Delaunay mesh); a failure is reported."""
    outcomes = {"reinserted": 0, "refused": 0, "error": 0}
    for n in (3, 4, 5, 6, 8):
        for seed in range(8):
            xy = torus_points(n, 1000 + 37 * n + seed)
            try:
                ev, en, eo = P.periodic_mesh(xy, L)
            except ValueError:
                continue  # too few points for the period: no torus triangulation
            rng = np.random.default_rng(seed)
            for v in range(n):
                t = (2 * L + rng.random(2) * L).astype(np.float32)
                st, re, pos, ev2, en2, eo2 = run_reinsert(reinsert_harness, tmp_path, xy, ev, en, eo, [v], [t],
                                                          rounds)
                if st != 0:
                    outcomes["error"] += 1
                    continue
                assert torus_faces_consistent(ev2, en2, eo2), (n, seed, v)
                assert np.array_equal(P.mesh_edges(ev2, eo2), P.periodic_edges(pos, L)), (n, seed, v)
                if re == 1:
                    assert (pos[v] == t).all()
                    outcomes["reinserted"] += 1
                else:
                    assert (pos[v] == xy[v]).all()
                    outcomes["refused"] += 1
    assert outcomes["refused"] > 0 and outcomes["reinserted"] > 0, outcomes


def test_many_reinsertions_in_rounds_do_not_depend_on_order(reinsert_harness, tmp_path):
    """Two hundred vertices removed and reinserted far from where they were by
    the launch's claim-based rounds (contested stars and faces, several
    rounds), every phase taken in three different orders: the same positions
    and the oracle's triangulation each time."""
    n = 4000
    xy = torus_points(n, 91)
    ev, en, eo = P.periodic_mesh(xy, L)
    rng = np.random.default_rng(92)
    verts = np.sort(rng.choice(n, 200, replace=False))
    targets = (2 * L + rng.random((len(verts), 2)) * L).astype(np.float32)
    results = []
    for seed in (1, 2, 3):
        st, re, pos, ev2, en2, eo2 = run_reinsert(reinsert_harness, tmp_path, xy, ev, en, eo, verts, targets, seed)
        assert st == 0 and re == len(verts), (st, re)
        assert (pos[verts] == targets).all()
        assert torus_faces_consistent(ev2, en2, eo2)
        edges = P.mesh_edges(ev2, eo2)
        assert np.array_equal(edges, P.periodic_edges(pos, L))
        results.append((pos, edges))
    assert all(np.array_equal(results[0][0], r[0]) and np.array_equal(results[0][1], r[1]) for r in results[1:])
