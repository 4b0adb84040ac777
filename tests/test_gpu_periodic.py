"""Periodic (flat torus) meshes on the GPU against the torus oracle: the exact
build (edge numbering included) and kinetic steps with wraps and flips."""
import numpy as np
import pytest

from helpers import TORUS_L as L
from helpers import torus_faces_consistent, torus_points, torus_settle, torus_wrap
from oracle import periodic as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import torch

    import mcleap_gb300 as M
    from mcleap_gb300 import build as B

    assert torch.cuda.is_available()
    B.build()
    M.lib()
    return M


def cuda(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.mark.parametrize("n,seed", [(500, 1), (20000, 2)])
def test_build_is_the_oracle_mesh(M, n, seed):
    xy = torus_points(n, seed)
    pt = M.PeriodicTriangulation(xy, L)
    assert (pt.n, pt.E, pt.L) == (n, 3 * n, L)
    pos, ev, en, eo = pt.download()
    assert np.array_equal(pos, xy)
    ev0, en0, eo0 = P.periodic_mesh(xy, L)
    assert np.array_equal(ev, ev0) and np.array_equal(en, en0) and np.array_equal(eo, eo0)


def test_identity_step_changes_nothing(M):
    xy = torus_points(3000, 4)
    pt = M.PeriodicTriangulation(xy, L)
    before = pt.download()
    st = pt.step(cuda(np.zeros_like(xy)))
    assert st["status"] == 0 and st["lawson_flips"] == 0 and st["wrapped"] == 0 and st["lawson_rounds"] == 1
    after = pt.download()
    assert all(np.array_equal(a, b) for a, b in zip(before, after))


def test_steps_with_wraps_match_the_oracle(M):
    n = 20000
    xy = torus_points(n, 3)
    pt = M.PeriodicTriangulation(xy, L)
    h = L / np.sqrt(n)
    rng = np.random.default_rng(7)
    pos = xy
    wrapped = flips = 0
    for shift in [(0.0, 0.0), (0.37, -0.61), (-0.9, 0.45), (0.2, 0.2)]:
        _, ev, _, eo = pt.download()
        drift = (np.array(shift) * h).astype(np.float32)
        d = (rng.normal(0, 0.08 * h, (n, 2)) + drift).astype(np.float32)
        d = torus_settle(pos, d, ev, eo, drift)
        st = pt.step(cuda(d))
        assert st["status"] == 0 and st["inverted_faces"] == 0 and st["reverted_vertices"] == 0, st
        want = torus_wrap(pos + d)
        pos2, ev2, en2, eo2 = pt.download()
        assert np.array_equal(pos2, want)
        assert torus_faces_consistent(ev2, en2, eo2)
        assert np.array_equal(M.periodic.canonical_edges(ev2, eo2), P.periodic_edges(want, L))
        wrapped += st["wrapped"]
        flips += st["lawson_flips"]
        pos = want
    assert wrapped > 0 and flips > 0


def test_mesh_from_arrays_steps_like_the_built_one(M):
    n = 3000
    xy = torus_points(n, 5)
    ev, en, eo = P.periodic_mesh(xy, L)
    a = M.PeriodicTriangulation(xy, L)
    b = M.periodic.PeriodicTriangulation.from_arrays(xy, L, ev, en, eo)
    h = L / np.sqrt(n)
    drift = np.float32([0.3 * h, 0.1 * h])
    d = (np.random.default_rng(2).normal(0, 0.05 * h, (n, 2)) + drift).astype(np.float32)
    d = torus_settle(xy, d, ev, eo, drift)
    a.step(cuda(d))
    b.step_host(d)
    assert all(np.array_equal(x, y) for x, y in zip(a.download(), b.download()))


def check_step(M, st, xy, d, pos, ev, en, eo):
    """Every point at its target or counted behind; the mesh valid and the
    periodic Delaunay triangulation of where the points are."""
    assert st["status"] == 0, st
    at = (pos == torus_wrap(xy + d)).all(1)
    assert (~at).sum() == st["reverted_vertices"]
    assert torus_faces_consistent(ev, en, eo)
    assert np.array_equal(M.periodic.canonical_edges(ev, eo), P.periodic_edges(pos, L))


def test_a_face_turned_over_is_refused_then_resumed(M):
    """A vertex jumping across its neighbour is sent back, then taken to its
    target by sub-steps or by removal and reinsertion."""
    xy = torus_points(2000, 12)
    pt = M.PeriodicTriangulation(xy, L)
    _, ev, _, eo = pt.download()
    a, b = ev[0, 0], ev[0, 1]
    B = M.periodic.eo_offsets(eo[:1])[0][0].astype(np.float32)
    d = np.zeros_like(xy)
    d[a] = 2.0 * (xy[b] + B * np.float32(L) - xy[a])
    st = pt.step(cuda(d))
    assert st["inverted_faces"] > 0 and st["reverted_vertices"] == 0, st
    assert st["substep_vertices"] + st["removed_vertices"] == 1
    check_step(M, st, xy, d, *pt.download())


@pytest.mark.parametrize("sigma,shift,seed", [(0.1, (0.0, 0.0), 51), (0.2, (0.4, -0.3), 52), (1.0, (0.3, 0.3), 55)])
def test_tangling_moves_all_arrive(M, sigma, shift, seed):
    n = 4000
    xy = torus_points(n, seed)
    pt = M.PeriodicTriangulation(xy, L)
    h = L / np.sqrt(n)
    d = (np.random.default_rng(seed).normal(0, sigma * h, (n, 2)) + np.array(shift) * h).astype(np.float32)
    st = pt.step(cuda(d))
    assert st["inverted_faces"] > 0 and st["substep_vertices"] > 0 and st["removed_vertices"] > 0, st
    assert st["reverted_vertices"] == 0
    check_step(M, st, xy, d, *pt.download())


def test_ring_and_closest_after_steps(M):
    """One-ring (clockwise from the smallest neighbour) and closest neighbour on
    the torus, after steps with wraps, against the oracle's edges and brute force."""
    import torch

    n = 5000
    xy = torus_points(n, 8)
    pt = M.PeriodicTriangulation(xy, L)
    h = L / np.sqrt(n)
    pos = xy
    for shift in [(0.6, 0.1), (-0.2, -0.7)]:
        _, ev, _, eo = pt.download()
        drift = (np.array(shift) * h).astype(np.float32)
        d = (np.random.default_rng(3).normal(0, 0.05 * h, (n, 2)) + drift).astype(np.float32)
        d = torus_settle(pos, d, ev, eo, drift)
        pt.step(cuda(d))
        pos = torus_wrap(pos + d)
    R = 32
    ring = torch.full((R * n,), -1, dtype=torch.int32, device="cuda")
    offs = torch.zeros((R * n,), dtype=torch.uint8, device="cuda")
    assert pt.oneRing(R, ring, offs) == 0
    closest = torch.full((n,), -2, dtype=torch.int32, device="cuda")
    pt.closestNeighbors(R, ring, offs, closest)
    ring = ring.cpu().numpy().reshape(R, n)
    offs = offs.cpu().numpy().reshape(R, n).astype(np.int64)
    closest = closest.cpu().numpy()
    want = {}
    for u, v, ox, oy in P.periodic_edges(pos, L):
        want.setdefault(u, set()).add((v, ox, oy))
        want.setdefault(v, set()).add((u, -ox, -oy))
    for v in range(n):
        cnt = ring[0, v]
        nb, ob = ring[1:cnt + 1, v], offs[1:cnt + 1, v]
        o = np.stack([(ob & 15) - 8, ((ob >> 4) & 15) - 8], 1)
        assert {(int(a), int(b), int(c)) for a, (b, c) in zip(nb, o)} == want[v] and cnt == len(want[v])
        assert (nb[0], ob[0]) == min(zip(nb, ob))
        # the nearest point on the torus is a Delaunay neighbour
        dx = (pos[v, 0] - (pos[nb, 0] + (o[:, 0] * L).astype(np.float32))).astype(np.float32)
        dy = (pos[v, 1] - (pos[nb, 1] + (o[:, 1] * L).astype(np.float32))).astype(np.float32)
        dd = (dx * dx + dy * dy).astype(np.float32)
        assert closest[v] == nb[np.lexsort((nb, dd))[0]]


def test_frnn_after_steps(M):
    """getFRNN on the torus: every other point with a copy within r, by the
    reference's float distance, ascending ids, against brute force."""
    import torch

    n = 4000
    xy = torus_points(n, 9)
    pt = M.PeriodicTriangulation(xy, L)
    h = L / np.sqrt(n)
    _, ev, _, eo = pt.download()
    drift = np.float32([0.5 * h, 0.5 * h])
    d = (np.random.default_rng(5).normal(0, 0.05 * h, (n, 2)) + drift).astype(np.float32)
    d = torus_settle(xy, d, ev, eo, drift)
    pt.step(cuda(d))
    pos = pt.download()[0]
    F, r = 64, np.float32(2.5 * h)
    out = torch.full((F * n,), -1, dtype=torch.int32, device="cuda")
    offs = torch.zeros((F * n,), dtype=torch.uint8, device="cuda")
    assert pt.getFRNN(F, float(r), out, offs) == 0
    out = out.cpu().numpy().reshape(F, n)
    offs = offs.cpu().numpy().reshape(F, n).astype(np.int64)
    r2 = r * r
    for i in range(0, n, 7):
        cnt = out[0, i]
        got = {(int(a), int((b & 15) - 8), int(((b >> 4) & 15) - 8)) for a, b in zip(out[1:cnt + 1, i], offs[1:cnt + 1, i])}
        want = set()
        for oy in (-1, 0, 1):
            for ox in (-1, 0, 1):
                q = (pos + np.float32([ox * L, oy * L])).astype(np.float32)
                dx = (pos[i, 0] - q[:, 0]).astype(np.float32)
                dy = (pos[i, 1] - q[:, 1]).astype(np.float32)
                for j in np.nonzero((dx * dx + dy * dy).astype(np.float32) <= r2)[0]:
                    if j != i:
                        want.add((int(j), ox, oy))
        assert got == want and (np.diff(out[1:cnt + 1, i]) > 0).all(), i
