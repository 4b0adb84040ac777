"""GPU parity tests: the CUDA engine through the C ABI against the oracle.

Bar: bit-identical sorted edge sets (the unique Delaunay triangulation with
symbolic perturbation), identical neighbour sets, identical predicate signs.
"""
import os

import numpy as np
import pytest

from helpers import csr_from_table, gaussian_disp, spacing, taylor_green_disp, uniform_points
from oracle import oracle as O

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


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

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def build_pair(M, pts):
    """GPU-built mesh and the oracle's exact triangulation of the same points."""
    p = pts.copy()
    ht = M.HostTriangulation()
    ht.addDelaunayPoints(p)
    return ht, p


def test_build_matches_oracle_and_reference_order(M):
    g = np.load(os.path.join(G, "test_frnn_1000.npz"))
    ht, srt = build_pair(M, g["points"])
    assert np.array_equal(srt, g["sorted_points"])
    assert np.array_equal(ht.edges(), g["edges"])
    for n, seed in ((10, 1), (1000, 2), (20000, 3)):
        pts = uniform_points(n, seed)
        ht, srt = build_pair(M, pts)
        assert np.array_equal(srt, O.morton_sort(pts))
        ref = O.Mesh.build(srt, exact=True)
        assert np.array_equal(ht.edges(), ref.edges())
        assert ht.m_he.shape[0] == 6 * n + 10 and ht.m_t.shape[0] == 2 * n + 2
        # the downloaded AoS is a valid reference-layout mesh
        chk = O.Mesh.from_aos(ht.m_pos, ht.m_v, ht.m_he, ht.m_t, exact=True)
        assert chk.check(exact=True) == dict(non_delaunay=0, creased=0, inverted_faces=0, zero_faces=0)


def test_build_lattice_degenerate(M):
    # cocircular and collinear lattice points: the perturbed triangulation is unique
    xs, ys = np.meshgrid(np.arange(40), np.arange(30))
    pts = (np.stack([xs.ravel(), ys.ravel()], 1) * 8 + 1).astype(np.float32)
    ht, srt = build_pair(M, pts)
    ref = O.Mesh.build(srt, exact=True)
    assert np.array_equal(ht.edges(), ref.edges())


SMALL_CASES = {
    "empty": np.zeros((0, 2), np.float32),
    "one": np.array([[4096.0, 4096.0]], np.float32),
    "two": np.array([[100.0, 200.0], [8000.0, 7000.0]], np.float32),
    "three_collinear": np.array([[10.0, 10.0], [20.0, 20.0], [30.0, 30.0]], np.float32),
    "line": np.stack([np.linspace(1, 8000, 50, dtype=np.float32), np.full(50, 4096, np.float32)], 1),
    "square_lattice": (np.stack(np.meshgrid(np.arange(8), np.arange(8)), -1).reshape(-1, 2) * 1000 + 100)
    .astype(np.float32),
    "box_border": np.array([[0, 0], [0, 8191.5], [8191.5, 0], [8191.5, 8191.5], [0, 4000], [4000, 0]], np.float32),
}


@pytest.mark.parametrize("name", sorted(SMALL_CASES))
def test_small_and_degenerate_inputs(M, name):
    # empty and tiny point sets, collinear and cocircular points, points on the
    # edge of the unit box: build, kinetic steps, a zero step and the queries
    # agree with the oracle's exact triangulation
    import torch

    pts = SMALL_CASES[name]
    ht, srt = build_pair(M, pts)
    assert np.array_equal(ht.edges(), O.Mesh.build(srt, exact=True).edges())
    dt = M.DeviceTriangulation(ht)
    pos = ht.m_pos.copy()
    V = len(pos)
    for k in range(3):
        d = gaussian_disp(V, 300.0, 17 * k + len(pts), clamp_pos=pos)
        st = dt.step(cuda(d))
        assert st["status"] == 0, st
        pos = (pos + d).astype(np.float32)
        dt.transferToHost()
        assert np.array_equal(ht.m_pos, pos)
        if len(pts):
            assert np.array_equal(ht.edges(), O.Mesh.build(pos[4:], exact=True).edges()), k
        else:
            # the bare bounding square: four exactly cocircular corners; the
            # step's Lawson pass picks the diagonal by the symbolic perturbation
            # (the reference's build keeps its construction diagonal)
            assert len(ht.edges()) == 5
    e0 = ht.edges()
    st = dt.step(cuda(np.zeros_like(pos)))
    assert st["status"] == 0 and st["lawson_flips"] == 0 and st["inverted_faces"] == 0
    dt.transferToHost()
    assert np.array_equal(ht.edges(), e0)
    # one-ring: every vertex's ring is its set of mesh neighbours
    Mr = 128
    ring = torch.zeros(V * Mr, dtype=torch.int32, device="cuda")
    assert dt.oneRing(Mr, ring, layout=1) == 0
    c, rows = csr_from_table(ring.cpu().numpy(), 1, V, Mr)
    nb = [set() for _ in range(V)]
    for a, b in e0:
        nb[a].add(int(b))
        nb[b].add(int(a))
    for v in range(V):
        assert c[v] == len(nb[v]) and set(rows[v].tolist()) == nb[v], v


def test_kinetic_golden_steps(M):
    g = np.load(os.path.join(G, "kinetic_2000.npz"))
    ht, srt = build_pair(M, g["sorted_points"])
    assert np.array_equal(srt, g["sorted_points"])
    assert np.array_equal(ht.edges(), g["edges_step0"])
    dt = M.DeviceTriangulation(ht)
    for step in (1, 2, 3):
        st = dt.step(cuda(g[f"disp_step{step}"]))
        assert st["status"] == 0
        dt.transferToHost()
        assert np.array_equal(ht.edges(), g[f"dt_edges_step{step}"]), step


@pytest.mark.parametrize("n,sigma,steps", [(10000, 0.1, 5), (10000, 0.3, 3), (3000, 1.0, 4), (1000, 3.0, 4)])
def test_random_walk_matches_exact_dt(M, n, sigma, steps):
    pts = uniform_points(n, 100 + n)
    ht, srt = build_pair(M, pts)
    dt = M.DeviceTriangulation(ht)
    ref = O.Mesh.build(srt, exact=True)
    total_inverted = 0
    for k in range(steps):
        pos = ref.positions()
        d = gaussian_disp(n + 4, sigma * spacing(n), 1000 * k + n, clamp_pos=pos)
        st = dt.step(cuda(d))
        assert st["status"] == 0, st
        assert all(v == 0 for v in dt.validate().values())
        total_inverted += st["inverted_faces"]
        ref.move(d)
        dt.transferToHost()
        assert np.array_equal(ht.m_pos, ref.positions())
        exact = O.Mesh.build(ref.positions()[4:], exact=True)
        assert np.array_equal(ht.edges(), exact.edges()), (k, st)
    assert total_inverted > 0  # the untangling path was exercised


def test_taylor_green_matches_exact_dt(M):
    n = 20000
    pts = uniform_points(n, 77)
    ht, srt = build_pair(M, pts)
    dt = M.DeviceTriangulation(ht)
    pos = ht.m_pos.copy()
    for k in range(4):
        d = taylor_green_disp(pos, n)
        st = dt.step(cuda(d))
        assert st["status"] == 0, st
        pos = (pos + d).astype(np.float32)
        pos[:4] = ht.m_pos[:4]
        dt.transferToHost()
        assert np.array_equal(ht.m_pos, pos)
        exact = O.Mesh.build(pos[4:], exact=True)
        assert np.array_equal(ht.edges(), exact.edges()), (k, st)


def test_separate_calls_equal_fused_step(M):
    n = 5000
    pts = uniform_points(n, 9)
    ht1, srt = build_pair(M, pts)
    ht2 = M.HostTriangulation()
    ht2.m_pos, ht2.m_v, ht2.m_he, ht2.m_t = [a.copy() for a in (ht1.m_pos, ht1.m_v, ht1.m_he, ht1.m_t)]
    a, b = M.DeviceTriangulation(ht1), M.DeviceTriangulation(ht2)
    d = gaussian_disp(n + 4, 0.2 * spacing(n), 5, clamp_pos=ht1.m_pos)
    a.step(cuda(d))
    b.movePoints(cuda(d))
    b.untangle2()
    b.delonize2()
    a.transferToHost()
    b.transferToHost()
    assert np.array_equal(ht1.edges(), ht2.edges())
    assert np.array_equal(ht1.m_pos, ht2.m_pos)


def test_single_point_moves_match_exact_dt(M):
    """moveUntangling / moveFlipflopDelaunay (stubs in the reference) move one
    point across the mesh and leave the exact Delaunay triangulation."""
    n = 3000
    ht, srt = build_pair(M, uniform_points(n, 21))
    dt = M.DeviceTriangulation(ht)
    assert not dt.moveUntangling(1, (5.0, 5.0)) and not ht.moveFlipflop(3, (5.0, 5.0))
    p, q = 4 + n // 2, 4 + n // 5
    want = ht.m_pos.copy()
    d = np.float32([4096.5, 4100.25]) - want[p]
    assert dt.moveUntangling(p, d)
    want[p] = want[p] + d
    dt.transferToHost()
    assert np.array_equal(ht.m_pos, want)
    assert np.array_equal(ht.edges(), O.Mesh.build(want[4:], exact=True).edges())
    e = np.float32([100.0, 8000.0]) - want[q]
    assert ht.moveFlipflopDelaunay(q, e)
    want[q] = want[q] + e
    assert np.array_equal(ht.m_pos, want)
    assert np.array_equal(ht.edges(), O.Mesh.build(want[4:], exact=True).edges())


def test_one_ring_and_closest(M):
    import torch

    g = np.load(os.path.join(G, "test_frnn_1000.npz"))
    ht, _ = build_pair(M, g["points"])
    dt = M.DeviceTriangulation(ht)
    V = dt.m_pos_size
    counts, ids = O.ring_sets_from_edges(g["edges"], V)
    offs = np.concatenate([[0], np.cumsum(counts)])
    for layout in (0, 1):
        Mr = 64
        ring = torch.zeros(V * Mr, dtype=torch.int32, device="cuda")
        trunc = dt.oneRing(Mr, ring, layout=layout)
        assert trunc == 0
        c, rows = csr_from_table(ring.cpu().numpy(), layout, V, Mr)
        assert np.array_equal(c, counts)
        for i in range(V):
            r = rows[i]
            assert r[0] == r.min()  # starts at the smallest id
            assert np.array_equal(np.sort(r), ids[offs[i]:offs[i + 1]])
    # truncation to M-1 like the reference
    ring = torch.zeros(V * 4, dtype=torch.int32, device="cuda")
    assert dt.oneRing(4, ring) > 0
    # closest neighbours (tests/test_closest_neighbors.cu): brute-force argmin
    cl = np.load(os.path.join(G, "closest.npz"))
    for n in (10, 100, 1000):
        pts = cl[f"points_{n}"].copy()
        ht2, _ = build_pair(M, pts)
        assert np.array_equal(ht2.m_pos, cl[f"pos_{n}"])
        dt2 = M.DeviceTriangulation(ht2)
        Vn = dt2.m_pos_size
        ring = torch.zeros(Vn * 100, dtype=torch.int32, device="cuda")
        out = torch.zeros(Vn, dtype=torch.int32, device="cuda")
        dt2.oneRing2(100, ring)
        dt2.closestNeighbors2(100, ring, out)
        assert np.array_equal(out.cpu().numpy(), cl[f"closest_{n}"])


@pytest.mark.parametrize("r", [5, 10, 20, 30, 40, 50])
def test_mesh_frnn_reference_test(M, r):
    # tests/test_frnn.cu: counts must equal brute force; here the sets must
    import torch

    g = np.load(os.path.join(G, "test_frnn_1000.npz"))
    ht, _ = build_pair(M, g["points"])
    dt = M.DeviceTriangulation(ht)
    V = dt.m_pos_size
    F = 100
    for layout in (0, 1):
        out = torch.zeros(V * F, dtype=torch.int32, device="cuda")
        assert dt.getFRNN(F, float(r), out, layout=layout) == 0
        c, rows = csr_from_table(out.cpu().numpy(), layout, V, F)
        assert np.array_equal(c, g[f"frnn_counts_r{r}"])
        assert np.array_equal(np.concatenate(rows), g[f"frnn_ids_r{r}"])


def test_mesh_frnn_random(M):
    import torch

    n = 20000
    pts = uniform_points(n, 4)
    ht, _ = build_pair(M, pts)
    dt = M.DeviceTriangulation(ht)
    V = dt.m_pos_size
    r = 3 * spacing(n)
    F = 64
    out = torch.zeros(V * F, dtype=torch.int32, device="cuda")
    assert dt.getFRNN2(F, r, out) == 0
    c, rows = csr_from_table(out.cpu().numpy(), 1, V, F)
    bc, bids = O.frnn_brute(ht.m_pos, r)
    assert np.array_equal(c, bc)
    assert np.array_equal(np.concatenate(rows), bids)


def grid_check(M, pos, cell, ncell, mn, rad, max_nb, periodic=False, L=0.0):
    import torch

    n = len(pos)
    g = M.GridCount2d(n, mn, (cell, cell), (ncell, ncell), periodic=periodic)
    d = cuda(pos)
    g.update(d)
    sp = d.cpu().numpy()
    perm = None
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    ids = torch.zeros(n * max_nb, dtype=torch.int32, device="cuda")
    ov = g.frnn(d, rad, max_nb, counts, ids)
    c = counts.cpu().numpy()
    rows = ids.cpu().numpy().reshape(n, max_nb)
    bc, bids = O.frnn_brute(sp, rad, periodic=periodic, L=L)
    assert np.array_equal(np.sort(sp, axis=0), np.sort(pos, axis=0))
    return g, sp, c, rows, bc, bids, ov, perm


def test_grid_reference_lattices(M):
    # tests/grid2d_frnn.cu lattice tests: on-boundary distances counted exactly
    for side, step, rad, ncell in ((10, 1.0, 1.0, 10), (20, 0.5, 1.0, 10), (40, 0.25, 0.25, 10)):
        xs, ys = np.meshgrid(np.arange(side), np.arange(side))
        pos = (np.stack([xs.ravel(), ys.ravel()], 1) * step).astype(np.float32)
        g, sp, c, rows, bc, bids, ov, _ = grid_check(M, pos, 1.0, ncell, (0.0, 0.0), rad, 40)
        assert ov == 0
        assert np.array_equal(c, bc)
        assert np.array_equal(np.concatenate([np.sort(rows[i, :c[i]]) for i in range(len(pos))]), bids)


def test_grid_random_and_permutation(M):
    rng = np.random.default_rng(10)
    pos = rng.uniform(-50, 50, (10000, 2)).astype(np.float32)
    g, sp, c, rows, bc, bids, ov, _ = grid_check(M, pos, 1.0, 100, (-50.0, -50.0), 1.0, 40)
    assert ov == 0 and np.array_equal(c, bc)
    assert np.array_equal(np.concatenate([np.sort(rows[i, :c[i]]) for i in range(len(pos))]), bids)
    from helpers import d2h

    t = g.tables()
    perm = d2h(t["perm"], len(pos))
    # d_ind: input point i now sits at sorted slot perm[i]
    assert np.array_equal(sp[perm], pos)
    assert np.array_equal(np.sort(perm), np.arange(len(pos)))
    assert g.mean_num_particle_in_cell() > 0


def test_grid_periodic_torus(M):
    n = 20000
    pos = uniform_points(n, 12)
    h = spacing(n)
    ncell = int(8192 // (3 * h))
    cell = 8192.0 / ncell
    g, sp, c, rows, bc, bids, ov, _ = grid_check(M, pos, cell, ncell, (0.0, 0.0), 3 * h, 64, periodic=True, L=8192.0)
    assert ov == 0 and np.array_equal(c, bc)
    assert np.array_equal(np.concatenate([np.sort(rows[i, :c[i]]) for i in range(n)]), bids)


def test_grid_build_keeps_input_order_and_answers_in_input_ids(M):
    # the mesh's own positions, queried without permuting them (torus, r = 3h)
    import torch

    n = 30000
    pos = uniform_points(n, 14)
    h = spacing(n)
    for periodic, ncell, max_nb in ((True, 256, 64), (False, 128, 64)):
        cell = 8192.0 / ncell
        r = 3 * h if periodic else 2.5 * h
        g = M.GridCount2d(n, (0.0, 0.0), (cell, cell), (ncell, ncell), periodic=periodic)
        d = cuda(pos)
        g.build(d)
        assert np.array_equal(d.cpu().numpy(), pos)
        counts = torch.zeros(n, dtype=torch.int32, device="cuda")
        ids = torch.full((n * max_nb,), -7, dtype=torch.int32, device="cuda")
        assert g.frnn_ids(r, max_nb, counts, ids) == 0
        c = counts.cpu().numpy()
        rows = ids.cpu().numpy().reshape(n, max_nb)
        bc, bids = O.frnn_brute(pos, r, periodic=periodic, L=8192.0)
        assert np.array_equal(c, bc)
        assert np.array_equal(np.concatenate([np.sort(rows[i, :c[i]]) for i in range(n)]), bids)
        # a second build after the points moved reuses the grid
        pos2 = np.mod(pos + np.float32(0.37 * h), np.float32(8192)).astype(np.float32)
        g.build(cuda(pos2))
        assert g.frnn_ids(r, max_nb, counts, ids) == 0
        bc2, bids2 = O.frnn_brute(pos2, r, periodic=periodic, L=8192.0)
        c2 = counts.cpu().numpy()
        rows2 = ids.cpu().numpy().reshape(n, max_nb)
        assert np.array_equal(c2, bc2)
        assert np.array_equal(np.concatenate([np.sort(rows2[i, :c2[i]]) for i in range(n)]), bids2)
        g.close()


def stencil_order_lists(sp, start, count, nx, ny, cell, mn, r, periodic, L):
    """Neighbour lists of every sorted point in the full (2w+1)^2 stencil order
    (rows bottom to top, cells left to right, points of a cell in sorted
    order), float32 distances as the reference formula."""
    f = np.float32
    w = int(np.ceil(r / cell))
    r2 = f(f(r) * f(r))
    h = f(0.5) * f(L)
    out = []
    for i, p in enumerate(sp):
        x0 = int(np.floor((p[0] - mn[0]) / cell))
        y0 = int(np.floor((p[1] - mn[1]) / cell))
        if periodic:
            x0 %= nx
            y0 %= ny
        else:
            x0 = min(max(x0, 0), nx - 1)
            y0 = min(max(y0, 0), ny - 1)
        row = []
        for yy in range(y0 - w, y0 + w + 1):
            if periodic:
                y = yy % ny
            elif not 0 <= yy < ny:
                continue
            else:
                y = yy
            for xx in range(x0 - w, x0 + w + 1):
                if periodic:
                    x = xx % nx
                elif not 0 <= xx < nx:
                    continue
                else:
                    x = xx
                c = y * nx + x
                for j in range(start[c], start[c] + count[c]):
                    if j == i:
                        continue
                    dx = f(p[0]) - f(sp[j][0])
                    dy = f(p[1]) - f(sp[j][1])
                    if periodic:
                        if abs(dx) > h:
                            dx = f(dx - f(np.copysign(f(L), dx)))
                        if abs(dy) > h:
                            dy = f(dy - f(np.copysign(f(L), dy)))
                    if f(f(dx * dx) + f(dy * dy)) <= r2:
                        row.append(j)
        out.append(row)
    return out


@pytest.mark.parametrize("outside,nc", [(False, 256), (True, 256), (False, 640)])
def test_grid_frnn_ids_minimum_image_by_segment(M, outside, nc):
    # on the torus, mcl_grid_frnn_ids takes the minimum image per row segment
    # when every point is inside the domain; it must return exactly the
    # neighbours, in the same order, as the per-candidate minimum image of
    # mcl_grid_frnn on the same sorted points (points outside the domain
    # switch the segment form off)
    import torch

    from helpers import d2h

    n, L = 40000, 8192.0
    pos = uniform_points(n, 61 + outside)
    hi = np.nextafter(np.float32(L), np.float32(0))
    edge = np.array([[0, 0], [hi, hi], [0, hi], [hi, 0], [0, 4096], [hi, 17.5], [4096, hi]], np.float32)
    pos[:len(edge)] = edge
    if outside:
        pos[10] = (-3.0, 100.0)
        pos[11] = (L + 2.5, 8000.0)
    r = 3 * spacing(n)
    cell = L / nc
    max_nb = 64
    a = M.GridCount2d(n, (0.0, 0.0), (cell, cell), (nc, nc), periodic=True)
    a.build(cuda(pos))
    ca = torch.zeros(n, dtype=torch.int32, device="cuda")
    ia = torch.zeros(n * max_nb, dtype=torch.int32, device="cuda")
    assert a.frnn_ids(r, max_nb, ca, ia) == 0
    b = M.GridCount2d(n, (0.0, 0.0), (cell, cell), (nc, nc), periodic=True)
    d = cuda(pos)
    b.update(d)
    cb = torch.zeros(n, dtype=torch.int32, device="cuda")
    ib = torch.zeros(n * max_nb, dtype=torch.int32, device="cuda")
    assert b.frnn(d, r, max_nb, cb, ib) == 0
    perm = d2h(b.tables()["perm"], n)  # sorted slot of input point i
    src = np.empty(n, np.int64)
    src[perm] = np.arange(n)
    ca, ia = ca.cpu().numpy(), ia.cpu().numpy().reshape(n, max_nb)
    cb, ib = cb.cpu().numpy(), ib.cpu().numpy().reshape(n, max_nb)
    assert np.array_equal(ca, cb[perm])
    for i in range(n):
        k = ca[i]
        assert ia[i, :k].tolist() == src[ib[perm[i], :k]].tolist(), i
    assert ca[:len(edge)].min() > 0  # the corner points found neighbours across the wrap
    a.close()
    b.close()


@pytest.mark.parametrize("periodic", [False, True])
def test_grid_frnn_order_is_the_stencil_order(M, periodic):
    # the disk-shaped stencil visits fewer cells than the (2w+1)^2 square but
    # must return the same neighbours in the same order
    import torch

    from helpers import d2h

    rng = np.random.default_rng(21 + periodic)
    n, nc, cell, r = 1500, 20, 50.0, 60.0
    pos = (rng.random((n, 2), dtype=np.float32) * np.float32(1000)).astype(np.float32)
    g = M.GridCount2d(n, (0.0, 0.0), (cell, cell), (nc, nc), periodic=periodic)
    d = cuda(pos)
    g.update(d)
    sp = d.cpu().numpy()
    t = g.tables()
    start = d2h(t["start"], nc * nc)
    count = d2h(t["count"], nc * nc)
    max_nb = 64
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    ids = torch.zeros(n * max_nb, dtype=torch.int32, device="cuda")
    assert g.frnn(d, r, max_nb, counts, ids) == 0
    c = counts.cpu().numpy()
    rows = ids.cpu().numpy().reshape(n, max_nb)
    want = stencil_order_lists(sp, start, count, nc, nc, cell, (0.0, 0.0), r, periodic, 1000.0)
    for i in range(n):
        assert rows[i, :c[i]].tolist() == want[i], i


def test_device_predicates_match_host_and_golden(M):
    import torch

    from mcleap_gb300 import _lib as L

    g = np.load(os.path.join(G, "predicates.npz"))
    for kind, key, gold in ((0, "orient_pts", "orient_exact"), (1, "incircle_pts", "incircle_exact")):
        pts = cuda(g[key])
        n = len(g[key])
        sign = torch.zeros(n, dtype=torch.int32, device="cuda")
        stage = torch.zeros(n, dtype=torch.int32, device="cuda")
        L.check(L.lib().mcl_debug_predicates_device(kind, pts.data_ptr(), None, n, sign.data_ptr(), stage.data_ptr(),
                                                    None))
        torch.cuda.synchronize()
        assert np.array_equal(sign.cpu().numpy(), g[gold])
        hs, hst = L.predicates_host(kind, g[key])
        assert np.array_equal(stage.cpu().numpy(), hst)


def test_errors_are_reported(M):
    from mcleap_gb300 import McleapError

    pts = uniform_points(100, 1)
    dup = np.concatenate([pts, pts[:1]]).astype(np.float32)
    with pytest.raises(McleapError) as ei:
        M.HostTriangulation().addDelaunayPoints(dup)
    assert ei.value.code == 6
    bad = pts.copy()
    bad[3] = (2e7, 0)
    with pytest.raises(McleapError):
        M.HostTriangulation().addDelaunayPoints(bad)
    # a malformed mesh is rejected before it reaches the device
    ht = M.HostTriangulation()
    ht.addDelaunayPoints(pts.copy())
    ht.m_he[5, 0] = 10 ** 6
    with pytest.raises(McleapError):
        M.DeviceTriangulation(ht)


def test_step_host_async_matches_step(M):
    """The pipelined host-displacement call gives the same meshes and counters."""
    import ctypes as C

    import torch

    from mcleap_gb300 import _lib as L

    n = 8000
    pts = uniform_points(n, 31)
    ht1, _ = build_pair(M, pts)
    ht2 = M.HostTriangulation()
    ht2.m_pos, ht2.m_v, ht2.m_he, ht2.m_t = [a.copy() for a in (ht1.m_pos, ht1.m_v, ht1.m_he, ht1.m_t)]
    a, b = M.DeviceTriangulation(ht1), M.DeviceTriangulation(ht2)
    pos = ht1.m_pos.copy()
    nstat = C.sizeof(L.StepStats)
    pin = torch.empty(6 * nstat, dtype=torch.uint8, pin_memory=True)
    hosts, want = [], []
    stream = torch.cuda.Stream()
    for k in range(6):
        d = gaussian_disp(n + 4, 0.3 * spacing(n), 60 + k, clamp_pos=pos)
        pos = (pos + d).astype(np.float32)
        want.append(a.step(cuda(d)))
        hosts.append(torch.from_numpy(d).pin_memory())
    for k in range(6):
        L.check(L.lib().mcl_step_host_async(b.handle, hosts[k].data_ptr(), stream.cuda_stream,
                                            pin.data_ptr() + k * nstat))
    stream.synchronize()
    for k in range(6):
        got = L.StepStats.from_address(pin.data_ptr() + k * nstat).as_dict()
        # the classification's counts are deterministic; how many vertices the
        # repair sends back depends on thread timing (the result does not)
        assert got["status"] == 0 and got["inverted_faces"] == want[k]["inverted_faces"], k
        assert got["incircle_tests"] > 0
    a.transferToHost()
    b.transferToHost()
    assert np.array_equal(ht1.m_pos, ht2.m_pos)
    assert np.array_equal(ht1.edges(), ht2.edges())
    # a pageable record (not addressable by the device) is copied instead of
    # written by the step: the same counters arrive
    page = np.zeros(nstat, np.uint8)
    d = gaussian_disp(n + 4, 0.3 * spacing(n), 99, clamp_pos=pos)
    hd = torch.from_numpy(d).pin_memory()
    want2 = a.step(cuda(d))
    L.check(L.lib().mcl_step_host_async(b.handle, hd.data_ptr(), stream.cuda_stream, page.ctypes.data))
    stream.synchronize()
    got = L.StepStats.from_buffer(page).as_dict()
    assert got["status"] == 0 and got["inverted_faces"] == want2["inverted_faces"]
    assert got["incircle_tests"] > 0


def test_device_aos_arrays_equal_the_download(M):
    """DeviceTriangulation's public device arrays m_v / m_he / m_t
    (reference include/Device_Triangulation.h:139-142), written on the device
    from the engine's layout, equal the records transferToHost produces, for a
    built mesh and after repair steps."""
    import torch

    n = 30000
    ht, _ = build_pair(M, uniform_points(n, 55))
    dt = M.DeviceTriangulation(ht)
    V, HE, T = dt.m_v_size, dt.m_he_size, dt.m_t_size
    v = torch.empty((V, 2), dtype=torch.int32, device="cuda")
    he = torch.empty((HE, 4), dtype=torch.int32, device="cuda")
    t = torch.empty(T, dtype=torch.int32, device="cuda")
    for k in range(3):
        dt.export_aos(v, he, t)
        torch.cuda.synchronize()
        dt.transferToHost()
        assert np.array_equal(v.cpu().numpy(), ht.m_v.reshape(V, 2)), k
        assert np.array_equal(he.cpu().numpy(), ht.m_he.reshape(HE, 4)), k
        assert np.array_equal(t.cpu().numpy(), ht.m_t.reshape(T)), k
        d = gaussian_disp(n + 4, 0.3 * spacing(n), 77 + k, clamp_pos=ht.m_pos)
        st = dt.step(cuda(d))
        assert st["status"] == 0 and st["inverted_faces"] > 0, st


@pytest.mark.parametrize("frac,sigma", [(0.002, 0.3), (0.01, 2.0), (0.2, 0.5)])
def test_steps_moving_few_points_match_exact_dt(M, frac, sigma):
    """Steps that move a small fraction of the points classify only the edges
    whose quads hold a moved point (the rest of the mesh is Delaunay from the
    step before); the mesh is the exact Delaunay triangulation after every
    step, with and without inverted faces to repair."""
    n = 20000
    ht, _ = build_pair(M, uniform_points(n, 91))
    dt = M.DeviceTriangulation(ht)
    rng = np.random.default_rng(int(frac * 1e4))
    pos = ht.m_pos.copy()
    inverted = 0
    for k in range(6):
        d = gaussian_disp(n + 4, sigma * spacing(n), 500 + k, clamp_pos=pos)
        still = rng.random(n + 4) > frac
        d[still] = 0
        st = dt.step(cuda(d))
        assert st["status"] == 0, st
        inverted += st["inverted_faces"]
        pos = (pos + d).astype(np.float32)
        dt.transferToHost()
        assert np.array_equal(ht.m_pos, pos)
        assert np.array_equal(ht.edges(), O.Mesh.build(pos[4:], exact=True).edges()), (k, st)
    if sigma >= 2.0:
        assert inverted > 0
