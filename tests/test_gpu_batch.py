"""Batches of meshes through the C ABI: one launch steps every mesh, and each
mesh of the batch ends exactly where it ends when stepped alone (and equals the
oracle's exact Delaunay triangulation).  Also the motion models (random walk,
settling of coincident moves, aggregation contact) and per-mesh FRNN radii.
"""
import numpy as np
import pytest

from helpers import gaussian_disp, spacing, uniform_points
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HI = float(np.nextafter(np.float32(8192), np.float32(0)))


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


SIZES = [100, 2000, 50, 3000, 800, 7]


def make_points():
    return [uniform_points(n, 500 + i) for i, n in enumerate(SIZES)]


def test_batch_equals_meshes_stepped_alone(M):
    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    assert batch.count == len(SIZES)
    assert list(batch.nv) == [n + 4 for n in SIZES]
    alone = []
    for p in pts:
        ht = M.HostTriangulation()
        q = p.copy()
        ht.addDelaunayPoints(q)
        alone.append((ht, M.DeviceTriangulation(ht)))
    for i, (ht, _) in enumerate(alone):
        assert np.array_equal(batch.edges(i), ht.edges())
    sigmas = [0.1, 0.3, 1.0, 0.2, 0.5, 0.3]
    pos = [ht.m_pos.copy() for ht, _ in alone]
    inverted = 0
    for k in range(4):
        ds = [gaussian_disp(len(pos[i]), sigmas[i] * spacing(SIZES[i]), 900 * k + i, clamp_pos=pos[i])
              for i in range(len(SIZES))]
        st = batch.step(cuda(np.concatenate(ds)))
        assert st["status"] == 0, st
        inverted += st["inverted_faces"]
        assert not batch.validate().any()
        for i, (ht, dt) in enumerate(alone):
            assert dt.step(cuda(ds[i]))["status"] == 0
            dt.transferToHost()
            pos[i] = (pos[i] + ds[i]).astype(np.float32)
            bpos = batch.download(i)[0]
            assert np.array_equal(bpos, pos[i])
            e = batch.edges(i)
            assert np.array_equal(e, ht.edges()), (k, i)
            assert np.array_equal(e, O.Mesh.build(pos[i][4:], exact=True).edges()), (k, i)
    assert inverted > 0  # some mesh went through the repair path


def test_batch_with_empty_and_tiny_meshes(M):
    sizes = [0, 1, 2, 5, 300, 0]
    pts = [uniform_points(n, 40 + i) if n else np.zeros((0, 2), np.float32) for i, n in enumerate(sizes)]
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    assert list(batch.nv) == [n + 4 for n in sizes]
    pos = [batch.download(i)[0] for i in range(batch.count)]
    for k in range(3):
        d = np.concatenate([gaussian_disp(len(pos[i]), 200.0, 50 * k + i, clamp_pos=pos[i])
                            for i in range(batch.count)])
        st = batch.step(cuda(d))
        assert st["status"] == 0, st
        assert not batch.validate().any()
        pos = [batch.download(i)[0] for i in range(batch.count)]
        for i in range(batch.count):
            assert matches_oracle(batch.edges(i), pos[i]), (k, i)


def matches_oracle(got, pos):
    """The oracle's exact Delaunay triangulation.  For the bare bounding square
    (four exactly cocircular corners, no point) the step's Lawson pass picks
    the diagonal by the symbolic perturbation where the reference's build keeps
    the construction diagonal: both triangulate the square, either is taken."""
    want = O.Mesh.build(pos[4:], exact=True).edges()
    if len(pos) > 4:
        return np.array_equal(got, want)
    sides = [[0, 1], [0, 3], [1, 2], [2, 3]]
    square = [np.array(sorted(sides + [dg]), np.int32) for dg in ([0, 2], [1, 3])]
    return any(np.array_equal(got, sq) for sq in square)


def test_clone_and_tuning_do_not_change_results(M):
    pts = make_points()
    a = M.MeshBatch.from_points([p.copy() for p in pts])
    b = a.clone()
    t = b.tuning()
    assert t["max_blocks_per_sm"] >= 1
    b.set_tuning(blocks_per_sm=1, tail_items=64, removal_tile=1)
    assert b.tuning()["blocks_per_sm"] == 1 and b.tuning()["tail_items"] == 64 and b.tuning()["removal_tile"] == 1
    pos = [a.download(i)[0] for i in range(a.count)]
    for k in range(3):
        d = np.concatenate([gaussian_disp(len(pos[i]), 0.4 * spacing(SIZES[i]), 77 * k + i, clamp_pos=pos[i])
                            for i in range(a.count)])
        assert a.step(cuda(d))["status"] == 0
        assert b.step(cuda(d))["status"] == 0
        pos = [a.download(i)[0] for i in range(a.count)]
    for i in range(a.count):
        assert np.array_equal(a.edges(i), b.edges(i))


@pytest.mark.parametrize("sigma", [0.1, 0.5, 2.0])
def test_repair_substeps_and_removal_give_the_same_mesh(M, sigma):
    # sub-steps bring most sent-back vertices to their targets without
    # removal; with none every one is removed and reinserted: the mesh must
    # be the same exact Delaunay triangulation either way
    pts = make_points()
    a = M.MeshBatch.from_points([p.copy() for p in pts])
    b = a.clone()
    a.set_substeps(8)
    b.set_substeps(0)
    pos = [a.download(i)[0] for i in range(a.count)]
    sub = removed_a = removed_b = 0
    for k in range(3):
        d = np.concatenate([gaussian_disp(len(pos[i]), sigma * spacing(SIZES[i]), 313 * k + i, clamp_pos=pos[i])
                            for i in range(a.count)])
        sa, sb = a.step(cuda(d)), b.step(cuda(d))
        assert sa["status"] == 0 and sb["status"] == 0, (sa, sb)
        # each sent-back vertex reaches its target by sub-steps or by reinsertion
        assert sa["reverted_vertices"] == sa["substep_vertices"] + sa["removed_vertices"]
        assert sb["substep_vertices"] == 0 and sb["removed_vertices"] == sb["reverted_vertices"]
        sub += sa["substep_vertices"]
        removed_a += sa["removed_vertices"]
        removed_b += sb["removed_vertices"]
        assert not a.validate().any() and not b.validate().any()
        pos = [a.download(i)[0] for i in range(a.count)]
        for i in range(a.count):
            assert np.array_equal(b.download(i)[0], pos[i])
            e = a.edges(i)
            assert np.array_equal(e, b.edges(i)), (k, i)
            assert np.array_equal(e, O.Mesh.build(pos[i][4:], exact=True).edges()), (k, i)
    assert sub > 0 and removed_b > 0


def test_walk_is_counter_based_and_stays_in_the_box(M):
    import torch

    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    V = batch.V
    sigma = cuda(np.array([5.0 * (i + 1) for i in range(batch.count)], np.float32))
    counter = torch.zeros(batch.count, dtype=torch.int64, device="cuda")
    d1 = torch.zeros((V, 2), dtype=torch.float32, device="cuda")
    d2 = torch.zeros_like(d1)
    frozen = torch.zeros(V, dtype=torch.uint8, device="cuda")
    frozen[4::2] = 1
    batch.walk(sigma, counter, d1, seed=7, frozen=frozen)
    assert counter.tolist() == [1] * batch.count
    counter.zero_()
    batch.walk(sigma, counter, d2, seed=7, frozen=frozen)
    assert torch.equal(d1, d2)
    batch.walk(sigma, counter, d2, seed=7, frozen=frozen)
    assert not torch.equal(d1, d2)
    d = d1.cpu().numpy()
    fz = frozen.cpu().numpy().astype(bool)
    pos = np.concatenate([batch.download(i)[0] for i in range(batch.count)])
    corners = np.concatenate([np.arange(4) + v0 for v0 in batch.v0])
    assert not d[corners].any() and not d[fz].any()
    new = (pos + d).astype(np.float32)
    free = np.ones(V, bool)
    free[corners] = False
    assert (new[free] >= 0).all() and (new[free] <= HI).all()
    # a mesh draws the same numbers alone (seed + its index) as inside the batch
    from mcleap_gb300.batch import build_mesh

    one = M.MeshBatch(build_mesh(pts[1].copy()))
    d_one = torch.zeros((one.V, 2), dtype=torch.float32, device="cuda")
    c1 = torch.zeros(1, dtype=torch.int64, device="cuda")
    one.walk(sigma[1:2], c1, d_one, seed=8, frozen=frozen[batch.v0[1]:batch.v0[1] + batch.nv[1]].contiguous())
    assert torch.equal(d_one, d1[batch.v0[1]:batch.v0[1] + batch.nv[1]])
    # per-mesh sigma: the spread grows with the mesh index
    spread = [np.abs(d[batch.v0[i] + 4:batch.v0[i] + batch.nv[i]]).mean() for i in range(batch.count)
              if batch.nv[i] > 200]
    assert spread == sorted(spread)


def test_settle_moves_matches_the_rule(M):
    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    pos = np.concatenate([batch.download(i)[0] for i in range(batch.count)])
    comp = np.concatenate([np.full(batch.nv[i], i) for i in range(batch.count)])
    fixed = np.zeros(batch.V, bool)
    for v0 in batch.v0:
        fixed[v0:v0 + 4] = True
    rng = np.random.default_rng(3)
    d = (rng.standard_normal((batch.V, 2)) * 2.0).astype(np.float32)
    d[fixed] = 0
    b0, b1 = int(batch.v0[1]), int(batch.v0[3])  # meshes with 2000 and 3000 points

    def window(v0, nv):
        # vertices with both coordinates in [3000, 5000]: every difference of two
        # such coordinates (and of 4000.5 / 4000.25) is exact in float32
        # (Sterbenz), so pos + (target - pos) lands exactly on the target
        p = pos[v0 + 4:v0 + nv]
        return v0 + 4 + np.nonzero(((p >= 3000) & (p <= 5000)).all(1))[0]

    w0, w1 = window(b0, int(batch.nv[1])), window(b1, int(batch.nv[3]))
    assert len(w0) >= 8 and len(w1) >= 8
    # a mover onto a vertex that stays
    a, b = w0[0], w0[1]
    d[a] = pos[b] - pos[a]
    d[b] = 0
    # two movers onto one point
    tgt = np.float32([4000.5, 4000.25])
    c0, c1 = w0[2], w0[3]
    d[c0] = tgt - pos[c0]
    d[c1] = tgt - pos[c1]
    # a chain: x -> old(y), y -> z (z stays): y goes back, then x must too
    x, y, z = w1[0], w1[1], w1[2]
    d[y] = pos[z] - pos[y]
    d[z] = 0
    d[x] = pos[y] - pos[x]
    # the same point in two different meshes is not a coincidence
    e0, e1 = w0[4], w1[4]
    d[e0] = pos[e1] - pos[e0]
    d[e1] = 0
    for v, t in ((a, pos[b]), (c0, tgt), (c1, tgt), (y, pos[z]), (x, pos[y]), (e0, pos[e1])):
        assert np.array_equal((pos[v] + d[v]).astype(np.float32), t)
    d = d.astype(np.float32)
    want = O.settle_moves(pos, d, comp, fixed)
    dd = cuda(d)
    sent = batch.settle(dd)
    got = dd.cpu().numpy()
    assert np.array_equal(got, want)
    assert sent == int(((want != d).any(1)).sum())
    for v in (a, c0, c1, x, y):
        assert not got[v].any(), v
    assert got[e0].any()
    # the settled move is then a valid step
    assert batch.step(dd)["status"] == 0
    assert not batch.validate().any()
    # a second call on clean displacements changes nothing
    d2 = np.zeros_like(d)
    d2[w0[5]] = [0.5, 0.25]
    dd2 = cuda(d2)
    assert batch.settle(dd2) == 0
    assert np.array_equal(dd2.cpu().numpy(), d2)


def test_batch_frnn_per_mesh_radius(M):
    import torch

    from helpers import csr_from_table

    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    radii = np.array([2.0 * spacing(n) for n in SIZES], np.float32)
    F = 48
    out = torch.zeros(batch.V * F, dtype=torch.int32, device="cuda")
    assert batch.frnn(cuda(radii), F, out) == 0
    c, rows = csr_from_table(out.cpu().numpy(), 1, batch.V, F)
    for i in range(batch.count):
        v0, nv = int(batch.v0[i]), int(batch.nv[i])
        pos = batch.download(i)[0]
        bc, bids = O.frnn_brute(pos, float(radii[i]))
        assert np.array_equal(c[v0:v0 + nv], bc)
        got = np.concatenate([rows[v0 + j] - v0 for j in range(nv)]) if nv else np.zeros(0, np.int32)
        assert np.array_equal(got, bids), i


def test_dla_freeze_matches_brute_force(M):
    import torch

    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    radii = np.array([1.0 * spacing(n) for n in SIZES], np.float32)
    rng = np.random.default_rng(8)
    fin = (rng.random(batch.V) < 0.2).astype(np.uint8)
    for v0 in batch.v0:
        fin[v0:v0 + 4] = 0
    fi = cuda(fin)
    newly = batch.dla_freeze(cuda(radii), fi)
    got = fi.cpu().numpy()
    want = fin.copy()
    for i in range(batch.count):
        v0, nv = int(batch.v0[i]), int(batch.nv[i])
        pos = batch.download(i)[0]
        bc, bids = O.frnn_brute(pos, float(radii[i]))
        offs = np.concatenate([[0], np.cumsum(bc)])
        for j in range(4, nv):
            if not fin[v0 + j] and fin[v0 + bids[offs[j]:offs[j + 1]]].any():
                want[v0 + j] = 1
    assert np.array_equal(got, want)
    assert newly == int((want != fin).sum())


def test_active_subset_steps_only_those_meshes(M):
    """Steps restricted to some meshes of a batch leave the others untouched and
    equal the same meshes stepped alone (the position double buffer of an
    idle mesh is kept in step)."""
    import torch

    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    alone = []
    for p in pts:
        ht = M.HostTriangulation()
        q = p.copy()
        ht.addDelaunayPoints(q)
        alone.append((ht, M.DeviceTriangulation(ht)))
    pos = [ht.m_pos.copy() for ht, _ in alone]
    plan = [[1, 3], [0, 1], [5, 2, 4], [], [3]]
    for k, active in enumerate(plan):
        batch.set_active(active)
        ds = [np.zeros_like(pos[i]) for i in range(len(SIZES))]
        for i in (active or range(len(SIZES))):
            ds[i] = gaussian_disp(len(pos[i]), 0.3 * spacing(SIZES[i]), 31 * k + i, clamp_pos=pos[i])
        st = batch.step(cuda(np.concatenate(ds)))
        assert st["status"] == 0, st
        for i in (active or range(len(SIZES))):
            ht, dt = alone[i]
            assert dt.step(cuda(ds[i]))["status"] == 0
            dt.transferToHost()
            pos[i] = (pos[i] + ds[i]).astype(np.float32)
        batch.set_active(None)
        assert not batch.validate().any()
        for i, (ht, _) in enumerate(alone):
            bpos = batch.download(i)[0]
            assert np.array_equal(bpos, pos[i]), (k, i)
            assert np.array_equal(batch.edges(i), ht.edges()), (k, i)
    # the motion calls follow the active set too
    counter = torch.zeros(batch.count, dtype=torch.int64, device="cuda")
    d = torch.zeros((batch.V, 2), dtype=torch.float32, device="cuda")
    sigma = cuda(np.full(batch.count, 3.0, np.float32))
    batch.set_active([2, 4])
    batch.walk(sigma, counter, d, seed=1)
    assert counter.tolist() == [0, 0, 1, 0, 1, 0]
    dn = d.cpu().numpy()
    for i in range(batch.count):
        sl = dn[batch.v0[i]:batch.v0[i] + batch.nv[i]]
        assert sl.any() == (i in (2, 4))
    assert batch.settle(d) == 0
    assert batch.step(d)["status"] == 0
    batch.set_active(None)
    assert not batch.validate().any()


def test_query_lists_match_full_queries(M):
    import torch

    from helpers import csr_from_table

    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    radii = cuda(np.array([2.0 * spacing(n) for n in SIZES], np.float32))
    F, RM = 48, 32
    full = torch.zeros(batch.V * F, dtype=torch.int32, device="cuda")
    batch.frnn(radii, F, full)
    ring = torch.zeros(batch.V * RM, dtype=torch.int32, device="cuda")
    batch.one_ring(RM, ring, layout=1)
    rng = np.random.default_rng(2)
    verts = rng.choice(batch.V, 500, replace=False).astype(np.int32)
    vq = cuda(verts)
    out = torch.zeros(len(verts) * F, dtype=torch.int32, device="cuda")
    assert batch.frnn_list(radii, vq, F, out) == 0
    c_full, rows_full = csr_from_table(full.cpu().numpy(), 1, batch.V, F)
    c_l, rows_l = csr_from_table(out.cpu().numpy(), 1, len(verts), F)
    for q, v in enumerate(verts):
        assert np.array_equal(rows_l[q], rows_full[v])
    outr = torch.zeros(len(verts) * RM, dtype=torch.int32, device="cuda")
    assert batch.one_ring_list(vq, RM, outr) == 0
    c_r, rows_r = csr_from_table(ring.cpu().numpy(), 1, batch.V, RM)
    c_rl, rows_rl = csr_from_table(outr.cpu().numpy(), 1, len(verts), RM)
    for q, v in enumerate(verts):
        assert np.array_equal(rows_rl[q], rows_r[v])


def test_batch_frnn_grid_equals_mesh_walk(M):
    import torch

    pts = make_points()
    batch = M.MeshBatch.from_points([p.copy() for p in pts])
    radii = np.array([2.0 * spacing(n) for n in SIZES], np.float32)
    rd = cuda(radii)
    F = 48
    a = torch.full((batch.V * F,), -5, dtype=torch.int32, device="cuda")
    b = torch.full((batch.V * F,), -7, dtype=torch.int32, device="cuda")
    assert batch.frnn(rd, F, a) == 0
    assert batch.frnn_grid(radii, rd, F, b) == 0
    ra, rb = a.view(batch.V, F).cpu().numpy(), b.view(batch.V, F).cpu().numpy()
    assert np.array_equal(ra[:, 0], rb[:, 0])
    for v in range(batch.V):
        c = ra[v, 0]
        assert np.array_equal(ra[v, 1:1 + c], rb[v, 1:1 + c]), v
    # after some steps (points moved, grid rebuilt from the new positions)
    pos = [batch.download(i)[0] for i in range(batch.count)]
    d = np.concatenate([gaussian_disp(len(pos[i]), 0.3 * spacing(SIZES[i]), 3 + i, clamp_pos=pos[i])
                        for i in range(batch.count)])
    assert batch.step(cuda(d))["status"] == 0
    batch.frnn(rd, F, a)
    batch.frnn_grid(radii, rd, F, b)
    ra, rb = a.view(batch.V, F).cpu().numpy(), b.view(batch.V, F).cpu().numpy()
    assert np.array_equal(ra[:, 0], rb[:, 0])
    assert all(np.array_equal(ra[v, 1:1 + ra[v, 0]], rb[v, 1:1 + ra[v, 0]]) for v in range(batch.V))


def test_captured_step_pipeline_equals_direct_steps(M):
    """StepPipeline (walk + settle + step + per-mesh grid FRNN captured in a
    CUDA graph, replayed) leaves every mesh exactly as the same calls made
    one by one, and every mesh the exact Delaunay triangulation; its FRNN rows
    are the mesh-walk FRNN rows.  Autotuning changes the launch shape only."""
    import torch

    from mcleap_gb300 import batch as MB

    pts = make_points()
    a = M.MeshBatch.from_points([p.copy() for p in pts])
    b = a.clone()
    sizes = np.array([len(p) for p in pts])
    h = (8192.0 / np.sqrt(np.maximum(sizes, 1))).astype(np.float32)
    sigma = torch.tensor(0.3 * h, device="cuda")
    r_host = (2.0 * h).astype(np.float32)
    radius = torch.tensor(r_host, device="cuda")
    F = 48
    pipe = MB.StepPipeline(a, sigma, r_host, radius, F, seed=9, steps_per_graph=2, tune=True)
    for _ in range(3):
        pipe.replay()
    pipe.check()
    assert pipe.tuned is not None
    # the same seven steps (one before the capture, two per replay) made directly
    ctr = torch.zeros(b.count, dtype=torch.int64, device="cuda")
    d = torch.zeros((b.V, 2), dtype=torch.float32, device="cuda")
    for _ in range(7):
        b.walk(sigma, ctr, d, seed=9)
        b.settle(d)
        assert b.step(d)["status"] == 0
    out = torch.empty(b.V * F, dtype=torch.int32, device="cuda")
    b.frnn(radius, F, out)
    for i in range(a.count):
        assert np.array_equal(a.download(i)[0], b.download(i)[0]), i
        assert np.array_equal(a.edges(i), b.edges(i)), i
        assert matches_oracle(a.edges(i), a.download(i)[0]), i
    rows_a = pipe.out.view(a.V, F).cpu().numpy()
    rows_b = out.view(b.V, F).cpu().numpy()
    points_only = np.concatenate([np.arange(int(a.v0[i]) + 4, int(a.v0[i] + a.nv[i])) for i in range(a.count)])
    for v in points_only:
        c = rows_b[v, 0]
        assert rows_a[v, 0] == c and np.array_equal(np.sort(rows_a[v, 1:1 + c]), np.sort(rows_b[v, 1:1 + c])), v
