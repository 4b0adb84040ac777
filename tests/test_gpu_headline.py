"""Parity at the headline sizes: the 1M-point Taylor-Green mesh and the
4M-point precision-stress mesh, stepped on the GPU, are compared after every
step with the oracle's exact Delaunay triangulation of the same positions
(bit-identical sorted edge sets), and every predicate sign the engine's ladder
gives on the live mesh's quads and faces is compared with the exact oracle.
Also integrateMovePoints (reference include/Device_Triangulation.h:403-410,
include/kernels.cuh:45-50: pos[i] += v[i] * dt[i] for i >= 4)."""
import numpy as np
import pytest

from helpers import spacing, uniform_points
from oracle import oracle as O

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


def live_quads(pos, he):
    """The (a, b, c, d) quad of every interior edge and the (a, b, c) corners of
    every face of a reference-layout mesh (HalfEdge = {next, v, t, op})."""
    org, apex = he[:, 1], he[:, 3]
    inner = np.nonzero((apex[0::2] >= 0) & (apex[1::2] >= 0))[0]
    a, b, c, d = org[2 * inner], org[2 * inner + 1], apex[2 * inner], apex[2 * inner + 1]
    pts8 = np.stack([pos[a], pos[b], pos[c], pos[d]], 1).reshape(-1, 8).astype(np.float32)
    ids = np.stack([a, b, c, d], 1).astype(np.int32)
    h = np.nonzero(apex >= 0)[0]
    pts6 = np.stack([pos[org[h]], pos[org[h ^ 1]], pos[apex[h]]], 1).reshape(-1, 6).astype(np.float32)
    return pts8, ids, pts6


def device_signs(kind, pts, ids=None):
    import torch

    from mcleap_gb300 import _lib as L

    dp = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    di = torch.from_numpy(np.ascontiguousarray(ids)).cuda() if ids is not None else None
    sg = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    st = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    L.check(L.lib().mcl_debug_predicates_device(kind, dp.data_ptr(), di.data_ptr() if di is not None else None,
                                                len(pts), sg.data_ptr(), st.data_ptr(), None))
    return sg.cpu().numpy(), st.cpu().numpy()


def check_signs(pos, he):
    """Engine ladder = exact oracle on every live quad (plain and with symbolic
    perturbation) and every face; returns the number of quads checked."""
    pts8, ids, pts6 = live_quads(pos, he)
    s1, _ = device_signs(1, pts8)
    assert int((s1 != O.incircle(pts8, mode=1)).sum()) == 0
    s2, st2 = device_signs(2, pts8, ids)
    assert int((s2 != O.incircle(pts8, mode=2, ids=ids)).sum()) == 0
    assert (s2 <= 0).all()  # a Delaunay mesh: no quad has its fourth point strictly inside
    assert (st2 >= 0).all()  # no expansion overflow
    s0, _ = device_signs(0, pts6)
    assert np.array_equal(s0, O.orient2d(pts6, mode=1))
    assert (s0 > 0).all()  # every face counter-clockwise
    return len(pts8) + len(pts6)


def test_taylor_green_1m_matches_exact_dt(M):
    """Config 2's mesh: 1M points, dt = 0.5 x spacing, three steps."""
    import torch

    from mcleap_gb300 import workloads as W

    n = 1_000_000
    ht = M.HostTriangulation()
    ht.addDelaunayPoints(W.uniform_points(n, 2026))
    dt = M.DeviceTriangulation(ht)
    disp = W.taylor_green_displacements_device(ht.m_pos, n, 3)
    pos = ht.m_pos.copy()
    flips = 0
    for k in range(3):
        st = dt.step(disp[k])
        assert st["status"] == 0, st
        flips += st["lawson_flips"]
        pos = (pos + disp[k].cpu().numpy()).astype(np.float32)
        dt.transferToHost()
        assert np.array_equal(ht.m_pos, pos), k
        exact = O.Mesh.build(pos[4:], exact=True)
        assert np.array_equal(ht.edges(), exact.edges()), (k, st)
    assert flips > 0
    assert check_signs(ht.m_pos, ht.m_he) > 5_000_000
    torch.cuda.synchronize()


def test_precision_stress_4m_matches_exact_dt(M):
    """Config 3's point set at its full 4M size: jittered lattice (exactly
    cocircular quads), tight clusters and uniform points; two Gaussian-walk
    steps of 0.05 x spacing."""
    import torch

    from mcleap_gb300 import batch as MB
    from mcleap_gb300 import workloads as W

    n = 4_000_000
    mesh = MB.MeshBatch(MB.build_mesh(W.precision_points(n, 3)))
    pos, _, he, _ = mesh.download(0)
    assert np.array_equal(mesh.edges(0), O.Mesh.build(pos[4:], exact=True).edges())
    sigma = torch.tensor([0.05 * spacing(n)], dtype=torch.float32, device="cuda")
    counter = torch.zeros(1, dtype=torch.int64, device="cuda")
    d = torch.zeros((mesh.V, 2), dtype=torch.float32, device="cuda")
    sos = 0
    for k in range(2):
        mesh.walk(sigma, counter, d, seed=21)
        mesh.settle(d)
        st = mesh.step(d)
        assert st["status"] == 0, st
        sos += st["sos_decisions"]
        pos, _, he, _ = mesh.download(0)
        assert np.array_equal(mesh.edges(0), O.Mesh.build(pos[4:], exact=True).edges()), (k, st)
    assert check_signs(pos, he) > 20_000_000
    print(f"4M precision stress: {sos} symbolic-perturbation decisions in 2 steps")


def test_integrate_move_points(M):
    """pos[i] += v[i] * dt[i] in float32 (product rounded, then the sum) for
    the moving points; the four bounding corners stay; a Delaunay restore
    afterwards gives the exact triangulation of the new positions."""
    import torch

    n = 20_000
    ht = M.HostTriangulation()
    ht.addDelaunayPoints(uniform_points(n, 31))
    dt = M.DeviceTriangulation(ht)
    rng = np.random.default_rng(8)
    V = n + 4
    h = spacing(n)
    pos0 = ht.m_pos.copy()
    v = (rng.standard_normal((V, 2)) * 0.1 * h).astype(np.float32)
    tau = rng.uniform(0.0, 1.0, V).astype(np.float32)
    tau[rng.random(V) < 0.3] = 0.0  # frozen walkers, as in the DLA driver
    # keep every target inside the box and distinct
    want = pos0.copy()
    want[4:] = (pos0[4:] + (v[4:] * tau[4:, None]).astype(np.float32)).astype(np.float32)
    inside = ((want >= 0) & (want < 8192)).all(1)
    tau[~inside] = 0.0
    want = pos0.copy()
    want[4:] = (pos0[4:] + (v[4:] * tau[4:, None]).astype(np.float32)).astype(np.float32)
    assert len(np.unique(want, axis=0)) == V
    dt.integrateMovePoints(torch.from_numpy(tau).cuda(), torch.from_numpy(v).cuda())
    dt.delonize()
    st = dt.last_stats
    assert st["status"] == 0, st
    dt.transferToHost()
    assert np.array_equal(ht.m_pos, want)
    assert np.array_equal(ht.m_pos[:4], pos0[:4])
    assert np.array_equal(ht.edges(), O.Mesh.build(want[4:], exact=True).edges()), st
