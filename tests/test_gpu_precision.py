"""Precision stress: points on a jittered lattice (nearly and sometimes exactly
cocircular quads), in tight clusters and uniform; a small Gaussian walk.  Every predicate sign the
engine takes on the live mesh agrees with the exact oracle (orientation,
incircle, incircle with symbolic perturbation), the mesh stays the exact
Delaunay triangulation, and the reference's own FP64 incircle is shown to get
some of these signs wrong."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    from mcleap_gb300 import build as B

    assert torch.cuda.is_available()
    B.build()
    return torch


def sampled_quads(mesh, rng, sample):
    pos, _, he, _ = mesh.download(0)
    org, apex = he[:, 1], he[:, 3]
    inner = np.nonzero((apex[0::2] >= 0) & (apex[1::2] >= 0))[0]
    e = rng.choice(inner, size=min(sample, len(inner)), replace=False)
    a, b, c, d = org[2 * e], org[2 * e + 1], apex[2 * e], apex[2 * e + 1]
    pts8 = np.stack([pos[a], pos[b], pos[c], pos[d]], 1).reshape(-1, 8).astype(np.float32)
    ids = np.stack([a, b, c, d], 1).astype(np.int32)
    pts6 = np.stack([pos[a], pos[b], pos[c]], 1).reshape(-1, 6).astype(np.float32)
    return pos, pts8, ids, pts6


def device_signs(torch, kind, pts, ids=None):
    from mcleap_gb300 import _lib as L

    dp = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    di = torch.from_numpy(np.ascontiguousarray(ids)).cuda() if ids is not None else None
    sg = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    st = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    L.check(L.lib().mcl_debug_predicates_device(kind, dp.data_ptr(), di.data_ptr() if di is not None else None,
                                                len(pts), sg.data_ptr(), st.data_ptr(), None))
    return sg.cpu().numpy(), st.cpu().numpy()


def test_precision_stress_signs_and_edges(env):
    torch = env
    from mcleap_gb300 import batch as MB
    from mcleap_gb300 import workloads as W

    n = 100_000
    pts = W.precision_points(n, 9)
    mesh = MB.MeshBatch(MB.build_mesh(pts.copy()))
    h = 8192.0 / np.sqrt(n)
    sigma = torch.tensor([0.05 * h], dtype=torch.float32, device="cuda")
    counter = torch.zeros(1, dtype=torch.int64, device="cuda")
    d = torch.zeros((mesh.V, 2), dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(4)
    ref_wrong = cocircular = sos = 0
    stages = np.zeros(4, np.int64)
    for k in range(5):
        pos, pts8, ids, pts6 = sampled_quads(mesh, rng, 100_000)
        exact = O.incircle(pts8, mode=1)
        s1, st1 = device_signs(torch, 1, pts8)
        assert np.array_equal(s1, exact), k
        s2, st2 = device_signs(torch, 2, pts8, ids)
        assert np.array_equal(s2, O.incircle(pts8, mode=2, ids=ids)), k
        s0, _ = device_signs(torch, 0, pts6)
        assert np.array_equal(s0, O.orient2d(pts6, mode=1)), k
        assert (st2 >= 0).all()  # no expansion overflow
        stages += np.bincount(st2, minlength=4)[:4]
        cocircular += int((exact == 0).sum())
        sos += int((st2 == 3).sum())
        ref_wrong += int((O.incircle(pts8, mode=0) != exact).sum())
        # the live mesh is the exact Delaunay triangulation of its positions
        assert np.array_equal(mesh.edges(0), O.Mesh.build(pos[4:], exact=True).edges()), k
        mesh.walk(sigma, counter, d, seed=5)
        mesh.settle(d)
        st = mesh.step(d)
        assert st["status"] == 0, st
    assert stages[1] + stages[2] + stages[3] > 0  # quads the FP32 filter could not decide
    print(f"sampled incircles: stage counts fp32/fp64/exact/sos {stages.tolist()}, exactly cocircular "
          f"{cocircular}, reference FP64 incircle wrong on {ref_wrong}")


@pytest.mark.parametrize("exponent,rotation", [(23, 0.0), (30, 0.0), (22, 0.3)])
def test_sign_map_is_exact(env, exponent, rotation):
    # the reference's precision experiment as counts: every cell of the
    # engine's map has the exact sign; near the circle the FP32 filter hands
    # the cells to the later stages
    from mcleap_gb300 import signmap as S

    R = 128
    counts, grid = S.sign_map(R, exponent, rotation)
    exact = O.incircle(S.quad_points(R, exponent, rotation), mode=1)
    assert np.array_equal(grid.ravel(), exact)
    assert counts["positive"] + counts["zero"] + counts["negative"] == R * R
    assert sum(counts["stages"].values()) == R * R
    assert counts["stages"]["fp32"] < R * R
    if rotation == 0.0:
        assert counts["zero"] > 0  # d itself is on the circle
    print(counts)
