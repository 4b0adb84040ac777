"""Plain method, small workload, end to end against the CPU oracle.

10,000 points i.i.d. uniform in the (scaled) unit square, seed 1; 100 kinetic
steps, each an i.i.d. Gaussian displacement with sigma = 0.1 x mean spacing,
clamped to the box, then untangle + Delaunay restore on the GPU.  After every
step: the sorted edge set equals the oracle's exact Delaunay triangulation of
the same positions, and the FRNN lists at r = 2 x mean spacing (mesh walk and
grid, both in vertex-id space) equal brute force; every tenth step the one-ring
sets equal the exact triangulation's.  The reference's own CPU kinetic path
(movePoint, untangle until false, delonize; FP64 predicates) runs beside it for
the first steps and must agree wherever it produced a valid Delaunay mesh.
"""
import numpy as np
import pytest

from helpers import csr_from_table, gaussian_disp, spacing, uniform_points
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N, STEPS, SIGMA, REF_STEPS = 10000, 100, 0.1, 4


@pytest.fixture(scope="module")
def M():
    import torch

    import mcleap_gb300 as M
    from mcleap_gb300 import build as B

    assert torch.cuda.is_available()
    B.build()
    M.lib()
    return M


def test_plain_small_100_steps(M):
    import torch

    pts = uniform_points(N, 1)
    ht = M.HostTriangulation()
    srt = pts.copy()
    ht.addDelaunayPoints(srt)
    dt = M.DeviceTriangulation(ht)
    V = dt.m_pos_size
    h = spacing(N)
    r = 2 * h
    F, RM = 48, 32
    ref_kin = O.Mesh.build(srt, exact=False)  # the reference's build + kinetic path
    pos = ht.m_pos.copy()
    assert np.array_equal(ht.edges(), O.Mesh.build(srt, exact=True).edges())
    frnn_tab = torch.zeros(V * F, dtype=torch.int32, device="cuda")
    ring_tab = torch.zeros(V * RM, dtype=torch.int32, device="cuda")
    grid = M.GridCount2d(N, (0.0, 0.0), (r, r), (int(8192 // r), int(8192 // r)))
    gc = torch.zeros(N, dtype=torch.int32, device="cuda")
    gi = torch.zeros(N * F, dtype=torch.int32, device="cuda")
    inverted = ref_agree = 0
    for k in range(STEPS):
        d = gaussian_disp(V, SIGMA * h, 5000 + k, clamp_pos=pos)
        st = dt.step(torch.from_numpy(d).cuda())
        assert st["status"] == 0, (k, st)
        inverted += st["inverted_faces"]
        pos = (pos + d).astype(np.float32)
        dt.transferToHost()
        assert np.array_equal(ht.m_pos, pos)
        exact = O.Mesh.build(pos[4:], exact=True)
        edges = ht.edges()
        assert np.array_equal(edges, exact.edges()), k
        # FRNN r = 2h: brute force over all vertices (the corners are far away)
        bc, bids = O.frnn_brute(pos, r)
        assert dt.getFRNN(F, r, frnn_tab) == 0
        c, rows = csr_from_table(frnn_tab.cpu().numpy(), 0, V, F)
        assert np.array_equal(c, bc), k
        assert np.array_equal(np.concatenate(rows), bids), k
        # the grid over the moving points, answered in their own index order
        grid.build(torch.from_numpy(pos[4:].copy()).cuda())
        assert grid.frnn_ids(r, F, gc, gi) == 0
        gcn = gc.cpu().numpy()
        grows = gi.cpu().numpy().reshape(N, F)
        gb_c, gb_ids = O.frnn_brute(pos[4:], r)
        assert np.array_equal(gcn, gb_c), k
        assert np.array_equal(np.concatenate([np.sort(grows[i, :gcn[i]]) for i in range(N)]), gb_ids), k
        if k % 10 == 0:
            assert dt.oneRing(RM, ring_tab) == 0
            rc, rrows = csr_from_table(ring_tab.cpu().numpy(), 0, V, RM)
            ec, eids = O.ring_sets_from_edges(edges, V)
            assert np.array_equal(rc, ec)
            assert np.array_equal(np.concatenate([np.sort(x) for x in rrows]), eids)
        if k < REF_STEPS:
            ref_kin.kinetic_step_ref(d)
            chk = ref_kin.check(exact=True)
            if chk == dict(non_delaunay=0, creased=0, inverted_faces=0, zero_faces=0):
                assert np.array_equal(ref_kin.edges(), edges), k
                ref_agree += 1
    assert inverted > 0  # the untangling path ran
    print(f"inverted faces over {STEPS} steps: {inverted}; reference CPU path valid and equal on "
          f"{ref_agree}/{REF_STEPS} steps")
