"""Serving with continuous batching: every request's result is the same alone
and in the mix, and the plain one-at-a-time form gives the same results."""
import numpy as np
import pytest

from helpers import uniform_points

pytestmark = pytest.mark.gpu

SIZES = [300, 2500, 800, 1500, 120, 3000]


@pytest.fixture(scope="module")
def S():
    import torch

    from mcleap_gb300 import build as B
    from mcleap_gb300 import serving as S

    assert torch.cuda.is_available()
    B.build()
    return S


def points():
    return [uniform_points(n, 700 + i) for i, n in enumerate(SIZES)]


def fresh(S):
    return S.MeshServer(points(), budget_bytes=1 << 34, seed=11, max_query_rows=1 << 16)


def requests(S):
    reqs = S.poisson_requests(len(SIZES), rate=400.0, duration=0.2, seed=5, k_max=6, q_lo=20, q_hi=400,
                              mesh_sizes=np.array(SIZES))
    assert 40 < len(reqs) < 120
    return reqs


def snapshot(server):
    b = server.batch
    return [(b.download(i)[0], b.edges(i)) for i in range(b.count)], server.frozen.cpu().numpy()


def rows_equal(a, b):
    # each row: count, then that many ids (the slots past the count are not written)
    if a.shape != b.shape or not np.array_equal(a[:, 0], b[:, 0]):
        return False
    return all(np.array_equal(a[i, 1:1 + a[i, 0]], b[i, 1:1 + b[i, 0]]) for i in range(len(a)))


def copy_requests(reqs, keep=None):
    import dataclasses

    return [dataclasses.replace(r, result=None, t_done=None) for r in reqs if keep is None or r.mesh == keep]


def test_results_same_alone_and_in_the_mix(S):
    reqs = requests(S)
    mix = fresh(S)
    done = mix.serve(copy_requests(reqs), batched=True, realtime=False, keep_results=True)
    assert len(done) == len(reqs)
    assert mix.iterations < sum(r.k if r.kind == "step" else 1 for r in reqs)  # work was batched
    meshes_mix, frozen_mix = snapshot(mix)
    res_mix = {r.rid: r.result for r in done if r.kind != "step"}
    assert not mix.batch.validate().any()
    b = mix.batch
    # each mesh alone (the same resident set, only its own requests)
    for m in range(len(SIZES)):
        alone = fresh(S)
        mine = copy_requests(reqs, keep=m)
        d2 = alone.serve(mine, batched=True, realtime=False, keep_results=True)
        meshes_alone, frozen_alone = snapshot(alone)
        pos_a, e_a = meshes_alone[m]
        pos_m, e_m = meshes_mix[m]
        assert np.array_equal(pos_a, pos_m), m
        assert np.array_equal(e_a, e_m), m
        sl = slice(int(b.v0[m]), int(b.v0[m] + b.nv[m]))
        assert np.array_equal(frozen_alone[sl], frozen_mix[sl]), m
        for r in d2:
            if r.kind != "step":
                assert rows_equal(r.result, res_mix[r.rid]), r.rid
    # the plain form serves the same sequence one request at a time
    plain = fresh(S)
    d3 = plain.serve(copy_requests(reqs), batched=False, realtime=False, keep_results=True)
    meshes_plain, frozen_plain = snapshot(plain)
    for m in range(len(SIZES)):
        assert np.array_equal(meshes_plain[m][0], meshes_mix[m][0])
        assert np.array_equal(meshes_plain[m][1], meshes_mix[m][1])
    assert np.array_equal(frozen_plain, frozen_mix)
    for r in d3:
        if r.kind != "step":
            assert rows_equal(r.result, res_mix[r.rid])
    # the aggregation advanced and queries returned neighbours
    assert frozen_mix.sum() > sum((n + 1) // 2 for n in SIZES)
    assert any(len(v) and (v[:, 0] > 0).any() for v in res_mix.values())


def test_budget_admission_rejects_what_does_not_fit(S):
    pts = points()
    budget = sum(S.mesh_bytes(n) for n in SIZES[:3])
    server = S.MeshServer(pts, budget_bytes=budget, seed=1)
    assert server.admitted == [0, 1, 2]
    assert server.rejected == [3, 4, 5]
    assert server.batch.count == 3
