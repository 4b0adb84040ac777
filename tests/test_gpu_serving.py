"""Serving with continuous batching: every request's result is the same alone
and in the mix, the plain one-at-a-time form gives the same results, every
served mesh is the oracle's exact Delaunay triangulation of its positions, and
meshes waiting for HBM budget are admitted as closed meshes free it."""
import numpy as np
import pytest

from helpers import uniform_points
from oracle import oracle as O

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
    states = [server.mesh_state(g) for g in range(len(SIZES))]
    return [(p, e) for p, e, _ in states], [f for _, _, f in states]


def assert_exact(meshes):
    for m, (pos, edges) in enumerate(meshes):
        assert np.array_equal(edges, O.Mesh.build(pos[4:], exact=True).edges()), m


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
    assert_exact(meshes_mix)  # every served mesh is the exact Delaunay triangulation
    res_mix = {r.rid: r.result for r in done if r.kind != "step"}
    assert all(not grp.batch.validate().any() for grp in mix.groups)
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
        assert np.array_equal(frozen_alone[m], frozen_mix[m]), m
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
    assert all(np.array_equal(a, b) for a, b in zip(frozen_plain, frozen_mix))
    for r in d3:
        if r.kind != "step":
            assert rows_equal(r.result, res_mix[r.rid])
    # the aggregation advanced and queries returned neighbours
    assert sum(int(f.sum()) for f in frozen_mix) > sum((n + 1) // 2 for n in SIZES)
    assert any(len(v) and (v[:, 0] > 0).any() for v in res_mix.values())


def test_meshes_wait_for_budget_and_are_admitted_as_meshes_close(S):
    """A budget that holds the first four meshes: the rest wait; requests on
    a waiting mesh wait with it; closing meshes frees their bytes (their group
    is compacted) and the waiting meshes are admitted, in order, with the same
    results as when everything is resident from the start."""
    pts = points()
    budget = sum(S.mesh_bytes(n) for n in SIZES[:4])
    assert S.mesh_bytes(SIZES[1]) + S.mesh_bytes(SIZES[3]) >= S.mesh_bytes(SIZES[4]) + S.mesh_bytes(SIZES[5])
    server = S.MeshServer(pts, budget_bytes=budget, seed=11, max_query_rows=1 << 16)
    assert server.admitted == [0, 1, 2, 3]
    assert [g for g, _ in server.waiting] == [4, 5] and server.rejected == []
    assert server.admission.used <= budget
    huge = server.submit_mesh(uniform_points(200_000, 9))  # larger than the whole budget
    assert server.status[huge] == "rejected"
    reqs = requests(S)
    # close meshes 1 and 3 after their own requests: they sit in the group of
    # 0..3, which is compacted to make room for 4 and 5
    t_end = reqs[-1].t_arrival
    closes = [S.Request(len(reqs), t_end + 0.001, 1, "close"), S.Request(len(reqs) + 1, t_end + 0.002, 3, "close")]
    done = server.serve(copy_requests(reqs) + closes, batched=True, realtime=False, keep_results=True)
    assert len(done) == len(reqs) + 2
    assert server.status[:6] == ["resident", "closed", "resident", "closed", "resident", "resident"]
    assert server.compactions >= 1 and server.admission.used <= budget
    # the meshes admitted late end as they do when everything is resident at once
    ref = fresh(S)
    ref.serve(copy_requests(reqs), batched=True, realtime=False)
    for m in (0, 2, 4, 5):
        a, b = server.mesh_state(m), ref.mesh_state(m)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), m
        assert np.array_equal(a[1], O.Mesh.build(a[0][4:], exact=True).edges()), m
    # a mesh opened by a request joins once there is room
    new = S.Request(0, 0.0, 7, "open", points=uniform_points(400, 1))
    step = S.Request(1, 0.0, 7, "step", k=3)
    server.serve([new, step], batched=True, realtime=False)
    assert server.status[7] == "resident" and step.t_done is not None
    pos, edges, _ = server.mesh_state(7)
    assert np.array_equal(edges, O.Mesh.build(pos[4:], exact=True).edges())
