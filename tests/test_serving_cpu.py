"""Host logic of the serving layer (no GPU): admission against the HBM budget
and the open-loop request generator."""
import numpy as np

from mcleap_gb300 import serving as S


def test_admission_respects_the_budget():
    a = S.Admission(10 * S.mesh_bytes(1000))
    sizes = [1000] * 12
    took = [a.try_admit(S.mesh_bytes(n)) for n in sizes]
    assert took == [True] * 10 + [False] * 2
    a.release(S.mesh_bytes(1000))
    assert a.try_admit(S.mesh_bytes(1000))
    assert not a.try_admit(1)
    # the estimate grows with the mesh: about 360 bytes per point
    per_point = S.mesh_bytes(1_000_000) / 1e6
    assert 300 < per_point < 450


def test_a_150_gb_budget_holds_the_serving_meshes():
    rng = np.random.default_rng(5)
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(1e6), 512)).astype(np.int64)
    a = S.Admission(150e9)
    assert all(a.try_admit(S.mesh_bytes(int(n))) for n in sizes)
    assert a.used < 150e9


def test_poisson_requests_are_seeded_and_shaped():
    sizes = np.array([5000, 20000, 300])
    r1 = S.poisson_requests(3, 2000.0, 1.0, seed=3, mesh_sizes=sizes)
    r2 = S.poisson_requests(3, 2000.0, 1.0, seed=3, mesh_sizes=sizes)
    assert [(r.t_arrival, r.mesh, r.kind, r.k) for r in r1] == [(r.t_arrival, r.mesh, r.kind, r.k) for r in r2]
    assert 1800 < len(r1) < 2200  # rate x duration
    t = np.array([r.t_arrival for r in r1])
    assert (np.diff(t) > 0).all()
    kinds = [r.kind for r in r1]
    assert 0.4 < kinds.count("step") / len(r1) < 0.6
    for r in r1:
        if r.kind == "step":
            assert 1 <= r.k <= 16
        else:
            assert len(r.verts) <= sizes[r.mesh]
            assert r.verts.min() >= 4 and r.verts.max() < sizes[r.mesh] + 4
            assert len(np.unique(r.verts)) == len(r.verts)
