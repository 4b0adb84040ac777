"""The periodic (torus) Delaunay oracle: a valid torus triangulation, invariant
under translation with wrap-around, and equal to the planar Delaunay
triangulation away from the domain's sides."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import periodic as P

L = 8192.0


def torus_points(n, seed):
    rng = np.random.default_rng(seed)
    x0 = P.domain_origin(L)
    p = (x0 + rng.random((n, 2)) * L).astype(np.float32)
    p[p >= x0 + L] = np.nextafter(np.float32(x0 + L), np.float32(0))
    assert len(np.unique(p, axis=0)) == n
    return p


@pytest.mark.parametrize("n,seed", [(500, 1), (3000, 2)])
def test_is_a_torus_triangulation(n, seed):
    xy = torus_points(n, seed)
    e = P.periodic_edges(xy, L)
    assert P.is_torus_triangulation(e, n)
    # every edge crosses at most one period per axis
    assert (np.abs(e[:, 2:]) <= 1).all()
    assert (e[:, 2:] != 0).any(axis=1).sum() > 0


def test_translation_with_wrap_around():
    n = 2000
    xy = torus_points(n, 5)
    e = P.periodic_edges(xy, L)
    s = np.array([L / 4, 3 * L / 8])
    moved = xy.astype(np.float64) + s
    wrapped = (moved >= P.domain_origin(L) + L).astype(np.int64)
    xy2 = P.wrap(moved, L)
    assert np.array_equal(xy2.astype(np.float64), moved - wrapped * L)
    assert np.array_equal(P.periodic_edges(xy2, L), P.shift_edges(e, wrapped))


def test_interior_matches_the_planar_triangulation():
    n = 4000
    xy = torus_points(n, 7)
    e = P.periodic_edges(xy, L)
    planar = O.Mesh.build(xy, exact=True).edges().astype(np.int64)
    planar = planar[(planar >= 4).all(1)] - 4
    x0, m = P.domain_origin(L), 0.15 * L
    inner = ((xy >= x0 + m) & (xy < x0 + L - m)).all(1)
    a = {tuple(r) for r in planar if inner[r[0]] and inner[r[1]]}
    b = {(r[0], r[1]) for r in e if inner[r[0]] and inner[r[1]] and r[2] == 0 and r[3] == 0}
    assert len(a) > n and a == b


def test_domain_and_exactness_guards():
    with pytest.raises(ValueError):
        P.domain_origin(1000.0)
    with pytest.raises(ValueError):
        P.cover(np.array([[1.0, 2.0]], np.float32), L)
    # any float32 of the domain has exact translates by one period
    x0 = P.domain_origin(L)
    p = np.array([[x0, np.nextafter(np.float32(x0 + L), np.float32(0))],
                  [x0 + 0.001953125, x0 + L / 3]], np.float32)
    c = P.cover(p, L).reshape(9, 2, 2).astype(np.float64)
    assert np.array_equal(c - P.OFFSETS[:, None, :] * L, np.broadcast_to(p.astype(np.float64), (9, 2, 2)))


def test_point_order_is_a_relabelling():
    """The periodic triangulation does not depend on the order of the points:
    a permutation relabels the edges and nothing else."""
    n = 2500
    xy = torus_points(n, 13)
    perm = np.random.default_rng(4).permutation(n)
    e = P.periodic_edges(xy, L)
    e2 = P.periodic_edges(xy[perm], L)
    back = np.column_stack([perm[e2[:, 0]], perm[e2[:, 1]], e2[:, 2:]])
    assert np.array_equal(P.canonical(back), e)
