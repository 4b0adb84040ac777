"""Periodic (flat torus) Delaunay triangulation oracle (test infrastructure only).

The reference's periodic triangulation (include/Host_PeriodicTriangulation.h) is
a stub: its constructor (:101-104) keeps an iso-rectangle domain for CGAL's
Periodic_2_Delaunay_triangulation_2, commented out (:3-21), and the rest is the
bounding-square code.  So parity here is unpinned: this module restates the
definition, not the reference's code.  The triangulation of n points on the
torus [x0, x0 + L)^2 is the exact Delaunay triangulation of the 3 x 3 cover
(nine copies translated by (ox L, oy L), ox, oy in {-1, 0, 1}) restricted to
the edges with an endpoint in the central copy.  Each edge is reported as
(u, v, ox, oy): from point u to the copy of point v translated by (ox, oy)
periods.  For point sets dense enough that every such edge is shorter than L/2
the restriction is a valid triangulation of the torus (3n edges, 2n faces).

The translates must be exact floats, or the copies are not congruent.  With
L a power of two and the domain [2L, 3L)^2, x + L stays in the binade
[2L, 4L) and x - L lands in [L, 2L), whose grid is finer: every translate is
exact in float32, and the oracle's exact builder sees congruent copies.
"""
import numpy as np

from . import oracle as O

OFFSETS = np.array([(ox, oy) for oy in (-1, 0, 1) for ox in (-1, 0, 1)], np.int64)
CENTER = 4


def domain_origin(L):
    """Lower corner of the torus domain whose translates are exact: 2L."""
    if not (L > 0 and float(L) == 2.0 ** np.round(np.log2(L))):
        raise ValueError("the period must be a power of two")
    return 2.0 * L


def wrap(xy, L):
    """Positions brought into [2L, 3L)^2 by whole periods (exact)."""
    x0 = domain_origin(L)
    p = np.asarray(xy, np.float64)
    k = np.floor((p - x0) / L)
    out = (p - k * L).astype(np.float32)
    assert np.array_equal(out.astype(np.float64), p - k * L), "wrapped position not exact"
    return out


def cover(xy, L):
    """The nine translated copies, copy k = 3 (oy + 1) + (ox + 1) in rows
    k n .. k n + n - 1; raises if a translate is not an exact float32."""
    x0 = domain_origin(L)
    p = np.asarray(xy, np.float32)
    if len(p) and not ((p >= x0) & (p < x0 + L)).all():
        raise ValueError("points outside the domain [2L, 3L)^2")
    c64 = p.astype(np.float64)[None] + OFFSETS[:, None, :].astype(np.float64) * L
    c32 = c64.astype(np.float32)
    if not np.array_equal(c32.astype(np.float64), c64):
        raise ValueError("a translate is not an exact float32")
    return c32.reshape(-1, 2)


def canonical(rows):
    """Each undirected edge once: u < v, or u == v with (ox, oy) > (0, 0)."""
    r = np.array(rows, np.int64).reshape(-1, 4)
    swap = (r[:, 0] > r[:, 1]) | ((r[:, 0] == r[:, 1]) & ((r[:, 2] < 0) | ((r[:, 2] == 0) & (r[:, 3] < 0))))
    r[swap] = np.column_stack([r[swap, 1], r[swap, 0], -r[swap, 2], -r[swap, 3]])
    return np.unique(r, axis=0)


def periodic_edges(xy, L):
    """Sorted canonical edges (u, v, ox, oy) of the periodic Delaunay
    triangulation of xy (point ids 0..n-1)."""
    n = len(xy)
    m = O.Mesh.build(cover(xy, L), exact=True)
    e = m.edges().astype(np.int64)
    e = e[(e >= 4).all(1)] - 4
    k, i = e // n, e % n
    rows = []
    for a, b in ((0, 1), (1, 0)):
        sel = k[:, a] == CENTER
        o = OFFSETS[k[sel, b]] - OFFSETS[k[sel, a]]
        rows.append(np.column_stack([i[sel, a], i[sel, b], o]))
    return canonical(np.concatenate(rows))


def is_torus_triangulation(edges, n):
    """Euler's relation on the torus (E = 3n) and no vertex of degree < 3."""
    deg = np.bincount(edges[:, 0], minlength=n) + np.bincount(edges[:, 1], minlength=n)
    return len(edges) == 3 * n and (deg >= 3).all()


def shift_edges(edges, wrapped):
    """The edges after every point i moved by whole periods -wrapped[i] (its
    canonical copy changed): offsets pick up wrapped[v] - wrapped[u]."""
    w = np.asarray(wrapped, np.int64)
    e = np.array(edges, np.int64)
    e[:, 2:] += w[e[:, 1]] - w[e[:, 0]]
    return canonical(e)
