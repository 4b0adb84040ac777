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


def _byte(o):
    o = np.asarray(o, np.int64)
    return (o[..., 0] + 8) | ((o[..., 1] + 8) << 4)


def eo_pack(B, C, X1):
    """Edge words in the engine's periodic encoding: one byte per offset
    (B, C, X1), a nibble per component biased by 8."""
    return (_byte(B) | (_byte(C) << 8) | (_byte(X1) << 16)).astype(np.uint32)


def eo_unpack(eo):
    w = np.asarray(eo, np.int64)
    out = []
    for k in range(3):
        b = (w >> (8 * k)) & 0xFF
        out.append(np.stack([(b & 15) - 8, ((b >> 4) & 15) - 8], -1))
    return out


def periodic_mesh(xy, L):
    """The periodic Delaunay triangulation of xy as a mesh in the engine's
    layout: ev[e] = (a, b, c, d), en[e] = (next(h0), prev(h0), next(h1),
    prev(h1)), eo[e] = (B, C, X1) offsets; vertex ids 0..n-1, 3n edges.

    Faces come from the 3 x 3 cover's exact triangulation: a cover face stands
    for its torus face when the copy of its smallest-id vertex is the central
    one.  Half-edges pair up as (u -> v, t) with (v -> u, -t)."""
    n = len(xy)
    pos, _, he, _ = O.Mesh.build(cover(xy, L), exact=True).aos()
    h = np.arange(len(he))
    f = he[:, 2]
    keep = f >= 0
    # one half-edge per face, then its two successors
    first = np.full(f.max() + 1, -1, np.int64)
    first[f[keep]] = h[keep]
    first = first[first >= 0]
    tri = np.stack([first, he[first, 0], he[he[first, 0], 0]], 1)
    cv = he[tri, 1].astype(np.int64) - 4        # cover vertex ids of each face's origins
    tri, cv = tri[(cv >= 0).all(1)], cv[(cv >= 0).all(1)]
    k, i = cv // n, cv % n
    rep = k[np.arange(len(k)), np.argmin(i, 1)] == CENTER
    k, i = k[rep], i[rep]
    si = np.sort(i, 1)
    if not ((si[:, 0] < si[:, 1]) & (si[:, 1] < si[:, 2])).all():
        raise ValueError("a face uses two copies of one vertex: too few points for the period")
    F = len(i)
    if F != 2 * n:
        raise ValueError("the cover does not give a torus triangulation (%d faces for %d points)" % (F, n))
    off = OFFSETS[k]                              # (F, 3, 2) copy of each corner
    # half-edge (f, j): origin corner j, target corner j+1, apex corner j+2
    j0, j1, j2 = np.arange(3), (np.arange(3) + 1) % 3, (np.arange(3) + 2) % 3
    org, tgt, apx = i[:, j0].ravel(), i[:, j1].ravel(), i[:, j2].ravel()
    t = (off[:, j1] - off[:, j0]).reshape(-1, 2)
    x = (off[:, j2] - off[:, j0]).reshape(-1, 2)
    # h0 of each edge: org < tgt, or org == tgt with t > 0
    first_side = (org < tgt) | ((org == tgt) & ((t[:, 0] > 0) | ((t[:, 0] == 0) & (t[:, 1] > 0))))
    key_u = np.where(first_side, org, tgt)
    key_v = np.where(first_side, tgt, org)
    key_t = np.where(first_side[:, None], t, -t)
    keys = np.column_stack([key_u, key_v, key_t])
    uniq, inv, cnt = np.unique(keys, axis=0, return_inverse=True, return_counts=True)
    inv = inv.ravel()
    if len(uniq) != 3 * n or (cnt != 2).any():
        raise ValueError("half-edges do not pair into 3n edges")
    hid = 2 * inv + (~first_side).astype(np.int64)   # half-edge id of (f, j)
    if len(np.unique(hid)) != 6 * n:
        raise ValueError("two half-edges of one side")
    hf = hid.reshape(F, 3)
    nxt = np.empty(6 * n, np.int64)
    prv = np.empty(6 * n, np.int64)
    nxt[hf[:, j0].ravel()] = hf[:, j1].ravel()
    prv[hf[:, j0].ravel()] = hf[:, j2].ravel()
    origin = np.empty(6 * n, np.int64)
    apex = np.empty(6 * n, np.int64)
    tt = np.empty((6 * n, 2), np.int64)
    xx = np.empty((6 * n, 2), np.int64)
    origin[hid], apex[hid], tt[hid], xx[hid] = org, apx, t, x
    ev = np.stack([origin[0::2], origin[1::2], apex[0::2], apex[1::2]], 1).astype(np.int32)
    en = np.stack([nxt[0::2], prv[0::2], nxt[1::2], prv[1::2]], 1).astype(np.int32)
    eo = eo_pack(tt[0::2], xx[0::2], xx[1::2])
    return ev, en, eo


def mesh_edges(ev, eo):
    """Canonical (u, v, ox, oy) edges of a periodic mesh in the engine layout."""
    B = eo_unpack(eo)[0]
    return canonical(np.column_stack([ev[:, 0], ev[:, 1], B]))
