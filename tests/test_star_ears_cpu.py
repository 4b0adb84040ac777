"""The removal's constant-time ear test (mcleap_gb300/csrc/engine.cu,
clip_star), checked with exact integer arithmetic on the star polygons of
random Delaunay triangulations: while the removed vertex v lies strictly inside
the kernel of the remaining polygon, a convex corner b between a and c whose
diagonal a -> c has v strictly on its left is an ear (its closed triangle holds
no other corner), and the new side keeps v strictly inside the kernel."""
import numpy as np
import pytest

spatial = pytest.importorskip("scipy.spatial")


def orient(a, b, c):
    return (int(b[0]) - int(a[0])) * (int(c[1]) - int(a[1])) - (int(b[1]) - int(a[1])) * (int(c[0]) - int(a[0]))


def in_closed_triangle(p, a, b, c):
    return orient(a, b, p) >= 0 and orient(b, c, p) >= 0 and orient(c, a, p) >= 0


def stars(pts, tri):
    """Each interior vertex's link, counter-clockwise (vertices of the hull skipped)."""
    hull = set(np.unique(tri.convex_hull))
    nb = tri.vertex_neighbor_vertices
    for v in range(len(pts)):
        if v in hull:
            continue
        ring = nb[1][nb[0][v]:nb[0][v + 1]]
        ang = np.arctan2(pts[ring, 1] - pts[v, 1], pts[ring, 0] - pts[v, 0])
        yield v, [int(w) for w in ring[np.argsort(ang)]]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fast_ears_are_ears(seed):
    rng = np.random.default_rng(seed)
    pts = np.unique(rng.integers(0, 1 << 20, (3000, 2)), axis=0)
    tri = spatial.Delaunay(pts.astype(np.float64))
    fast = general = 0
    for v, link in stars(pts, tri):
        P = {w: pts[w] for w in link}
        pv = pts[v]
        poly = list(link)
        # the star is valid: v strictly inside the kernel
        kernel = all(orient(P[poly[i]], P[poly[(i + 1) % len(poly)]], pv) > 0 for i in range(len(poly)))
        assert kernel
        while len(poly) > 3:
            k = len(poly)
            j = None
            if kernel:
                for i in range(k):
                    a, b, c = poly[i - 1], poly[i], poly[(i + 1) % k]
                    if orient(P[a], P[c], pv) > 0 and orient(P[a], P[b], P[c]) > 0:
                        j = i
                        break
            if j is not None:
                fast += 1
                a, b, c = poly[j - 1], poly[j], poly[(j + 1) % k]
                others = [w for w in poly if w not in (a, b, c)]
                assert not any(in_closed_triangle(P[w], P[a], P[b], P[c]) for w in others)
                del poly[j]
                # v stays strictly inside the kernel of what remains
                assert all(orient(P[poly[i]], P[poly[(i + 1) % len(poly)]], pv) > 0 for i in range(len(poly)))
            else:
                general += 1
                for i in range(k):
                    a, b, c = poly[i - 1], poly[i], poly[(i + 1) % k]
                    others = [w for w in poly if w not in (a, b, c)]
                    if orient(P[a], P[b], P[c]) > 0 and not any(
                            in_closed_triangle(P[w], P[a], P[b], P[c]) for w in others):
                        kernel = kernel and orient(P[a], P[c], pv) > 0
                        del poly[i]
                        break
                else:
                    raise AssertionError("no ear")
    assert fast > 10 * max(general, 1), (fast, general)
