"""Periodic (flat torus) kinetic Delaunay meshes over the C ABI.

The reference's periodic triangulation (include/Host_PeriodicTriangulation.h)
is a stub; this is the working form: n points on the torus [2L, 3L)^2 (L a
power of two), 3n edges and 2n faces, built exactly on the GPU and stepped
with move + wrap + parallel flip rounds (``mcl_periodic_*`` in
include/mcl_gb300.h).  Edges are reported as (u, v, ox, oy): from point u to
the copy of point v translated by (ox, oy) periods.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _stream_ptr(stream):
    if stream is None:
        return None
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def eo_offsets(eo):
    """(B, C, X1) offsets of the edge words: B = the copy of b relative to a,
    C = the apex c relative to a, X1 = the apex d relative to b."""
    w = np.asarray(eo, np.int64)
    return [np.stack([((w >> (8 * k)) & 15) - 8, ((w >> (8 * k + 4)) & 15) - 8], -1) for k in range(3)]


def canonical_edges(ev, eo):
    """Each undirected edge once as (u, v, ox, oy) with u < v, or u == v and
    (ox, oy) > (0, 0); rows sorted."""
    B = eo_offsets(eo)[0]
    r = np.column_stack([ev[:, 0], ev[:, 1], B]).astype(np.int64)
    swap = (r[:, 0] > r[:, 1]) | ((r[:, 0] == r[:, 1]) & ((r[:, 2] < 0) | ((r[:, 2] == 0) & (r[:, 3] < 0))))
    r[swap] = np.column_stack([r[swap, 1], r[swap, 0], -r[swap, 2], -r[swap, 3]])
    return np.unique(r, axis=0)


class PeriodicTriangulation:
    """A periodic Delaunay mesh resident on the GPU."""

    def __init__(self, points=None, period=8192.0, _handle=None):
        self.handle = C.c_void_p()
        if _handle is not None:
            self.handle = _handle
        else:
            pts = np.ascontiguousarray(points, np.float32)
            L.check(L.lib().mcl_periodic_build(L.ptr(pts), len(pts), float(period), C.byref(self.handle)))
        n, E, per = C.c_int64(), C.c_int64(), C.c_float()
        L.check(L.lib().mcl_periodic_sizes(self.handle, C.byref(n), C.byref(E), C.byref(per)))
        self.n, self.E, self.L = n.value, E.value, per.value
        self.last_stats = None

    @classmethod
    def from_arrays(cls, pos, period, ev, en, eo):
        pos = np.ascontiguousarray(pos, np.float32)
        ev = np.ascontiguousarray(ev, np.int32)
        en = np.ascontiguousarray(en, np.int32)
        eo = np.ascontiguousarray(eo, np.uint32)
        h = C.c_void_p()
        L.check(L.lib().mcl_periodic_create(L.ptr(pos), len(pos), float(period), L.ptr(ev), L.ptr(en), L.ptr(eo),
                                            C.byref(h)))
        return cls(_handle=h)

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            L.lib().mcl_periodic_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, d, stream=None):
        """Move by d (device float2[n]), wrap, flip back to Delaunay.  Moves
        that would turn faces over are refused, then resumed by sub-steps
        (``substep_vertices``) and, for the rest, removal and reinsertion
        (``removed_vertices``); ``reverted_vertices`` counts points that end
        the step away from their targets."""
        st = L.StepStats()
        wrapped = C.c_int64()
        rc = L.lib().mcl_periodic_step(self.handle, L.ptr(d), _stream_ptr(stream), C.byref(st), C.byref(wrapped))
        self.last_stats = st.as_dict()
        self.last_stats["wrapped"] = wrapped.value
        L.check(rc)
        return self.last_stats

    def step_host(self, d_host, stream=None):
        """step() with the displacements in host memory (float32 (n, 2))."""
        d = np.ascontiguousarray(d_host, np.float32)
        st = L.StepStats()
        wrapped = C.c_int64()
        rc = L.lib().mcl_periodic_step_host(self.handle, L.ptr(d), _stream_ptr(stream), C.byref(st),
                                            C.byref(wrapped))
        self.last_stats = st.as_dict()
        self.last_stats["wrapped"] = wrapped.value
        L.check(rc)
        return self.last_stats

    def download(self):
        pos = np.zeros((self.n, 2), np.float32)
        ev = np.zeros((self.E, 4), np.int32)
        en = np.zeros((self.E, 4), np.int32)
        eo = np.zeros(self.E, np.uint32)
        L.check(L.lib().mcl_periodic_download(self.handle, L.ptr(pos), L.ptr(ev), L.ptr(en), L.ptr(eo)))
        return pos, ev, en, eo

    def positions_ptr(self):
        p = C.c_void_p()
        L.check(L.lib().mcl_periodic_positions(self.handle, C.byref(p)))
        return p.value

    def edges(self):
        _, ev, _, eo = self.download()
        return canonical_edges(ev, eo)

    def oneRing(self, maxRingSize, ring_neighbors, offsets=None, stream=None, layout=L.LAYOUT_COLUMN):
        """Clockwise neighbours from the smallest (id, offset); slot 0 the
        count.  offsets (optional uint8 device tensor, same layout): each
        neighbour's copy offset byte.  Returns the number of truncated rings."""
        trunc = C.c_int64()
        L.check(L.lib().mcl_periodic_one_ring(self.handle, maxRingSize, layout, L.ptr(ring_neighbors), L.ptr(offsets),
                                              _stream_ptr(stream), C.byref(trunc)))
        return trunc.value

    def getFRNN(self, maxFRNNSize, r, neighbors, offsets=None, stream=None, layout=L.LAYOUT_COLUMN):
        """Every other point with a copy within r (< L/2), ascending ids, slot 0
        the count; offsets (optional uint8 device tensor): copy offset bytes.
        Returns the number of truncated lists."""
        trunc = C.c_int64()
        L.check(L.lib().mcl_periodic_frnn(self.handle, float(r), maxFRNNSize, layout, L.ptr(neighbors),
                                          L.ptr(offsets), _stream_ptr(stream), C.byref(trunc)))
        return trunc.value

    def closestNeighbors(self, maxRingSize, ring_neighbors, offsets, closest_neighbors, stream=None,
                         layout=L.LAYOUT_COLUMN):
        L.check(L.lib().mcl_periodic_closest(self.handle, maxRingSize, layout, L.ptr(ring_neighbors), L.ptr(offsets),
                                             L.ptr(closest_neighbors), _stream_ptr(stream)))
        return True


def from_planar(aos_view, vertex_point, vertex_copy, n):
    """The periodic mesh a planar triangulation of a cover stands for (host
    conversion, no device work): (ev, en, eo)."""
    vp = np.ascontiguousarray(vertex_point, np.int32)
    vc = np.ascontiguousarray(vertex_copy, np.int32)
    ev = np.zeros((3 * n, 4), np.int32)
    en = np.zeros((3 * n, 4), np.int32)
    eo = np.zeros(3 * n, np.uint32)
    L.check(L.lib().mcl_periodic_from_planar(C.byref(aos_view), L.ptr(vp), L.ptr(vc), n, L.ptr(ev), L.ptr(en),
                                             L.ptr(eo)))
    return ev, en, eo
