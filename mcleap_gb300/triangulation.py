"""Python mirror of the reference's call surface, over the C ABI.

Class and method names follow the reference's C++ structs so tests and tools
read like the reference's own drivers:

* ``HostTriangulation`` - the AoS container (include/Host_Triangulation.h:24-98);
  ``addDelaunayPoints`` sorts the points in place into the reference's Morton
  order and builds the Delaunay triangulation on the GPU.
* ``DeviceTriangulation`` - the device mesh (include/Device_Triangulation.h:128-223).
* ``GridCount2d`` - the uniform-grid neighbour search (include/gridCount2d.h:23-48).

Device buffers are torch CUDA tensors (or raw device addresses); torch is only
the allocator and stream plumbing here, all computation is in libmcl_gb300.so.
"""
import ctypes as C

import numpy as np

from . import _lib as L

BOX_LO = np.float32(-10000000.0)
BOX_HI = np.float32(10000000.0)

# The reference's bounding-square seed (include/Host_Triangulation.h:107-137).
_SEED_POS = np.array([[BOX_LO, BOX_LO], [BOX_HI, BOX_LO], [BOX_HI, BOX_HI], [BOX_LO, BOX_HI]], np.float32)
_SEED_V = np.array([[0, 0], [1, 2], [2, 6], [3, 8]], np.int32)
_SEED_HE = np.array([[2, 0, 0, 2], [9, 1, -1, -1], [4, 1, 0, 0], [1, 2, -1, -1], [0, 2, 0, 1],
                     [6, 0, 1, 3], [8, 2, 1, 0], [3, 3, -1, -1], [5, 3, 1, 2], [7, 0, -1, -1]], np.int32)
_SEED_T = np.array([[4], [5]], np.int32)


def _stream_ptr(stream):
    if stream is None:
        return None
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class HostTriangulation:
    """AoS mesh in the reference's interchange layout."""

    def __init__(self):
        self.m_pos = _SEED_POS.copy()
        self.m_v = _SEED_V.copy()
        self.m_he = _SEED_HE.copy()
        self.m_t = _SEED_T.copy()

    def addDelaunayPoints(self, points):
        """Sort ``points`` (n x 2 float32, C-contiguous) in place into Morton order
        and triangulate them with the bounding square on the GPU
        (include/Host_Triangulation.h:296-300)."""
        if not (isinstance(points, np.ndarray) and points.dtype == np.float32 and points.flags["C_CONTIGUOUS"]
                and points.ndim == 2 and points.shape[1] == 2):
            raise TypeError("points must be a C-contiguous (n, 2) float32 numpy array")
        h = C.c_void_p()
        L.check(L.lib().mcl_mesh_build(L.ptr(points), len(points), C.byref(h)))
        try:
            self._download(h)
        finally:
            L.lib().mcl_mesh_destroy(h)
        return True

    def _download(self, h):
        V, HE, T = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(L.lib().mcl_mesh_sizes(h, C.byref(V), C.byref(HE), C.byref(T)))
        self.m_pos = np.zeros((V.value, 2), np.float32)
        self.m_v = np.zeros((V.value, 2), np.int32)
        self.m_he = np.zeros((HE.value, 4), np.int32)
        self.m_t = np.zeros((T.value, 1), np.int32)
        L.check(L.lib().mcl_mesh_download_aos(h, L.ptr(self.m_pos), L.ptr(self.m_v), L.ptr(self.m_he),
                                               L.ptr(self.m_t)))

    def movePoint(self, p_index, d):
        """include/Host_Triangulation.h:403-406."""
        self.m_pos[p_index] += np.asarray(d, np.float32)
        return True

    def _move_one(self, p_index, d):
        """include/Host_Triangulation.h:77-80 (the reference's bodies at
        :408-413 return False): move one point and leave a valid Delaunay
        mesh, by stepping a device copy with a single nonzero displacement.
        The bounding corners (ids 0..3) refuse to move."""
        if not 4 <= p_index < len(self.m_pos):
            return False
        disp = np.zeros_like(self.m_pos)
        disp[p_index] = np.asarray(d, np.float32)
        view = self.aos_view()
        h = C.c_void_p()
        L.check(L.lib().mcl_mesh_create_from_aos(C.byref(view), C.byref(h)))
        try:
            st = L.StepStats()
            L.check(L.lib().mcl_step_host(h, L.ptr(disp), None, C.byref(st)))
            self._download(h)
        finally:
            L.lib().mcl_mesh_destroy(h)
        return True

    moveFlipflop = moveFlipflopDelaunay = moveUntangling = moveUntanglingDelaunay = _move_one

    def edges(self):
        """Sorted undirected edge list (u < v), one row per edge."""
        a, b = self.m_he[0::2, 1], self.m_he[1::2, 1]
        e = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)
        return e[np.lexsort((e[:, 1], e[:, 0]))]

    def aos_view(self):
        self._keep = [np.ascontiguousarray(a) for a in (self.m_pos, self.m_v, self.m_he, self.m_t)]
        p, v, he, t = self._keep
        return L.AosView(L.ptr(p), L.ptr(v), L.ptr(he), L.ptr(t), len(p), len(he), len(t))


class DeviceTriangulation:
    """Device mesh built from a HostTriangulation (include/Device_Triangulation.h:232-236)."""

    def __init__(self, h_triangulation):
        self.h_triangulation = h_triangulation
        self.handle = C.c_void_p()
        view = h_triangulation.aos_view()
        L.check(L.lib().mcl_mesh_create_from_aos(C.byref(view), C.byref(self.handle)))
        V, HE, T = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(L.lib().mcl_mesh_sizes(self.handle, C.byref(V), C.byref(HE), C.byref(T)))
        self.m_pos_size = self.m_v_size = V.value
        self.m_he_size = HE.value
        self.m_t_size = T.value
        self.last_stats = None

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            L.lib().mcl_mesh_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- transfers ---------------------------------------------------------------
    def transferToHost(self):
        """include/Device_Triangulation.h:245-253 (triangle ids are canonical)."""
        self.h_triangulation._download(self.handle)
        return True

    def transferToDevice(self):
        view = self.h_triangulation.aos_view()
        L.check(L.lib().mcl_mesh_upload_aos(self.handle, C.byref(view)))
        return True

    @property
    def m_pos(self):
        """Current device address of the positions (changes after every move)."""
        p = C.c_void_p()
        L.check(L.lib().mcl_mesh_positions(self.handle, C.byref(p)))
        return p.value

    def export_aos(self, v=None, he=None, t=None, stream=None):
        """The reference's public device arrays m_v / m_he / m_t
        (include/Device_Triangulation.h:139-142) written into caller-owned
        int32 CUDA tensors of shape (V, 2), (HE, 4), (T,) (any may be None),
        with the face numbering of transferToHost."""
        L.check(L.lib().mcl_mesh_export_aos(self.handle, L.ptr(v), L.ptr(he), L.ptr(t), _stream_ptr(stream)))

    def positions(self, out=None, stream=None):
        """Copy the current positions into ``out`` (torch CUDA tensor) or a numpy array."""
        if out is None:
            host = np.zeros((self.m_pos_size, 2), np.float32)
            L.check(L.lib().mcl_mesh_copy_positions(self.handle, L.ptr(host), 1, _stream_ptr(stream)))
            return host
        L.check(L.lib().mcl_mesh_copy_positions(self.handle, L.ptr(out), 0, _stream_ptr(stream)))
        return out

    # -- moving ------------------------------------------------------------------
    def movePoints(self, d, stream=None):
        L.check(L.lib().mcl_move(self.handle, L.ptr(d), _stream_ptr(stream)))
        return True

    def integrateMovePoints(self, dt, v, stream=None):
        L.check(L.lib().mcl_integrate(self.handle, L.ptr(dt), L.ptr(v), _stream_ptr(stream)))
        return True

    def _run(self, fn, stream):
        st = L.StepStats()
        L.check(fn(self.handle, _stream_ptr(stream), C.byref(st)))
        self.last_stats = st.as_dict()
        return True

    def untangle(self, stream=None):
        return self._run(L.lib().mcl_untangle, stream)

    untangle2 = untangle

    def delonize(self, stream=None):
        return self._run(L.lib().mcl_delaunay_restore, stream)

    delonize2 = delonize

    def step(self, d, stream=None, stats=True):
        """movePoints(d) + untangle + delonize in one persistent launch."""
        if stats:
            st = L.StepStats()
            L.check(L.lib().mcl_step(self.handle, L.ptr(d), _stream_ptr(stream), C.byref(st)))
            self.last_stats = st.as_dict()
            return self.last_stats
        L.check(L.lib().mcl_step(self.handle, L.ptr(d), _stream_ptr(stream), None))
        return None

    def step_host(self, d_host, stream=None, stats=True):
        st = L.StepStats()
        L.check(L.lib().mcl_step_host(self.handle, L.ptr(d_host), _stream_ptr(stream),
                                      C.byref(st) if stats else None))
        if stats:
            self.last_stats = st.as_dict()
            return self.last_stats
        return None

    def _move_one(self, p_index, d):
        """include/Device_Triangulation.h:183-186 (the reference's bodies at
        :411-417 return False): move one point and leave a valid Delaunay
        mesh, through one kinetic step on a host displacement with a single
        nonzero entry.  The bounding corners (ids 0..3) refuse to move."""
        if not 4 <= p_index < self.m_pos_size:
            return False
        disp = np.zeros((self.m_pos_size, 2), np.float32)
        disp[p_index] = np.asarray(d, np.float32)
        self.step_host(disp)
        return True

    moveFlipflop = moveFlipflopDelaunay = moveUntangling = moveUntanglingDelaunay = _move_one

    def totals(self):
        """Counters summed over every call since creation, and the call count."""
        st = L.StepStats()
        calls = C.c_int64()
        L.check(L.lib().mcl_mesh_totals(self.handle, C.byref(st), C.byref(calls)))
        d = st.as_dict()
        d["calls"] = calls.value
        return d

    def validate(self):
        """Counts of structural invariant violations (all zero for a valid mesh)."""
        out = np.zeros(8, np.int64)
        L.check(L.lib().mcl_mesh_validate(self.handle, L.ptr(out)))
        keys = ["next_prev", "not_triangle", "apex", "twin", "vertex_he", "orientation", "dead_edge", "range"]
        return dict(zip(keys, out.tolist()))

    def status(self, stream=None):
        st = L.StepStats()
        L.check(L.lib().mcl_mesh_last_status(self.handle, _stream_ptr(stream), C.byref(st)))
        return st.as_dict()

    # -- queries -------------------------------------------------------------------
    def oneRing(self, maxRingSize, ring_neighbors, stream=None, layout=L.LAYOUT_COLUMN):
        """include/Device_Triangulation.h:499-507; returns the number of truncated rings."""
        tr = C.c_int64()
        L.check(L.lib().mcl_one_ring(self.handle, layout, maxRingSize, L.ptr(ring_neighbors), _stream_ptr(stream),
                                     C.byref(tr)))
        return tr.value

    def oneRing2(self, maxRingSize, ring_neighbors, stream=None):
        return self.oneRing(maxRingSize, ring_neighbors, stream, L.LAYOUT_ROW)

    def closestNeighbors(self, maxRingSize, ring_neighbors, closest_neighbors, stream=None, layout=L.LAYOUT_COLUMN):
        L.check(L.lib().mcl_closest_neighbors(self.handle, layout, maxRingSize, L.ptr(ring_neighbors),
                                              L.ptr(closest_neighbors), _stream_ptr(stream)))
        return True

    def closestNeighbors2(self, maxRingSize, ring_neighbors, closest_neighbors, stream=None):
        return self.closestNeighbors(maxRingSize, ring_neighbors, closest_neighbors, stream, L.LAYOUT_ROW)

    def getFRNN(self, maxFRNNSize, r, neighbors, stream=None, layout=L.LAYOUT_COLUMN):
        """include/Device_Triangulation.h:529-537 (the ring table is not needed:
        the search walks the mesh directly); returns the number of overflowing lists."""
        ov = C.c_int64()
        L.check(L.lib().mcl_mesh_frnn(self.handle, float(r), layout, maxFRNNSize, L.ptr(neighbors),
                                      _stream_ptr(stream), C.byref(ov)))
        return ov.value

    def getFRNN2(self, maxFRNNSize, r, neighbors, stream=None):
        return self.getFRNN(maxFRNNSize, r, neighbors, stream, L.LAYOUT_ROW)


class GridCount2d:
    """Uniform-grid fixed-radius neighbours (include/gridCount2d.h:23-48)."""

    def __init__(self, numP, min_xy, cell_size, num_cells, periodic=False):
        self.numP = int(numP)
        self.handle = C.c_void_p()
        L.check(L.lib().mcl_grid_create(self.numP, float(min_xy[0]), float(min_xy[1]), float(cell_size[0]),
                                        float(cell_size[1]), int(num_cells[0]), int(num_cells[1]),
                                        L.GRID_PERIODIC if periodic else 0, C.byref(self.handle)))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            L.lib().mcl_grid_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, pos, vel=None, stream=None):
        """Sort points by cell and permute ``pos`` (and ``vel``) in place."""
        L.check(L.lib().mcl_grid_update(self.handle, L.ptr(pos), L.ptr(vel), _stream_ptr(stream)))

    def frnn(self, pos, rad, max_nb, counts, ids, stream=None):
        """apply_f_frnn with the reference tests' SaveNeighborsFunctor; returns overflow count."""
        ov = C.c_int64()
        L.check(L.lib().mcl_grid_frnn(self.handle, L.ptr(pos), float(rad), int(max_nb), L.ptr(counts), L.ptr(ids),
                                      _stream_ptr(stream), C.byref(ov)))
        return ov.value

    def build(self, pos, stream=None):
        """Cell tables for ``pos`` without permuting it (``pos`` is only read)."""
        L.check(L.lib().mcl_grid_build(self.handle, L.ptr(pos), _stream_ptr(stream)))

    def frnn_ids(self, rad, max_nb, counts, ids, stream=None, overflow=True):
        """Neighbours of the last build/update in input index space; returns the
        overflow count (or None when ``overflow`` is False: no host sync)."""
        ov = C.c_int64()
        L.check(L.lib().mcl_grid_frnn_ids(self.handle, float(rad), int(max_nb), L.ptr(counts), L.ptr(ids),
                                          _stream_ptr(stream), C.byref(ov) if overflow else None))
        return ov.value if overflow else None

    def tables(self):
        perm, start, count = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nx, ny = C.c_int(), C.c_int()
        L.check(L.lib().mcl_grid_tables(self.handle, C.byref(perm), C.byref(start), C.byref(count), C.byref(nx),
                                        C.byref(ny)))
        return dict(perm=perm.value, start=start.value, count=count.value, nx=nx.value, ny=ny.value)

    def mean_num_particle_in_cell(self):
        m = C.c_float()
        L.check(L.lib().mcl_grid_mean_occupancy(self.handle, C.byref(m)))
        return m.value
