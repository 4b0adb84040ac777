"""Batches of independent meshes stepped together, motion models, tuning.

A batch is one device mesh whose components are the meshes (each with its own
bounding square), so every engine call steps or queries all of them in one
launch.  The reference has no counterpart: it steps one DeviceTriangulation at
a time.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from .triangulation import _stream_ptr


def build_mesh(points):
    """GPU Delaunay build of ``points`` (sorted in place into the reference's
    Morton order, ids 4.. after the bounding corners); returns a raw handle."""
    if not (isinstance(points, np.ndarray) and points.dtype == np.float32 and points.flags["C_CONTIGUOUS"]):
        raise TypeError("points must be a C-contiguous float32 numpy array")
    h = C.c_void_p()
    L.check(L.lib().mcl_mesh_build(L.ptr(points), len(points), C.byref(h)))
    return h


class MeshBatch:
    """Handle to a batch (or, with one mesh, a plain mesh) on the device."""

    def __init__(self, handle):
        self.handle = handle
        V, HE, T = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(L.lib().mcl_mesh_sizes(self.handle, C.byref(V), C.byref(HE), C.byref(T)))
        self.V, self.E, self.T = V.value, HE.value // 2, T.value
        n = C.c_int64()
        L.check(L.lib().mcl_batch_count(self.handle, C.byref(n)))
        self.count = n.value
        r = np.zeros((self.count, 4), np.int64)
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        for i in range(self.count):
            L.check(L.lib().mcl_batch_range(self.handle, i, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
            r[i] = (a.value, b.value, c.value, d.value)
        self.v0, self.nv, self.e0, self.ne = r[:, 0], r[:, 1], r[:, 2], r[:, 3]

    @classmethod
    def from_handles(cls, handles, destroy_inputs=True):
        arr = (C.c_void_p * len(handles))(*[h.value for h in handles])
        out = C.c_void_p()
        try:
            L.check(L.lib().mcl_batch_create(arr, len(handles), C.byref(out)))
        finally:
            if destroy_inputs:
                for h in handles:
                    L.lib().mcl_mesh_destroy(h)
        return cls(out)

    @classmethod
    def from_points(cls, point_sets):
        """Build every mesh on the GPU (each array is Morton-sorted in place) and
        batch them in the given order."""
        return cls.from_handles([build_mesh(p) for p in point_sets])

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            L.lib().mcl_mesh_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ------------------------------------------------------------------
    @property
    def positions_ptr(self):
        p = C.c_void_p()
        L.check(L.lib().mcl_mesh_positions(self.handle, C.byref(p)))
        return p.value

    def vertex_mesh_ptr(self):
        p = C.c_void_p()
        L.check(L.lib().mcl_batch_vertex_mesh(self.handle, C.byref(p)))
        return p.value

    def download(self, i):
        """(pos, v, he, t) of mesh i in the reference's AoS layout, ids from 0."""
        nv, ne = int(self.nv[i]), int(self.ne[i])
        pos = np.zeros((nv, 2), np.float32)
        v = np.zeros((nv, 2), np.int32)
        he = np.zeros((2 * ne, 4), np.int32)
        t = np.zeros((2 * (nv - 4) + 2, 1), np.int32)
        L.check(L.lib().mcl_batch_download_aos(self.handle, i, L.ptr(pos), L.ptr(v), L.ptr(he), L.ptr(t)))
        return pos, v, he, t

    def edges(self, i):
        """Sorted undirected edge list of mesh i (local ids)."""
        he = self.download(i)[2]
        a, b = he[0::2, 1], he[1::2, 1]
        e = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)
        return e[np.lexsort((e[:, 1], e[:, 0]))]

    def clone(self):
        out = C.c_void_p()
        L.check(L.lib().mcl_mesh_clone(self.handle, C.byref(out)))
        return MeshBatch(out)

    def set_tuning(self, blocks_per_sm=0, tail_items=0, removal_tile=None):
        L.check(L.lib().mcl_mesh_set_tuning(self.handle, int(blocks_per_sm), int(tail_items)))
        if removal_tile is not None:
            L.check(L.lib().mcl_mesh_set_removal_tile(self.handle, int(removal_tile)))

    def set_substeps(self, substeps):
        """Repair sub-steps per step (0: straight to removal and reinsertion)."""
        L.check(L.lib().mcl_mesh_set_substeps(self.handle, int(substeps)))

    def tuning(self):
        a, b, c, t = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.check(L.lib().mcl_mesh_get_tuning(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        L.check(L.lib().mcl_mesh_get_removal_tile(self.handle, C.byref(t)))
        return dict(blocks_per_sm=a.value, tail_items=b.value, max_blocks_per_sm=c.value, removal_tile=t.value)

    # -- stepping and motion -------------------------------------------------------
    def step(self, d, stream=None, stats=True):
        if stats:
            st = L.StepStats()
            L.check(L.lib().mcl_step(self.handle, L.ptr(d), _stream_ptr(stream), C.byref(st)))
            return st.as_dict()
        L.check(L.lib().mcl_step(self.handle, L.ptr(d), _stream_ptr(stream), None))
        return None

    def totals(self):
        st = L.StepStats()
        calls = C.c_int64()
        L.check(L.lib().mcl_mesh_totals(self.handle, C.byref(st), C.byref(calls)))
        d = st.as_dict()
        d["calls"] = calls.value
        return d

    def status(self, stream=None):
        st = L.StepStats()
        L.check(L.lib().mcl_mesh_last_status(self.handle, _stream_ptr(stream), C.byref(st)))
        return st.as_dict()

    def validate(self):
        out = np.zeros(8, np.int64)
        L.check(L.lib().mcl_mesh_validate(self.handle, L.ptr(out)))
        return out

    def walk(self, sigma, counter, d, seed=0, frozen=None, lo=0.0, hi=float(np.nextafter(np.float32(8192), 0)),
             stream=None, seeds=None):
        """Gaussian random-walk displacements into ``d`` (sigma and step counter
        per mesh, device arrays); ``seeds`` (uint64 device array, one key per
        mesh) replaces the keys seed + mesh index."""
        if seeds is not None:
            L.check(L.lib().mcl_walk_seeded(self.handle, L.ptr(sigma), L.ptr(frozen), L.ptr(seeds), L.ptr(counter),
                                            float(lo), float(hi), L.ptr(d), _stream_ptr(stream)))
            return
        L.check(L.lib().mcl_walk(self.handle, L.ptr(sigma), L.ptr(frozen), int(seed), L.ptr(counter), float(lo),
                                 float(hi), L.ptr(d), _stream_ptr(stream)))

    def settle(self, d, stream=None, sync=True):
        """Zero the displacements that would make two vertices of one mesh
        coincide; returns how many were zeroed (None when sync is False)."""
        n = C.c_int64()
        L.check(L.lib().mcl_settle_moves(self.handle, L.ptr(d), _stream_ptr(stream), C.byref(n) if sync else None))
        return n.value if sync else None

    def dla_freeze(self, r, frozen, stream=None, sync=True):
        """Aggregation contact in place on ``frozen`` (uint8 per vertex)."""
        n = C.c_int64()
        L.check(L.lib().mcl_dla_freeze(self.handle, L.ptr(r), L.ptr(frozen), _stream_ptr(stream),
                                       C.byref(n) if sync else None))
        return n.value if sync else None

    def set_active(self, meshes=None, stream=None):
        """Restrict the following steps and motion calls to these mesh indices
        (None or empty: all meshes)."""
        if meshes is None or len(meshes) == 0:
            L.check(L.lib().mcl_batch_set_active(self.handle, None, 0, _stream_ptr(stream)))
            return
        a = np.ascontiguousarray(meshes, np.int32)
        L.check(L.lib().mcl_batch_set_active(self.handle, L.ptr(a), len(a), _stream_ptr(stream)))

    def frnn_grid(self, r_host, r, max_frnn, out, lo=0.0, hi=8192.0, stream=None, sync=True):
        """The rows of ``frnn`` (ROW layout) from per-mesh grids; ``r_host`` and
        ``r`` hold the same per-mesh radii on the host and the device."""
        rh = np.ascontiguousarray(r_host, np.float32)
        ov = C.c_int64()
        L.check(L.lib().mcl_batch_frnn_grid(self.handle, L.ptr(rh), L.ptr(r), float(lo), float(hi), int(max_frnn),
                                            L.ptr(out), _stream_ptr(stream), C.byref(ov) if sync else None))
        return ov.value if sync else None

    def frnn_list(self, r, verts, max_frnn, out, layout=L.LAYOUT_ROW, stream=None, sync=True):
        ov = C.c_int64()
        L.check(L.lib().mcl_batch_frnn_list(self.handle, L.ptr(r), L.ptr(verts), int(verts.numel()), layout,
                                            int(max_frnn), L.ptr(out), _stream_ptr(stream),
                                            C.byref(ov) if sync else None))
        return ov.value if sync else None

    def one_ring_list(self, verts, max_ring, out, layout=L.LAYOUT_ROW, stream=None, sync=True):
        tr = C.c_int64()
        L.check(L.lib().mcl_one_ring_list(self.handle, L.ptr(verts), int(verts.numel()), layout, int(max_ring),
                                          L.ptr(out), _stream_ptr(stream), C.byref(tr) if sync else None))
        return tr.value if sync else None

    # -- queries ----------------------------------------------------------------------
    def frnn(self, r, max_frnn, out, layout=L.LAYOUT_ROW, stream=None, sync=True):
        """Mesh-walk FRNN with radius r[mesh] (device float array)."""
        ov = C.c_int64()
        L.check(L.lib().mcl_batch_frnn(self.handle, L.ptr(r), layout, int(max_frnn), L.ptr(out), _stream_ptr(stream),
                                       C.byref(ov) if sync else None))
        return ov.value if sync else None

    def one_ring(self, max_ring, out, layout=L.LAYOUT_COLUMN, stream=None, sync=True):
        tr = C.c_int64()
        L.check(L.lib().mcl_one_ring(self.handle, layout, int(max_ring), L.ptr(out), _stream_ptr(stream),
                                     C.byref(tr) if sync else None))
        return tr.value if sync else None


class StepPipeline:
    """The per-step pipeline of a batch of random-walk meshes: Gaussian walk
    (sigma per mesh, clamped to each mesh's box), coincident moves settled, the
    kinetic step, and per-mesh grid FRNN (radius per mesh) into ``out`` (ROW
    layout, ``max_frnn`` slots per vertex) -- captured once in a CUDA graph of
    ``steps_per_graph`` steps and replayed.  Walk counters advance on the
    device, so every replay draws new steps.  A step reads the positions from
    one of the mesh's two position buffers and writes the other, and a graph
    replays the buffers it was captured with, so it must hold an even number
    of steps (it then ends on the buffer it starts from).  With ``tune`` the launch shape
    (blocks per SM, single-block flip-round threshold, removal tile) is
    autotuned on clones first.  The reference steps one DeviceTriangulation
    per call (include/Device_Triangulation.h:324-351, :461-495)."""

    def __init__(self, batch, sigma, radius_host, radius, max_frnn, seed=0, steps_per_graph=2, stream=None,
                 tune=False, frnn=True):
        import torch

        if steps_per_graph < 2 or steps_per_graph % 2:
            raise ValueError("steps_per_graph must be even: a replay must end on the position buffer it starts from")

        self.torch = torch
        self.batch = batch
        self.sigma, self.radius, self.radius_host = sigma, radius, np.ascontiguousarray(radius_host, np.float32)
        self.max_frnn, self.seed, self.frnn = int(max_frnn), int(seed), frnn
        self.stream = stream or torch.cuda.Stream()
        dev = sigma.device
        self.counter = torch.zeros(batch.count, dtype=torch.int64, device=dev)
        self.d = torch.zeros((batch.V, 2), dtype=torch.float32, device=dev)
        self.out = torch.empty(batch.V * self.max_frnn, dtype=torch.int32, device=dev)
        self.tuned = None
        if tune:
            from .autotune import autotune

            tune_ctr = torch.zeros(batch.count, dtype=torch.int64, device=dev)

            def one(m, k, s):
                with torch.cuda.stream(s):
                    tune_ctr.fill_(1 << 40 | k)
                m.walk(self.sigma, tune_ctr, self.d, seed=self.seed, stream=s)
                m.settle(self.d, stream=s, sync=False)
                L.check(L.lib().mcl_step(m.handle, L.ptr(self.d), s.cuda_stream, None))

            self.tuned, _ = autotune(batch, one, stream=self.stream)
        # first calls allocate their scratch: run one step outside the capture
        self._launch()
        self.stream.synchronize()
        self.failed0 = batch.totals()["failed_launches"]
        before = batch.positions_ptr
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            for _ in range(steps_per_graph):
                self._launch()
        if batch.positions_ptr != before:
            raise RuntimeError("the captured steps do not end on the position buffer they start from")
        self.steps_per_graph = steps_per_graph

    def _launch(self):
        b, s = self.batch, self.stream
        b.walk(self.sigma, self.counter, self.d, seed=self.seed, stream=s)
        b.settle(self.d, stream=s, sync=False)
        L.check(L.lib().mcl_step(b.handle, L.ptr(self.d), s.cuda_stream, None))
        if self.frnn:
            b.frnn_grid(self.radius_host, self.radius, self.max_frnn, self.out, stream=s, sync=False)

    def replay(self):
        """Launch ``steps_per_graph`` steps (asynchronous on the pipeline's stream)."""
        self.graph.replay()

    def check(self):
        """Wait for the replays and raise if any captured step failed."""
        self.stream.synchronize()
        st = self.batch.status(self.stream)
        if st["status"] != 0 or self.batch.totals()["failed_launches"] != self.failed0:
            raise RuntimeError(f"a replayed step failed: {st}")
