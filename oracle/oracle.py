"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this module: it is what the engine is compared with, never part of the
engine.  ``liboracle.so`` is the
restatement in this folder; ``_ref/libref.so`` (optional, built only where the
reference sources exist) is the reference's own HostTriangulation and
predicates.c, used to pin the restatement.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def build(ref=False):
    """Compile liboracle.so (and _ref/libref.so when ``ref`` and the sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_orient2d_batch.argtypes = [f32p, C.c_long, C.c_int, i32p]
        L.orc_incircle_batch.argtypes = [f32p, C.c_void_p, C.c_long, C.c_int, i32p]
        L.orc_exact_stats.argtypes = [u64p]
        L.orc_morton_sort.argtypes = [f32p, C.c_long]
        L.orc_morton_key.argtypes = [C.c_float, C.c_float]
        L.orc_morton_key.restype = C.c_ulonglong
        L.orc_mesh_build.argtypes = [f32p, C.c_long, C.c_int]
        L.orc_mesh_build.restype = C.c_void_p
        L.orc_mesh_import.argtypes = [f32p, C.c_long, i32p, i32p, C.c_long, i32p, C.c_long, C.c_int]
        L.orc_mesh_import.restype = C.c_void_p
        L.orc_mesh_free.argtypes = [C.c_void_p]
        L.orc_mesh_set_mode.argtypes = [C.c_void_p, C.c_int]
        L.orc_mesh_counts.argtypes = [C.c_void_p, i64p]
        L.orc_mesh_export.argtypes = [C.c_void_p, f32p, i32p, i32p, i32p]
        L.orc_mesh_set_positions.argtypes = [C.c_void_p, f32p]
        L.orc_mesh_move.argtypes = [C.c_void_p, f32p]
        L.orc_mesh_edges.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_mesh_edges.restype = C.c_long
        L.orc_mesh_check.argtypes = [C.c_void_p, C.c_int, i32p]
        L.orc_ref_untangle_pass.argtypes = [C.c_void_p]
        L.orc_ref_delonize.argtypes = [C.c_void_p]
        L.orc_ref_kinetic_step.argtypes = [C.c_void_p, f32p, i64p]
        L.orc_ref_one_ring.argtypes = [C.c_void_p, C.c_int, i32p, C.c_long]
        L.orc_ref_one_ring.restype = C.c_long
        L.orc_ref_frnn.argtypes = [C.c_void_p, C.c_int, C.c_float, i32p, C.c_long]
        L.orc_ref_frnn.restype = C.c_long
        L.orc_ref_frnn_all.argtypes = [C.c_void_p, C.c_float, i32p, i32p, C.c_long]
        L.orc_ref_frnn_all.restype = C.c_long
        L.orc_frnn_brute.argtypes = [f32p, C.c_long, C.c_float, C.c_int, C.c_float, i32p, i32p, C.c_long]
        L.orc_frnn_brute.restype = C.c_long
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's own code compiled here, or None where it cannot be built."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            return None
        R = C.CDLL(path)
        R.ref_build.argtypes = [f32p, C.c_long]
        R.ref_build.restype = C.c_void_p
        R.ref_free.argtypes = [C.c_void_p]
        R.ref_counts.argtypes = [C.c_void_p, i64p]
        R.ref_export.argtypes = [C.c_void_p, f32p, i32p, i32p, i32p]
        R.ref_move_all.argtypes = [C.c_void_p, f32p]
        R.ref_untangle.argtypes = [C.c_void_p]
        R.ref_delonize.argtypes = [C.c_void_p]
        R.ref_one_ring.argtypes = [C.c_void_p, C.c_int, i32p, C.c_long]
        R.ref_one_ring.restype = C.c_long
        R.ref_frnn.argtypes = [C.c_void_p, C.c_int, C.c_float, i32p, C.c_long]
        R.ref_frnn.restype = C.c_long
        for fn in ("ref_helpers_orient", "ref_shewchuk_orient", "ref_helpers_incircle",
                   "ref_shewchuk_incircle"):
            getattr(R, fn).argtypes = [f32p, C.c_long, i32p]
        _REF = R
    return _REF


# ---------------------------------------------------------------------------
def orient2d(pts6, mode=1):
    pts6 = np.ascontiguousarray(pts6, dtype=np.float32).reshape(-1, 6)
    out = np.zeros(len(pts6), np.int32)
    lib().orc_orient2d_batch(pts6.ravel(), len(pts6), mode, out)
    return out


def incircle(pts8, mode=1, ids=None):
    """mode 0 = reference FP64, 1 = exact, 2 = exact with symbolic perturbation."""
    pts8 = np.ascontiguousarray(pts8, dtype=np.float32).reshape(-1, 8)
    out = np.zeros(len(pts8), np.int32)
    if ids is not None:
        ids = np.ascontiguousarray(ids, dtype=np.int32).reshape(-1, 4)
        ptr = ids.ctypes.data
    else:
        ptr = None
    lib().orc_incircle_batch(pts8.ravel(), ptr, len(pts8), mode, out)
    return out


def exact_stats(reset=False):
    out = np.zeros(5, np.uint64)
    lib().orc_exact_stats(out)
    if reset:
        lib().orc_exact_stats_reset()
    return dict(zip(["orient_calls", "orient_exact", "incircle_calls", "incircle_exact", "sos_used"],
                    out.tolist()))


def morton_sort(xy):
    """The reference's Morton order (std::sort, include/Host_Triangulation.h:287-300)."""
    a = np.ascontiguousarray(xy, dtype=np.float32).copy()
    lib().orc_morton_sort(a.ravel(), len(a))
    return a


class Mesh:
    """Oracle half-edge mesh in the reference's AoS interchange layout."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def build(cls, xy, exact=True):
        """Insert xy (already in id order) into the bounding square; id = 4 + row."""
        a = np.ascontiguousarray(xy, dtype=np.float32)
        return cls(lib().orc_mesh_build(a.ravel(), len(a), 1 if exact else 0))

    @classmethod
    def from_aos(cls, pos, v, he, t, exact=True):
        pos = np.ascontiguousarray(pos, np.float32)
        v = np.ascontiguousarray(v, np.int32)
        he = np.ascontiguousarray(he, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        return cls(lib().orc_mesh_import(pos.ravel(), len(pos), v.ravel(), he.ravel(), len(he),
                                         t.ravel(), len(t), 1 if exact else 0))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_free(self.h)
            self.h = None

    def set_exact(self, exact):
        lib().orc_mesh_set_mode(self.h, 1 if exact else 0)

    def counts(self):
        out = np.zeros(5, np.int64)
        lib().orc_mesh_counts(self.h, out)
        return dict(V=int(out[0]), HE=int(out[1]), T=int(out[2]), error=int(out[3]), flips=int(out[4]))

    def aos(self):
        c = self.counts()
        pos = np.zeros((c["V"], 2), np.float32)
        v = np.zeros((c["V"], 2), np.int32)
        he = np.zeros((c["HE"], 4), np.int32)
        t = np.zeros((c["T"], 1), np.int32)
        lib().orc_mesh_export(self.h, pos.ravel(), v.ravel(), he.ravel(), t.ravel())
        return pos, v, he, t

    def positions(self):
        return self.aos()[0]

    def set_positions(self, pos):
        lib().orc_mesh_set_positions(self.h, np.ascontiguousarray(pos, np.float32).ravel())

    def move(self, d):
        lib().orc_mesh_move(self.h, np.ascontiguousarray(d, np.float32).ravel())

    def edges(self):
        n = lib().orc_mesh_edges(self.h, None)
        out = np.zeros((n, 2), np.int32)
        lib().orc_mesh_edges(self.h, out.ctypes.data)
        return out

    def check(self, exact=True):
        out = np.zeros(4, np.int32)
        lib().orc_mesh_check(self.h, 1 if exact else 0, out)
        return dict(zip(["non_delaunay", "creased", "inverted_faces", "zero_faces"], out.tolist()))

    def untangle_pass(self):
        return bool(lib().orc_ref_untangle_pass(self.h))

    def delonize(self):
        return bool(lib().orc_ref_delonize(self.h))

    def kinetic_step_ref(self, d):
        out = np.zeros(5, np.int64)
        lib().orc_ref_kinetic_step(self.h, np.ascontiguousarray(d, np.float32).ravel(), out)
        return dict(untangle_passes=int(out[0]), untangle_flips=int(out[1]),
                    delonize_flips=int(out[2]), seconds=out[3] * 1e-6, capped=bool(out[4]))

    def one_ring_ref(self, v):
        buf = np.zeros(4096, np.int32)
        n = lib().orc_ref_one_ring(self.h, v, buf, len(buf))
        return buf[:n].copy()

    def frnn_ref(self, v, r):
        buf = np.zeros(1 << 16, np.int32)
        n = lib().orc_ref_frnn(self.h, v, r, buf, len(buf))
        return buf[:n].copy()

    def frnn_ref_all(self, r):
        V = self.counts()["V"]
        counts = np.zeros(V, np.int32)
        cap = V * 64
        while True:
            ids = np.zeros(cap, np.int32)
            tot = lib().orc_ref_frnn_all(self.h, r, counts, ids, cap)
            if tot <= cap:
                return counts, ids[:tot]
            cap = tot


def frnn_brute(xy, r, periodic=False, L=0.0):
    """Sorted fixed-radius neighbour lists (CSR) by the float formula of the reference."""
    xy = np.ascontiguousarray(xy, np.float32)
    n = len(xy)
    counts = np.zeros(n, np.int32)
    cap = max(16, n * 32)
    while True:
        ids = np.zeros(cap, np.int32)
        tot = lib().orc_frnn_brute(xy.ravel(), n, r, 1 if periodic else 0, L, counts, ids, cap)
        if tot <= cap:
            return counts, ids[:tot]
        cap = tot


def ring_sets_from_edges(edges, V):
    """Sorted neighbour lists (CSR) of every vertex from an undirected edge list."""
    e = np.asarray(edges, np.int64)
    a = np.concatenate([e[:, 0], e[:, 1]])
    b = np.concatenate([e[:, 1], e[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    counts = np.bincount(a, minlength=V).astype(np.int32)
    return counts, b.astype(np.int32)


def settle_moves(pos, d, comp=None, fixed=None):
    """The coincident-move rule restated on the host: start with every vertex at
    fl(pos + d) (fixed vertices at pos); while two vertices of one component sit
    at the same point, every moving one among them gets d = 0; repeat.  Returns
    the settled displacements."""
    pos = np.ascontiguousarray(pos, np.float32)
    d = np.array(d, np.float32, copy=True)
    n = len(pos)
    comp = np.zeros(n, np.int64) if comp is None else np.asarray(comp, np.int64)
    fixed = np.zeros(n, bool) if fixed is None else np.asarray(fixed, bool)
    d[fixed] = 0
    for _ in range(n + 1):
        cand = (pos + d).astype(np.float32)
        cand[cand == 0] = 0  # -0 and +0 are one point
        key = np.stack([comp, cand[:, 0].view(np.int32).astype(np.int64),
                        cand[:, 1].view(np.int32).astype(np.int64)], 1)
        _, inv, counts = np.unique(key, axis=0, return_inverse=True, return_counts=True)
        shared = counts[inv.ravel()] > 1
        moving = (d[:, 0] != 0) | (d[:, 1] != 0)
        back = shared & moving & ~fixed
        if not back.any():
            return d
        d[back] = 0
    raise RuntimeError("settle_moves did not converge")
