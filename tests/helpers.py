"""Shared helpers for the tests: seeded synthetic inputs in the scaled unit
square (coordinates x 2^13, exact in float32), displacement generators and
comparison utilities."""
import numpy as np

SCALE = np.float32(8192.0)


def uniform_points(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.random((n, 2), dtype=np.float32) * SCALE).astype(np.float32)


def spacing(n):
    return float(SCALE) / np.sqrt(n)


def gaussian_disp(V, sigma, seed, clamp_pos=None):
    """N(0, sigma^2) per coordinate for vertices 4.., zero for the corners; when
    clamp_pos is given, the displacement is shrunk so pos+d stays in [0, 8192)."""
    rng = np.random.default_rng(seed)
    d = (rng.standard_normal((V, 2)) * sigma).astype(np.float32)
    d[:4] = 0
    if clamp_pos is not None:
        hi = np.nextafter(SCALE, np.float32(0))
        target = np.clip(clamp_pos + d, np.float32(0), hi).astype(np.float32)
        d = (target - clamp_pos).astype(np.float32)
        d[:4] = 0
        # clamping can stack points on the same spot (a box corner); exact
        # duplicates are rejected by the engine, so such points stay put
        for _ in range(64):
            new = (clamp_pos + d).astype(np.float32)
            _, inv, counts = np.unique(new, axis=0, return_inverse=True, return_counts=True)
            dup = counts[inv.ravel()] > 1
            if not dup.any():
                break
            d[dup] = 0
    return d


def taylor_green_disp(pos, n, frac=0.5):
    """Taylor-Green vortex u = (sin 2pi x cos 2pi y, -cos 2pi x sin 2pi y) on the
    unit torus, evaluated in float64 at the scaled positions; dt so that the
    largest displacement is `frac` x mean spacing.  Returned as float32 with
    zero for the corners; positions stay inside [0, 8192) by wrapping."""
    p = pos.astype(np.float64) / float(SCALE)
    u = np.sin(2 * np.pi * p[:, 0]) * np.cos(2 * np.pi * p[:, 1])
    v = -np.cos(2 * np.pi * p[:, 0]) * np.sin(2 * np.pi * p[:, 1])
    dt = frac * spacing(n)
    d = np.stack([u, v], 1) * dt
    new = (pos.astype(np.float64) + d) % float(SCALE)
    d32 = (new.astype(np.float32) - pos).astype(np.float32)
    d32[:4] = 0
    return d32


def csr_from_table(table, layout, V, M):
    """(counts, ids) from a reference-layout neighbour table."""
    t = np.asarray(table)
    if layout == 0:
        t = t.reshape(M, V)
        counts = t[0].astype(np.int32)
        rows = [t[1:1 + counts[i], i] for i in range(V)]
    else:
        t = t.reshape(V, M)
        counts = t[:, 0].astype(np.int32)
        rows = [t[i, 1:1 + counts[i]] for i in range(V)]
    return counts, rows


_CUDART = None


def cudart():
    """The CUDA runtime library already loaded by torch (for raw device copies)."""
    global _CUDART
    if _CUDART is None:
        import ctypes
        import glob
        import os

        import torch

        cands = []
        base = os.path.dirname(torch.__file__)
        cands += glob.glob(os.path.join(base, "lib", "libcudart.so*"))
        for sp in __import__("site").getsitepackages():
            cands += glob.glob(os.path.join(sp, "nvidia", "cuda_runtime", "lib", "libcudart.so*"))
        cands += glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        for c in cands:
            try:
                _CUDART = ctypes.CDLL(c)
                break
            except OSError:
                continue
        _CUDART.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return _CUDART


def d2h(ptr, count, dtype=np.int32):
    out = np.zeros(count, dtype)
    rc = cudart().cudaMemcpy(out.ctypes.data, ptr, out.nbytes, 2)
    assert rc == 0, rc
    return out


# -- the torus [2L, 3L)^2 of the periodic meshes (L = 8192) --------------------------

TORUS_L = 8192.0


def torus_points(n, seed, L=TORUS_L):
    """n distinct float32 points uniform in [2L, 3L)^2."""
    rng = np.random.default_rng(seed)
    x0 = 2.0 * L
    p = (x0 + rng.random((n, 2)) * L).astype(np.float32)
    p[p >= x0 + L] = np.nextafter(np.float32(x0 + L), np.float32(0))
    assert len(np.unique(p, axis=0)) == n
    return p


def torus_wrap(q, L=TORUS_L):
    """The engine's wrap of moved float32 coordinates into [2L, 3L)."""
    lo, hi = np.float32(2 * L), np.float32(3 * L)
    q = q.astype(np.float32).copy()
    up = q >= hi
    q[up] = q[up] - np.float32(L)
    dn = q < lo
    r = (q[dn] + np.float32(L)).astype(np.float32)
    r[r >= hi] = lo
    q[dn] = r
    return q


def eo_fields(eo):
    """(B, C, X1) offsets of periodic edge words (a nibble per component, bias 8)."""
    w = np.asarray(eo, np.int64)
    return [np.stack([((w >> (8 * k)) & 15) - 8, ((w >> (8 * k + 4)) & 15) - 8], -1) for k in range(3)]


def torus_settle(xy, d, ev, eo, drift, L=TORUS_L):
    """Reset to the common drift the moves of the vertices of faces the move
    would turn (or nearly turn) over, until none would: the periodic step
    restores Delaunay by flips only."""
    B, C, X1 = eo_fields(eo)
    D = B + X1
    a, b, c, dd = (ev[:, k] for k in range(4))
    d = d.copy()

    def orient(p, q, r):
        return (q[:, 0] - p[:, 0]) * (r[:, 1] - p[:, 1]) - (q[:, 1] - p[:, 1]) * (r[:, 0] - p[:, 0])

    tol = 1e-6 * L * L / len(xy)
    for _ in range(100):
        p = (xy + d).astype(np.float32).astype(np.float64)
        pa, pb, pc, pd = p[a], p[b] + B * L, p[c] + C * L, p[dd] + D * L
        bad = (orient(pa, pb, pc) <= tol) | (orient(pb, pa, pd) <= tol)
        if not bad.any():
            return d
        d[np.unique(ev[bad])] = drift
    raise RuntimeError("torus_settle did not converge")


def torus_faces_consistent(ev, en, eo):
    """t(h) + t(next h) + t(prev h) = 0 around every face and x(h) = t(h) + t(next h)."""
    B, C, X1 = eo_fields(eo)
    h = np.arange(2 * len(ev))
    e, s = h // 2, h % 2

    def t_of(hh):
        return np.where((hh % 2 == 1)[:, None], -B[hh // 2], B[hh // 2])

    nx = np.where(s == 0, en[e, 0], en[e, 2])
    pv = np.where(s == 0, en[e, 1], en[e, 3])
    x = np.where((s == 0)[:, None], C[e], X1[e])
    return bool((t_of(h) + t_of(nx) + t_of(pv) == 0).all() and (x == t_of(h) + t_of(nx)).all())
