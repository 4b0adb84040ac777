"""Regenerate the golden fixtures in this folder from the reference itself.

Runs the reference's own HostTriangulation and Shewchuk's predicates.c, compiled
from the reference sources by ``make -C oracle ref`` (oracle/_ref/libref.so).
Only possible where the reference sources exist; the fixtures are committed so
the tests never need the reference at run time.

    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402


def ref_build(R, xy):
    a = np.ascontiguousarray(xy, np.float32).copy()
    h = R.ref_build(a.ravel(), len(a))
    return h, a


def ref_aos(R, h):
    c = np.zeros(3, np.int64)
    R.ref_counts(h, c)
    V, HE, T = (int(x) for x in c)
    pos = np.zeros((V, 2), np.float32)
    v = np.zeros((V, 2), np.int32)
    he = np.zeros((HE, 4), np.int32)
    t = np.zeros((T, 1), np.int32)
    R.ref_export(h, pos.ravel(), v.ravel(), he.ravel(), t.ravel())
    return pos, v, he, t


def edges_of(he):
    a, b = he[0::2, 1], he[1::2, 1]
    e = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)
    return e[np.lexsort((e[:, 1], e[:, 0]))].astype(np.int32)


def aos_digest(aos):
    h = hashlib.sha256()
    for a in aos:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def gen_points(R, seed, n, bounds):
    out = np.zeros((n, 2), np.float32)
    R.ref_gen_points(seed, n, bounds, out.ravel())
    return out


def predicates(R, rng):
    recs6, recs8 = [], []
    n = 1500
    recs6.append(rng.random((n, 6), dtype=np.float32) * np.float32(8192))
    # exactly collinear lattice triples and their one-ulp perturbations
    a = rng.integers(0, 512, (n, 2)).astype(np.float32) * 4
    b = rng.integers(0, 512, (n, 2)).astype(np.float32) * 4
    k = rng.integers(-3, 4, (n, 1)).astype(np.float32)
    c = a + (b - a) * k
    col = np.concatenate([a, b, c], 1).astype(np.float32)
    recs6.append(col)
    pert = col.copy()
    idx = rng.integers(0, 6, n)
    pert[np.arange(n), idx] = np.nextafter(pert[np.arange(n), idx], np.float32(1e9))
    recs6.append(pert)
    recs8.append(rng.random((n, 8), dtype=np.float32) * np.float32(8192))
    base = rng.integers(0, 1000, (n, 2)).astype(np.float32) * 8
    sq = np.stack([base, base + [8, 0], base + [8, 8], base + [0, 8]], 1).astype(np.float32)
    recs8.append(sq.reshape(n, 8))
    jit = sq.reshape(n, 8).copy()
    idx = rng.integers(0, 8, n)
    jit[np.arange(n), idx] = np.nextafter(jit[np.arange(n), idx], np.float32(-1e9))
    recs8.append(jit)
    # quads touching the bounding-square corners
    corner = np.array([[-1e7, -1e7], [1e7, -1e7], [1e7, 1e7], [-1e7, 1e7]], np.float32)
    q = rng.random((n, 8), dtype=np.float32) * np.float32(8192)
    q[:, 0:2] = corner[rng.integers(0, 4, n)]
    recs8.append(q)
    p6 = np.ascontiguousarray(np.concatenate(recs6), np.float32)
    p8 = np.ascontiguousarray(np.concatenate(recs8), np.float32)
    o_ex = np.zeros(len(p6), np.int32)
    o_fp = np.zeros(len(p6), np.int32)
    i_ex = np.zeros(len(p8), np.int32)
    i_fp = np.zeros(len(p8), np.int32)
    R.ref_shewchuk_orient(p6.ravel(), len(p6), o_ex)
    R.ref_helpers_orient(p6.ravel(), len(p6), o_fp)
    R.ref_shewchuk_incircle(p8.ravel(), len(p8), i_ex)
    R.ref_helpers_incircle(p8.ravel(), len(p8), i_fp)
    np.savez_compressed(os.path.join(HERE, "predicates.npz"), orient_pts=p6, orient_exact=o_ex,
                        orient_ref_fp64=o_fp, incircle_pts=p8, incircle_exact=i_ex,
                        incircle_ref_fp64=i_fp)


def frnn_test(R):
    # tests/test_frnn.cu:13-112: 1000 points, mt19937{3}, U(-1000, 1000), r in 5..50
    pts = gen_points(R, 3, 1000, 1000.0)
    h, sorted_pts = ref_build(R, pts)
    pos, v, he, t = ref_aos(R, h)
    out = dict(points=pts, sorted_points=sorted_pts, edges=edges_of(he), he=he, v=v, t=t, pos=pos)
    buf = np.zeros(1 << 16, np.int32)
    ring_c, ring_i = [], []
    for vi in range(len(pos)):
        k = R.ref_one_ring(h, vi, buf, len(buf))
        ring_c.append(k)
        ring_i.extend(buf[:k].tolist())
    out["ring_counts"] = np.array(ring_c, np.int32)
    out["ring_ids"] = np.array(ring_i, np.int32)
    for r in (5, 10, 20, 30, 40, 50):
        cs, ids = [], []
        for vi in range(len(pos)):
            k = R.ref_frnn(h, vi, float(r), buf, len(buf))
            cs.append(k)
            ids.extend(sorted(buf[:k].tolist()))
        out[f"frnn_counts_r{r}"] = np.array(cs, np.int32)
        out[f"frnn_ids_r{r}"] = np.array(ids, np.int32)
    R.ref_free(h)
    np.savez_compressed(os.path.join(HERE, "test_frnn_1000.npz"), **out)


def closest_test(R):
    # tests/test_closest_neighbors.cu:13-89: N in {10, 100, 1000}, same generator;
    # expected = brute-force argmin over all vertices, strict <, first index wins
    out = {}
    for n in (10, 100, 1000):
        pts = gen_points(R, 3, n, 1000.0)
        h, _ = ref_build(R, pts)
        pos = ref_aos(R, h)[0]
        d = ((pos[:, None, :] - pos[None, :, :]).astype(np.float32) ** 2).sum(-1, dtype=np.float32)
        np.fill_diagonal(d, np.inf)
        out[f"points_{n}"] = pts
        out[f"pos_{n}"] = pos
        out[f"closest_{n}"] = d.argmin(1).astype(np.int32)
        R.ref_free(h)
    np.savez_compressed(os.path.join(HERE, "closest.npz"), **out)


def kinetic(R, rng):
    # 2000 points uniform in [0, 8192)^2 (the unit square scaled by 2^13), three
    # Gaussian random-walk steps with sigma = 0.1 x mean spacing.  For each step:
    # the displacement, the reference kinetic path's AoS digest (movePoint,
    # untangle until false, delonize), and the Delaunay edge set of the step's
    # positions from the reference's own builder, mapped back to the mesh's ids.
    n = 2000
    xy = (rng.random((n, 2), dtype=np.float32) * np.float32(8192)).astype(np.float32)
    h, sorted_pts = ref_build(R, xy)
    spacing = 8192.0 / np.sqrt(n)
    out = dict(sorted_points=sorted_pts, edges_step0=edges_of(ref_aos(R, h)[2]))
    for step in range(1, 4):
        d = (rng.standard_normal((n + 4, 2)) * 0.1 * spacing).astype(np.float32)
        d[:4] = 0
        R.ref_move_all(h, d.ravel())
        k = 0
        while R.ref_untangle(h) and k < 64:
            k += 1
        R.ref_delonize(h)
        aos = ref_aos(R, h)
        pos = aos[0]
        h2, srt = ref_build(R, pos[4:])
        he2 = ref_aos(R, h2)[2]
        # map the rebuilt mesh's ids (4 + Morton rank) back to the moving mesh's ids
        key = {(float(x), float(y)): i for i, (x, y) in enumerate(pos)}
        remap = np.array([0, 1, 2, 3] + [key[(float(x), float(y))] for x, y in srt], np.int32)
        e = edges_of(he2)
        e = remap[e]
        e = np.stack([e.min(1), e.max(1)], 1)
        e = e[np.lexsort((e[:, 1], e[:, 0]))].astype(np.int32)
        out[f"disp_step{step}"] = d
        out[f"dt_edges_step{step}"] = e
        out[f"ref_kinetic_digest_step{step}"] = np.array(aos_digest(aos))
        out[f"ref_untangle_passes_step{step}"] = np.array(k, np.int32)
        R.ref_free(h2)
    R.ref_free(h)
    np.savez_compressed(os.path.join(HERE, "kinetic_2000.npz"), **out)


def main():
    O.build(ref=True)
    R = O.ref_lib()
    if R is None:
        raise SystemExit("the reference build (oracle/_ref/libref.so) is not available")
    R.ref_gen_points.argtypes = [O.C.c_uint, O.C.c_long, O.C.c_float, O.f32p]
    rng = np.random.default_rng(20261203)
    predicates(R, rng)
    frnn_test(R)
    closest_test(R)
    kinetic(R, rng)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
