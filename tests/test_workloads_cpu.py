"""The synthetic workloads behind the benchmark configurations: seeded, in the
scaled unit square, free of exact duplicates, with the shapes the
configurations name."""
import numpy as np

from mcleap_gb300 import workloads as W

L = float(W.SCALE)


def test_uniform_points_distinct_seeded_in_box():
    a = W.uniform_points(50_000, 3)
    b = W.uniform_points(50_000, 3)
    assert a.dtype == np.float32 and a.shape == (50_000, 2)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, W.uniform_points(50_000, 4))
    assert (a >= 0).all() and (a < L).all()
    assert len(np.unique(a.view(np.int64))) == len(a)


def test_precision_points_shape():
    n = 40_000
    p = W.precision_points(n, 9)
    assert p.shape == (n, 2) and p.dtype == np.float32
    assert (p >= 0).all() and (p < L).all()
    assert len(np.unique(p.view(np.int64))) == n
    # half of them within the jitter (1e-7 of the unit square) of a 2048 x 1024 lattice site
    u = p.astype(np.float64) / L
    dx = np.abs(u[:, 0] * 2048 - np.round(u[:, 0] * 2048)) / 2048
    dy = np.abs(u[:, 1] * 1024 - np.round(u[:, 1] * 1024)) / 1024
    on = (dx <= 2e-7) & (dy <= 2e-7)
    assert 0.49 * n <= on.sum() <= 0.52 * n
    # and some exactly on a site (cocircular quads)
    assert ((dx == 0) & (dy == 0)).sum() > 0


def test_taylor_green_displacements():
    n = 20_000
    pts = W.uniform_points(n, 5)
    pos = np.concatenate([np.zeros((4, 2), np.float32), pts])
    ds = W.taylor_green_displacements(pos, n, 3)
    h = W.mean_spacing(n)
    p = pos.copy()
    for d in ds:
        assert d.dtype == np.float32 and not d[:4].any()
        step = np.hypot(d[4:, 0], d[4:, 1])
        assert step.max() <= 0.5 * h * 1.0001  # |u| <= 1, dt = 0.5 h
        p = (p + d).astype(np.float32)
        assert (p[4:] >= 0).all() and (p[4:] < L).all()
    # the field has no normal component on the cell's sides: nothing wraps
    assert np.hypot(ds[0][4:, 0], ds[0][4:, 1]).max() < L / 2
    assert np.array_equal(ds[1], W.taylor_green_displacements(pos, n, 3)[1])


def test_gaussian_displacements_keep_points_distinct():
    n = 5_000
    pts = W.uniform_points(n, 8)
    pos = np.concatenate([np.array([[-1e7, -1e7], [1e7, -1e7], [1e7, 1e7], [-1e7, 1e7]], np.float32), pts])
    ds = W.gaussian_displacements(pos, 0.3 * W.mean_spacing(n), 2, 4)
    p = pos.copy()
    for d in ds:
        assert not d[:4].any()
        p = (p + d).astype(np.float32)
        assert len(np.unique(p, axis=0)) == len(p)
        assert (p[4:] >= 0).all() and (p[4:] < L).all()
