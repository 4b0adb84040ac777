"""Seeded synthetic workloads with the shapes of the reference's benchmark
configurations (no dataset is involved).  Coordinates live in the unit square
scaled by 2^13 (exact in float32): the reference's CPU point location needs
inputs of magnitude >~ 1e3 next to its +-1e7 bounding square, and every exact
orientation / incircle sign and every float distance comparison is unchanged
by a power-of-two scale."""
import numpy as np

SCALE = np.float32(8192.0)


def uniform_points(n, seed):
    """n distinct float32 points i.i.d. uniform in [0, 8192)^2 (the unit square
    scaled by 2^13); the rare exact duplicates of the 2^24-per-axis grid are
    redrawn, since coincident points have no triangulation."""
    rng = np.random.default_rng(seed)
    p = (rng.random((n, 2), dtype=np.float32) * SCALE).astype(np.float32)
    for _ in range(64):
        key = p.view(np.int64).ravel()
        _, first = np.unique(key, return_index=True)
        if len(first) == n:
            return p
        dup = np.ones(n, bool)
        dup[first] = False
        p[dup] = (rng.random((int(dup.sum()), 2), dtype=np.float32) * SCALE).astype(np.float32)
    raise RuntimeError("could not draw distinct points")


def mean_spacing(n):
    return float(SCALE) / np.sqrt(n)


def taylor_green_displacements(pos, n, steps, frac=0.5):
    """Displacements of `steps` forward-Euler steps of the Taylor-Green vortex
    u = (sin 2pi x cos 2pi y, -cos 2pi x sin 2pi y) on the unit torus, dt such
    that the largest displacement is `frac` x mean spacing.  The velocity is
    evaluated in float64 at the current float32 positions; the new position is
    wrapped into [0, 8192) and the float32 displacement is what the engine adds
    (pos += d in float32), so host and device follow identical trajectories.
    pos: (V, 2) float32 with the 4 bounding corners first.  Returns a list of
    (V, 2) float32 arrays."""
    p = pos.astype(np.float32).copy()
    dt = frac * mean_spacing(n)
    out = []
    L = float(SCALE)
    for _ in range(steps):
        q = p[4:].astype(np.float64) / L
        u = np.sin(2 * np.pi * q[:, 0]) * np.cos(2 * np.pi * q[:, 1])
        v = -np.cos(2 * np.pi * q[:, 0]) * np.sin(2 * np.pi * q[:, 1])
        new = (p[4:].astype(np.float64) + np.stack([u, v], 1) * dt) % L
        new32 = new.astype(np.float32)
        new32[new32 >= SCALE] = 0.0
        d = np.zeros_like(p)
        d[4:] = (new32 - p[4:]).astype(np.float32)
        p[4:] = (p[4:] + d[4:]).astype(np.float32)
        out.append(d)
    return out


def gaussian_displacements(pos, sigma, seed, steps):
    """Gaussian random walk N(0, sigma^2) per coordinate, clamped to the box,
    points that would land on an occupied spot stay put (exact duplicates are
    not a triangulation input)."""
    rng = np.random.default_rng(seed)
    p = pos.astype(np.float32).copy()
    hi = np.nextafter(SCALE, np.float32(0))
    out = []
    for _ in range(steps):
        d = (rng.standard_normal(p.shape) * sigma).astype(np.float32)
        d[:4] = 0
        tgt = np.clip(p + d, np.float32(0), hi).astype(np.float32)
        d = (tgt - p).astype(np.float32)
        d[:4] = 0
        for _ in range(64):
            new = (p + d).astype(np.float32)
            _, inv, cnt = np.unique(new, axis=0, return_inverse=True, return_counts=True)
            dup = cnt[inv.ravel()] > 1
            if not dup.any():
                break
            d[dup] = 0
        p = (p + d).astype(np.float32)
        out.append(d)
    return out


def taylor_green_displacements_device(pos, n, steps, frac=0.5, device="cuda"):
    """taylor_green_displacements on the GPU with torch (velocity in float64,
    positions and displacements in float32 with the same IEEE operations as
    the engine's pos += d), for long benchmark runs.  Returns a list of
    (V, 2) float32 device tensors."""
    import torch

    L = float(SCALE)
    dt = frac * mean_spacing(n)
    p = torch.as_tensor(pos, dtype=torch.float32, device=device).clone()
    out = []
    two_pi = 2.0 * np.pi
    for _ in range(steps):
        q = p[4:].double() / L
        u = torch.sin(two_pi * q[:, 0]) * torch.cos(two_pi * q[:, 1])
        v = -torch.cos(two_pi * q[:, 0]) * torch.sin(two_pi * q[:, 1])
        new = torch.remainder(p[4:].double() + torch.stack([u, v], 1) * dt, L)
        new32 = new.float()
        new32[new32 >= L] = 0.0
        d = torch.zeros_like(p)
        d[4:] = new32 - p[4:]
        p[4:] = p[4:] + d[4:]
        out.append(d)
    return out


def precision_points(n, seed):
    """Precision-stress point set (n float32 points, scaled by 2^13):
    50% on distinct sites of the 2048 x 1024 lattice (i/2048, j/1024), each
    coordinate jittered by U(-1e-7, 1e-7) in unit coordinates (about one ulp
    near 0.5, so many land back on the lattice: exactly cocircular quads);
    30% from 64 isotropic Gaussian clusters (sigma 1e-3, centres uniform,
    clamped to the square); 20% uniform.  Exact duplicates are redrawn as
    uniform points."""
    rng = np.random.default_rng(seed)
    n_lat = n // 2
    n_clu = (3 * n) // 10
    n_uni = n - n_lat - n_clu
    sites = rng.choice(2048 * 1024, size=n_lat, replace=False)
    i, j = sites % 2048, sites // 2048
    lat = np.stack([i / 2048.0, j / 1024.0], 1) + rng.uniform(-1e-7, 1e-7, (n_lat, 2))
    centres = rng.random((64, 2))
    c = rng.integers(0, 64, n_clu)
    clu = centres[c] + rng.normal(0.0, 1e-3, (n_clu, 2))
    uni = rng.random((n_uni, 2))
    hi = 1.0 - 2.0 ** -24
    p = np.clip(np.concatenate([lat, clu, uni]), 0.0, hi).astype(np.float32) * SCALE
    p = p.astype(np.float32)
    for _ in range(64):
        key = p.view(np.int64).ravel()
        _, first = np.unique(key, return_index=True)
        if len(first) == n:
            return p
        dup = np.ones(n, bool)
        dup[first] = False
        p[dup] = (rng.random((int(dup.sum()), 2), dtype=np.float32) * SCALE).astype(np.float32)
    raise RuntimeError("could not draw distinct points")
