"""Predicate sign maps: the reference's precision experiment
(experiments/floating_point_predicates_precision.cu:178-271) as counts.

Four points a, b, c, d on the unit circle, (-1, 0), (0, -1), (1, 0), (0, 1),
rotated by pi * rotation; d is perturbed by ((i - R/2) 2^-e, (j - R/2) 2^-e)
over an R x R grid, and the incircle sign of (a, b, c, d + perturbation) is
taken on every cell.  The reference draws three such maps as PNG files (its
FP64 determinant, Shewchuk's exact predicate, an angle test).  Here the
engine's own predicate ladder (FP32 filter, exact integer / FP64 / expansion
stages) runs on the GPU over the same grid, and the result is a count per
sign and per deciding stage, plus how many cells the reference's FP64
determinant (`matrix_incircle`, :88-102, restated in numpy with the same
operation order) gets a different sign on.  The engine takes float32 inputs:
the points are rounded to float32 before any predicate sees them, so for
e > 23 neighbouring cells collapse onto the same inputs.

    python -m mcleap_gb300.signmap --resolution 1024 --exponent 23 --rotation 0 \\
        [--ppm map.ppm]

prints one JSON line; --ppm also writes the engine's map as a binary PPM (red
positive, green zero, blue negative, like the reference's images)."""
import argparse
import json

import numpy as np

from . import _lib as L

STAGES = ("fp32", "fp64", "exact", "perturbation")


def quad_points(resolution, exponent, rotation):
    """(R*R, 8) float32 records (a, b, c, d + perturbation), cell (i, j) at
    row i * R + j (i perturbs x, j perturbs y, as in the reference)."""
    base = np.array([(-1.0, 0.0), (0.0, -1.0), (1.0, 0.0), (0.0, 1.0)])
    t = np.pi * rotation
    cs, sn = np.cos(t), np.sin(t)
    q = np.stack([base[:, 0] * cs - base[:, 1] * sn, base[:, 0] * sn + base[:, 1] * cs], 1)
    eps = 2.0 ** -exponent
    k = (np.arange(resolution, dtype=np.float64) - resolution // 2) * eps
    px, py = np.meshgrid(k, k, indexing="ij")
    pts = np.empty((resolution * resolution, 8), np.float32)
    pts[:, 0:2] = q[0]
    pts[:, 2:4] = q[1]
    pts[:, 4:6] = q[2]
    pts[:, 6] = (q[3, 0] + px).ravel()
    pts[:, 7] = (q[3, 1] + py).ravel()
    return pts


def reference_fp64_sign(pts8):
    """Sign of the reference's FP64 incircle determinant on the same inputs."""
    p = pts8.astype(np.float64)
    ax, ay, bx, by, cx, cy, dx, dy = (p[:, k] for k in range(8))
    a00, a01 = ax - dx, ay - dy
    a02 = a00 * a00 + a01 * a01
    a10, a11 = bx - dx, by - dy
    a12 = a10 * a10 + a11 * a11
    a20, a21 = cx - dx, cy - dy
    a22 = a20 * a20 + a21 * a21
    det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20)
    return np.sign(det).astype(np.int32)


def device_signs(pts8):
    """Engine incircle signs and deciding stages on the GPU."""
    import torch

    d = torch.from_numpy(np.ascontiguousarray(pts8)).cuda()
    sign = torch.empty(len(pts8), dtype=torch.int32, device="cuda")
    stage = torch.empty(len(pts8), dtype=torch.int32, device="cuda")
    L.check(L.lib().mcl_debug_predicates_device(1, d.data_ptr(), None, len(pts8), sign.data_ptr(),
                                                stage.data_ptr(), None))
    return sign.cpu().numpy(), stage.cpu().numpy()


def sign_map(resolution=512, exponent=23, rotation=0.0):
    """Counts of the engine's signs and stages over the grid, and of the cells
    where the reference's FP64 determinant has another sign."""
    pts = quad_points(resolution, exponent, rotation)
    sign, stage = device_signs(pts)
    ref = reference_fp64_sign(pts)
    counts = {
        "resolution": resolution, "exponent": exponent, "rotation": rotation,
        "positive": int((sign > 0).sum()), "zero": int((sign == 0).sum()), "negative": int((sign < 0).sum()),
        "stages": {name: int((stage == k).sum()) for k, name in enumerate(STAGES)},
        "reference_fp64_disagrees": int((ref != sign).sum()),
    }
    return counts, sign.reshape(resolution, resolution)


def write_ppm(path, grid):
    """Binary PPM of a sign grid: red > 0, green = 0, blue < 0; cell (i, j) at
    column i, row R-1-j (the reference flips its images vertically)."""
    r = grid.shape[0]
    img = np.zeros((r, r, 3), np.uint8)
    g = grid.T[::-1]
    img[..., 0] = (g > 0) * 254
    img[..., 1] = (g == 0) * 254
    img[..., 2] = (g < 0) * 254
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (r, r))
        f.write(img.tobytes())


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--resolution", type=int, default=1024)
    ap.add_argument("--exponent", type=int, default=23)
    ap.add_argument("--rotation", type=float, default=0.0)
    ap.add_argument("--ppm", default=None)
    a = ap.parse_args(argv)
    counts, grid = sign_map(a.resolution, a.exponent, a.rotation)
    if a.ppm:
        write_ppm(a.ppm, grid)
    print(json.dumps(counts), flush=True)


if __name__ == "__main__":
    main()
