"""CPU-side checks of the engine library: it loads, exports every symbol the C
header declares, and its predicate ladder (run on the host, same source as the
device code) agrees with the golden exact signs."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mcl_gb300.h")
G = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def L():
    from mcleap_gb300 import _lib
    from mcleap_gb300 import build as B

    B.build()
    return _lib


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(mcl_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "mcl_step" in syms and "mcl_mesh_build" in syms and "mcl_grid_frnn" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol(L):
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (mcl_[a-z0-9_]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    lib = L.lib()
    for s in declared_symbols():
        assert getattr(lib, s) is not None
    assert set(L.EXPORTS) <= exported


def test_status_strings(L):
    lib = L.lib()
    assert lib.mcl_status_string(0) == b"ok"
    for code in range(1, 9):
        assert lib.mcl_status_string(code) != b"unknown status"


def test_host_ladder_orient_matches_golden(L):
    g = np.load(os.path.join(G, "predicates.npz"))
    sign, stage = L.predicates_host(0, g["orient_pts"])
    assert np.array_equal(sign, g["orient_exact"])
    assert (stage == 2).sum() > 0 and (stage == 0).sum() > 0 and (stage >= 0).all()


def test_host_ladder_incircle_matches_golden(L):
    g = np.load(os.path.join(G, "predicates.npz"))
    sign, stage = L.predicates_host(1, g["incircle_pts"])
    assert np.array_equal(sign, g["incircle_exact"])
    assert (stage >= 0).all()
    # random quads are decided by the FP32 filter almost always
    rnd = stage[:1500]
    assert (rnd == 0).mean() > 0.99


def test_host_ladder_sos_matches_oracle(L):
    rng = np.random.default_rng(11)
    n = 3000
    base = rng.integers(0, 64, (n, 2)).astype(np.float32) * 4
    sq = np.stack([base, base + [4, 0], base + [4, 4], base + [0, 4]], 1).astype(np.float32)
    for k in range(n):
        sq[k] = sq[k][rng.permutation(4)]
    pts = sq.reshape(n, 8)
    ids = np.stack([rng.choice(1000, 4, replace=False) for _ in range(n)]).astype(np.int32)
    sign, stage = L.predicates_host(2, pts, ids)
    ref = O.incircle(pts, 2, ids)
    assert np.array_equal(sign, ref)
    assert (stage == 3).all() and (sign != 0).all()


def test_host_ladder_near_degenerate(L):
    # one-ulp perturbations of cocircular and collinear sets, and huge coordinates
    g = np.load(os.path.join(G, "predicates.npz"))
    p = g["incircle_pts"].copy()
    rng = np.random.default_rng(2)
    idx = rng.integers(0, 8, len(p))
    p[np.arange(len(p)), idx] = np.nextafter(p[np.arange(len(p)), idx], np.float32(np.inf))
    sign, stage = L.predicates_host(1, p)
    assert np.array_equal(sign, O.incircle(p, 1))
    assert (stage >= 0).all()
