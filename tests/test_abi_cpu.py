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


# entry points taking a mesh, with the argument list after the mesh (all NULL /
# zero): each must refuse a NULL mesh with MCL_ERR_INVALID_ARGUMENT before it
# touches the device, so this runs without a GPU
NULL_MESH_CALLS = {
    "mcl_batch_count": 1, "mcl_batch_range": 5, "mcl_batch_vertex_mesh": 1, "mcl_batch_download_aos": 5,
    "mcl_batch_set_active": 3, "mcl_mesh_set_tuning": 2, "mcl_mesh_set_substeps": 1, "mcl_mesh_get_tuning": 3,
    "mcl_settle_moves": 3, "mcl_mesh_totals": 2, "mcl_debug_timeline": 1, "mcl_debug_insert_timeline": 1,
    "mcl_debug_counters": 2, "mcl_debug_state": 1, "mcl_mesh_validate": 1, "mcl_mesh_upload_aos": 1,
    "mcl_mesh_sizes": 3, "mcl_mesh_positions": 1, "mcl_mesh_copy_positions": 3, "mcl_mesh_download_aos": 4,
    "mcl_move": 2, "mcl_integrate": 3, "mcl_untangle": 2, "mcl_delaunay_restore": 2, "mcl_step": 3,
    "mcl_step_host": 3, "mcl_step_host_async": 3, "mcl_mesh_last_status": 2,
    "mcl_mesh_set_removal_tile": 1, "mcl_mesh_get_removal_tile": 1, "mcl_mesh_export_aos": 4,
    "mcl_walk_seeded": 8, "mcl_debug_remove_timeline": 1, "mcl_periodic_debug_timeline": 2,
}


def test_null_mesh_is_refused(L):
    import ctypes as C

    lib = L.lib()
    scalars = (C.c_int, C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_double)
    for name, nargs in NULL_MESH_CALLS.items():
        fn = getattr(lib, name)
        types = fn.argtypes or [C.c_void_p] * (nargs + 1)
        assert len(types) == nargs + 1, name
        args = [0 if t in scalars else None for t in types]
        assert args[0] is None
        assert fn(*args) == L.MCL_ERR_INVALID_ARGUMENT, name
    assert lib.mcl_mesh_destroy(None) == 0


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


def test_cpp_dropin_headers_compile_and_link(L, tmp_path):
    """The C++ drop-in headers compile with nvcc against the C ABI, and the
    reference-style driver program links against the library (not run here)."""
    from mcleap_gb300 import build as B

    exe = str(tmp_path / "test_dropin")
    cmd = [B.nvcc(), "-std=c++17", "-O0", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "test_dropin.cu"),
           "-L", os.path.dirname(L.LIB_PATH), "-lmcl_gb300", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.getsize(exe) > 0


def test_single_point_moves_refuse_the_bounding_corners():
    """moveFlipflop & co. leave ids 0..3 (the bounding square) alone and
    report False, before any device work."""
    import mcleap_gb300 as M

    ht = M.HostTriangulation()
    before = ht.m_pos.copy()
    for f in (ht.moveFlipflop, ht.moveFlipflopDelaunay, ht.moveUntangling, ht.moveUntanglingDelaunay):
        assert f(0, (1.0, 1.0)) is False and f(3, (1.0, 1.0)) is False and f(4, (1.0, 1.0)) is False
    assert np.array_equal(ht.m_pos, before)


def test_malformed_aos_meshes_are_refused_on_the_host(L):
    """mcl_mesh_create_from_aos validates the reference-layout arrays before any
    device work: each corruption of a valid mesh is refused with its reason."""
    import ctypes as C

    pts = np.random.default_rng(2).random((50, 2)).astype(np.float32) * 1000
    pos, v, he, t = (np.ascontiguousarray(a) for a in O.Mesh.build(pts, exact=True).aos())

    def create(pos, v, he, t):
        keep = [np.ascontiguousarray(a) for a in (pos, v, he, t)]
        view = L.AosView(*(L.ptr(a) for a in keep), len(keep[0]), len(keep[2]), len(keep[3]))
        h = C.c_void_p()
        rc = L.lib().mcl_mesh_create_from_aos(C.byref(view), C.byref(h))
        return rc, L.lib().mcl_last_error().decode()

    cases = []
    bad = he.copy(); bad[7, 0] = len(he) + 3
    cases.append((bad, v, "half-edge index out of range"))
    bad = he.copy(); bad[7, 0] = he[8, 0]
    cases.append((bad, v, "two half-edges share a next"))
    bad = he.copy(); bad[12, 1] = (he[12, 1] + 1) % len(pos)
    cases.append((bad, v, "inconsistent"))
    badv = v.copy(); badv[10, 1] = int(np.nonzero(he[:, 1] != 10)[0][0])
    cases.append((he, badv, "vertex he is not outgoing"))
    for h_, v_, why in cases:
        rc, msg = create(pos, v_, h_, t)
        assert rc == L.MCL_ERR_INVALID_ARGUMENT and why in msg, (rc, msg, why)
    odd = he[:-1]
    rc, msg = create(pos, v, odd, t)
    assert rc == L.MCL_ERR_INVALID_ARGUMENT and "bad sizes" in msg


PERIODIC_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "mcleap/Periodic_Triangulation.h"
int main() {
  std::vector<glm::vec2> pts;
  for (int i = 0; i < 1000; ++i) pts.push_back(glm::vec2(16384.f + (i * 37 % 1000) * 8.f, 16384.f + i * 8.f));
  PeriodicTriangulation pt(pts, 8192.f);
  glm::vec2* d = nullptr;
  int *ring = nullptr, *nb = nullptr, *cl = nullptr;
  uint8_t* offs = nullptr;
  pt.step(d);
  pt.step_host(std::vector<glm::vec2>(pts.size()));
  pt.oneRing<32>(ring, offs);
  pt.oneRing2<32>(ring, offs);
  pt.closestNeighbors<32>(ring, offs, cl);
  pt.getFRNN<32, 64>(20.f, ring, nb);
  std::vector<glm::vec2> pos;
  std::vector<int32_t> ev, en;
  std::vector<uint32_t> eo;
  pt.transferToHost(pos, ev, en, eo);
  std::printf("%p %lld\n", (void*)pt.positions(), (long long)pt.E);
  return 0;
}
"""


def test_periodic_cpp_header_compiles_and_links(L, tmp_path):
    from mcleap_gb300 import build as B

    src = tmp_path / "periodic_dropin.cu"
    src.write_text(PERIODIC_PROGRAM)
    exe = str(tmp_path / "periodic_dropin")
    cmd = [B.nvcc(), "-std=c++17", "-O0", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), str(src),
           "-L", os.path.dirname(L.LIB_PATH), "-lmcl_gb300", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
