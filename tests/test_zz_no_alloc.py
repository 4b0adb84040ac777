"""The allocation-free grid neighbour entry point against the allocating one.

mcl_grid_frnn_noalloc serves callers that cannot allocate device memory (a host
framework that owns the whole GPU, a loop that must not block in an allocator):
its scratch is a fixed array in the library, shared by every call.  This test
calls it through the C ABI twice in a row, on different inputs, and checks each
result bit for bit against mcl_grid_create + mcl_grid_update + mcl_grid_frnn
(integer outputs and a permutation of float positions: the tolerance is zero).
It sits in a file of its own, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_POINTS = 262144


@pytest.fixture(scope="module")
def L():
    import torch

    from mcleap_gb300 import _lib
    from mcleap_gb300 import build as B

    assert torch.cuda.is_available()
    B.build()
    _lib.lib()
    return _lib


def allocating(L, pos, mn, cell, ncell, flags, r, max_nb):
    import torch

    n = len(pos)
    lib = L.lib()
    g = C.c_void_p()
    L.check(lib.mcl_grid_create(n, mn[0], mn[1], cell, cell, ncell, ncell, flags, C.byref(g)))
    try:
        d = torch.from_numpy(pos).cuda()
        L.check(lib.mcl_grid_update(g, d.data_ptr(), None, None))
        counts = torch.zeros(n, dtype=torch.int32, device="cuda")
        ids = torch.zeros(n * max_nb, dtype=torch.int32, device="cuda")
        ov = C.c_int64()
        L.check(lib.mcl_grid_frnn(g, d.data_ptr(), r, max_nb, counts.data_ptr(), ids.data_ptr(), None, C.byref(ov)))
        perm_ptr, start, count = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nx, ny = C.c_int(), C.c_int()
        L.check(lib.mcl_grid_tables(g, C.byref(perm_ptr), C.byref(start), C.byref(count), C.byref(nx), C.byref(ny)))
        torch.cuda.synchronize()
        from helpers import d2h

        perm_h = d2h(perm_ptr.value, n)
        return d.cpu().numpy(), perm_h, counts.cpu().numpy(), ids.cpu().numpy(), ov.value
    finally:
        lib.mcl_grid_destroy(g)


def no_alloc(L, pos, mn, cell, ncell, flags, r, max_nb):
    import torch

    n = len(pos)
    d = torch.from_numpy(pos).cuda()
    sorted_pos = torch.zeros_like(d)
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    ids = torch.zeros(n * max_nb, dtype=torch.int32, device="cuda")
    ov = C.c_int64()
    L.check(L.lib().mcl_grid_frnn_noalloc(d.data_ptr(), n, mn[0], mn[1], cell, cell, ncell, ncell, flags, r, max_nb,
                                          sorted_pos.data_ptr(), perm.data_ptr(), counts.data_ptr(), ids.data_ptr(),
                                          None, C.byref(ov)))
    torch.cuda.synchronize()
    # the input stays untouched
    assert np.array_equal(d.cpu().numpy(), pos)
    return sorted_pos.cpu().numpy(), perm.cpu().numpy(), counts.cpu().numpy(), ids.cpu().numpy(), ov.value


def same(a, b, max_nb):
    sa, pa, ca, ia, oa = a
    sb, pb, cb, ib, ob = b
    assert np.array_equal(sa, sb)
    assert np.array_equal(pa, pb)
    assert np.array_equal(ca, cb)
    n = len(ca)
    ia = ia.reshape(n, max_nb)
    ib = ib.reshape(n, max_nb)
    for i in range(n):
        assert np.array_equal(ia[i, :ca[i]], ib[i, :cb[i]])
    assert oa == ob


def test_no_alloc_matches_allocating_entry_point_twice(L):
    rng = np.random.default_rng(31)
    # call 1: 200k random points, 256 x 256 cells
    pos1 = (rng.random((200000, 2), dtype=np.float32) * np.float32(8192)).astype(np.float32)
    args1 = ((0.0, 0.0), 32.0, 256, 0, 20.0, 32)
    same(no_alloc(L, pos1, *args1), allocating(L, pos1, *args1), 32)
    # call 2 right after, on a smaller periodic lattice-like set and a finer
    # grid: stale contents from call 1 must not leak into the result
    xs, ys = np.meshgrid(np.arange(100), np.arange(90))
    pos2 = (np.stack([xs.ravel(), ys.ravel()], 1) * np.float32(0.5)).astype(np.float32)
    args2 = ((0.0, 0.0), 1.0, 64, 1, 1.0, 40)
    same(no_alloc(L, pos2, *args2), allocating(L, pos2, *args2), 40)


def test_no_alloc_rejects_oversize(L):
    import torch

    n = MAX_POINTS + 1
    d = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = L.lib().mcl_grid_frnn_noalloc(d.data_ptr(), n, 0.0, 0.0, 1.0, 1.0, 16, 16, 0, 1.0, 1, d.data_ptr(),
                                       out.data_ptr(), out.data_ptr(), out.data_ptr(), None, None)
    assert rc == L.MCL_ERR_CAPACITY
    assert b"262144" in L.lib().mcl_last_error()
    rc = L.lib().mcl_grid_frnn_noalloc(d.data_ptr(), 10, 0.0, 0.0, 1.0, 1.0, 1024, 1024, 0, 1.0, 1, d.data_ptr(),
                                       out.data_ptr(), out.data_ptr(), out.data_ptr(), None, None)
    assert rc == L.MCL_ERR_CAPACITY
