"""The allocation-free entry point, ooc_dpotrf_L_static, against ooc_dpotrf_L.

ooc_dpotrf_L_static exists for callers that cannot call cudaMalloc: processes whose
device memory belongs to another allocator (a framework's caching pool that has reserved
the GPU, where a new allocation fails or fragments it) and servers that must not let an
allocation or a free synchronize the device under their other streams.  Its panel buffer
is a fixed 64 MiB array in the library's static device memory, shared by every call.

This file is collected last on purpose, so that a run stopping at the first failure has
run every other test before it.  It must also pass alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ATOL_REL = 1e-12  # the factor tolerance of the other GPU parity tests


def _static_call(L, A, n, lda, nb):
    info = ctypes.c_int(-1)
    rc = L.ooc_dpotrf_L_static(ctypes.c_void_p(A.ctypes.data), n, lda, nb, None, ctypes.byref(info))
    return rc, info.value


def test_static_entry_matches_existing_entry_on_two_calls(oracle_mod, ooc, handle):
    L = ooc.load()
    n, nb = 6000, 256  # 24 tile rows: several left-looking panels inside the 64 MiB array
    for seed in (1, 2):  # two calls in a row: the second reuses what the first left behind
        A = oracle_mod.gen_uniform(n, seed, float(n))
        ref = A.copy(order="F")
        r = handle.dpotrf_L(ref, n, n, nb, 64 << 20)  # the existing entry point
        got = A.copy(order="F")
        rc, info = _static_call(L, got, n, n, nb)
        assert rc == 0, L.ooc_last_error_string()
        assert info == 0 == r.info
        Lr = np.tril(ref)
        np.testing.assert_allclose(np.tril(got), Lr, rtol=0, atol=ATOL_REL * np.abs(Lr).max())
        np.testing.assert_array_equal(np.triu(got, 1), np.triu(A, 1))


def test_static_entry_reports_info_then_recovers(oracle_mod, ooc, handle):
    L = ooc.load()
    n, nb = 3000, 256
    A = oracle_mod.gen_uniform(n, 4, float(n))
    bad = A.copy(order="F")
    bad[1700, 1700] = -2.0
    rc, info = _static_call(L, bad, n, n, nb)
    assert rc == 0 and info == 1701
    # the status word left set by the failed call is cleared by the next one
    ref = A.copy(order="F")
    handle.dpotrf_L(ref, n, n, nb, 64 << 20)
    got = A.copy(order="F")
    rc, info = _static_call(L, got, n, n, nb)
    assert rc == 0 and info == 0
    Lr = np.tril(ref)
    np.testing.assert_allclose(np.tril(got), Lr, rtol=0, atol=ATOL_REL * np.abs(Lr).max())


def test_static_entry_rejects_sizes_beyond_its_array(ooc, handle):
    L = ooc.load()
    n, nb = 40000, 256  # needs ~313 tiles of 512 KiB; the array holds 128
    A = np.zeros((1, 1))  # never touched: the size check comes first
    info = ctypes.c_int(-1)
    rc = L.ooc_dpotrf_L_static(ctypes.c_void_p(A.ctypes.data), n, n, nb, None, ctypes.byref(info))
    assert rc == ooc.OOC_ERR_BUDGET
    assert b"static panel buffer" in L.ooc_last_error_string()


def test_static_entry_device_matrix_on_a_caller_stream(oracle_mod, ooc, handle):
    """A already in device memory (a torch tensor: the copies become device-to-device) on a
    stream the caller created, then a failing matrix on the device that stops early."""
    import torch

    L = ooc.load()
    n, nb = 2500, 256
    A = oracle_mod.gen_uniform(n, 9, float(n))
    ref = A.copy(order="F")
    assert handle.dpotrf_L(ref, n, n, nb, 64 << 20).info == 0
    s = torch.cuda.Stream()
    T = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # row-major (n, n) == column-major A
    torch.cuda.synchronize()
    info = ctypes.c_int(-1)
    rc = L.ooc_dpotrf_L_static(ctypes.c_void_p(T.data_ptr()), n, n, nb, ctypes.c_void_p(s.cuda_stream),
                               ctypes.byref(info))
    assert rc == 0, L.ooc_last_error_string()
    assert info.value == 0
    got = np.asfortranarray(T.cpu().numpy().T)
    Lr = np.tril(ref)
    np.testing.assert_allclose(np.tril(got), Lr, rtol=0, atol=ATOL_REL * np.abs(Lr).max())
    np.testing.assert_array_equal(np.triu(got, 1), np.triu(A, 1))
    bad = A.copy(order="F")
    bad[1900, 1900] = -4.0
    Tb = torch.from_numpy(np.ascontiguousarray(bad.T)).cuda()
    torch.cuda.synchronize()
    rc = L.ooc_dpotrf_L_static(ctypes.c_void_p(Tb.data_ptr()), n, n, nb, ctypes.c_void_p(s.cuda_stream),
                               ctypes.byref(info))
    assert rc == 0 and info.value == 1901


def test_static_entry_at_its_largest_order(oracle_mod, ooc, handle):
    # n=16384 at nb=256 needs exactly the array's 128 tiles for its first panel
    L = ooc.load()
    n, nb = 16384, 256
    A = oracle_mod.gen_uniform(n, 12, float(n))
    got = A.copy(order="F")
    rc, info = _static_call(L, got, n, n, nb)
    assert rc == 0, L.ooc_last_error_string()
    assert info == 0
    ref = A.copy(order="F")
    assert handle.dpotrf_L(ref, n, n, nb, 1 << 30).info == 0
    Lr = np.tril(ref)
    np.testing.assert_allclose(np.tril(got), Lr, rtol=0, atol=ATOL_REL * np.abs(Lr).max())
