"""CPU tests of the C-ABI library: it builds for sm_103a, loads, exports every symbol the
headers declare, and its host-side panel planner agrees with the reference's."""
import ctypes
import json
import os
import subprocess

import pytest

from conftest import gpu_available

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_library_exports_every_header_symbol(ooc):
    L = ooc.load()
    names = ooc.header_functions()
    assert "ooc_dpotrf_L" in names and "Cholesky" in names and "ooc_pdpotrf_" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the dynamic symbol table (what a cgo / JNI / ctypes binding resolves against)
    out = subprocess.run(["nm", "-D", "--defined-only", ooc.lib_path()], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert not [n for n in names if n not in exported]


def test_build_targets_sm103a_only(ooc):
    from oocdag_gb300 import build as b

    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_host_panel_plan_matches_reference(ooc):
    plans = json.load(open(os.path.join(GOLDEN, "panel_plans.json")))
    for label, v in plans.items():
        got = ooc.panel_plan(v["N"], v["NB"], v["memBlock"], nx=1)
        assert got == [tuple(p) for p in v["panels"]], label


def test_double_buffered_plan_invariants(ooc):
    # Two X buffers: every panel's trapezoid plus 2*Ym tiles fits in the budget, the
    # panels tile the matrix, and the width never shrinks except for the last panel.
    for n, nb, mem in [(163840, 1024, 2861), (40960, 1024, 256), (1001, 128, 40), (65536, 512, 3072)]:
        plan = ooc.panel_plan(n, nb, mem, nx=2)
        bb = (n + nb - 1) // nb
        jb = 0
        for k, (j, Ym, Yn) in enumerate(plan):
            assert j == jb and Ym == bb - jb and 1 <= Yn <= Ym
            assert Ym * Yn - Yn * (Yn - 1) // 2 + 2 * Ym <= mem or Yn == Ym
            if 0 < k < len(plan) - 1:
                assert Yn >= plan[k - 1][2]
            jb += Yn
        assert jb == bb


def test_budget_too_small_is_reported(ooc):
    with pytest.raises(ooc.OocError) as e:
        ooc.panel_plan(4096, 256, 20, nx=1)
    assert e.value.code == ooc.OOC_ERR_BUDGET


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_no_gpu_fails_loudly(ooc):
    with pytest.raises(ooc.OocError) as e:
        ooc.Handle(0)
    assert e.value.code == ooc.OOC_ERR_NODEVICE


def test_entry_point_argument_checks_need_no_gpu(ooc):
    L = ooc.load()
    info = ctypes.c_int(0)
    # NULL handle -> argument 1 invalid; never a crash
    assert L.ooc_dpotrf_L(None, None, 10, 10, 4, 0, ctypes.byref(info), None) == -1
    assert L.ooc_set_option(None, 1, 2) == -1


def test_every_entry_point_checks_its_handle_first(ooc):
    """A NULL handle (or factor, or server) is argument 1 invalid (-1) at every entry point,
    and the destroy calls accept NULL; none of this touches a device."""
    from oocdag_gb300 import server

    L = ooc.load()
    b = ctypes.byref
    info, it = ctypes.c_int(0), ctypes.c_int(0)
    F = ctypes.c_void_p()
    d = ctypes.c_double(0)
    v = ctypes.c_int64(0)
    buf = (ctypes.c_double * 16)()
    ns = (ctypes.c_int * 1)(4)
    off = (ctypes.c_int64 * 1)(0)
    assert L.ooc_spotrf_L(None, None, 10, 10, 4, 0, b(info), None) == -1
    assert L.ooc_factor_create(None, buf, 4, 4, 4, ooc.PREC_BF16X3, b(F), b(info), None) == -1
    assert L.ooc_factor_create_gen(None, 4, 1, 1.0, 4, ooc.PREC_FP64, b(F), b(info), None) == -1
    assert L.ooc_solve_refine(None, None, buf, 4, buf, 4, buf, 4, 1, 1e-14, 5, b(it), b(d)) == -1
    assert L.ooc_solve_refine_gen(None, None, 1, 1.0, buf, 4, buf, 4, 1, 1e-14, 5, b(it), b(d)) == -1
    assert L.ooc_factor_solve(None, None, buf, 4, 1) == -1
    assert L.ooc_factor_copy_L(None, buf, 4) == -1
    assert L.ooc_factor_destroy(None) == ooc.OOC_OK
    assert L.ooc_dsyrk_ln(None, ooc.PREC_FP64, 4, 4, buf, 4, buf, 4) == -1
    assert L.ooc_gen_normal(None, buf, 4, 4, 1, 1) == -1
    assert L.ooc_dmatgen_pdmatgen(None, buf, 4, 4, 2) == -1
    assert L.ooc_dmatgen_uniform(None, buf, 4, 4, 1, 1.0) == -1
    assert L.ooc_dresidual(None, buf, 4, 4, 2, 1, 1.0, b(d)) == -1
    assert L.ooc_fp64_peak_probe(None, 1.0, b(d)) == -1
    assert L.ooc_batched_dposv(None, 1, ns, off, off, buf, buf, b(info), None, 0, b(d)) == -1
    assert L.ooc_batched_sposv(None, 1, ns, off, off, buf, buf, b(info), None, 0, b(d)) == -1
    assert L.ooc_get_option(None, ooc.OPT_TAIL_ORDER, b(v)) == -1
    assert L.ooc_get_option(None, ooc.OPT_COPY_STREAMS, b(v)) == -1
    assert L.ooc_set_option(None, ooc.OPT_COPY_STREAMS, 2) == -1
    sp = ctypes.c_void_p()
    assert L.ooc_get_stream(None, 3, b(sp)) == -1
    assert L.ooc_last_info(None) == 0
    assert L.ooc_destroy(None) == ooc.OOC_OK
    assert L.ooc_dpotrs_L(None, buf, 4, 4, 4, 0, buf, 4, 1) == -1
    assert L.ooc_dpotrf_L_static(None, 10, 10, 4, None, b(info)) == -1  # NULL matrix, n > 0
    S = server._lib()
    cnt, p64 = ctypes.c_int(0), ctypes.c_int64(0)
    assert S.ooc_server_create(None, b(ctypes.c_void_p())) == -1
    assert S.ooc_server_submit(None, b(server.Request(0, 64, 1, 2, 1, 0)), b(p64)) == -1
    assert S.ooc_server_poll(None, None, 0, b(cnt), 0) == -1
    assert S.ooc_server_solution(None, 1, buf, 4) == -1
    assert S.ooc_server_status(None, b(p64), b(p64), b(p64), b(p64)) == -1
    assert S.ooc_server_now(None) == 0.0
    assert S.ooc_server_destroy(None) == ooc.OOC_OK


def test_factor_bytes_accounting(ooc):
    """The device bytes a factor object needs (host arithmetic): 4 n^2 + O(n nb) for the
    reduced precisions (FP32 working matrix), more for FP64 (n^2 doubles plus the inverses)."""
    L = ooc.load()
    for n, nb in [(65536, 512), (4096, 256), (1001, 128)]:
        b16 = L.ooc_factor_bytes(n, nb, ooc.PREC_BF16X3)
        b32 = L.ooc_factor_bytes(n, nb, ooc.PREC_FP32)
        b64 = L.ooc_factor_bytes(n, nb, ooc.PREC_FP64)
        assert 4 * n * n <= b32 <= b16 < 4 * n * n + 64 * n * nb + (64 << 20)
        assert b64 >= 8 * n * n
    assert L.ooc_factor_bytes(65536, 512, ooc.PREC_BF16X3) < 18 * 10 ** 9  # fits beside A in 280 GB
    assert L.ooc_factor_bytes(0, 512, ooc.PREC_FP64) == 0 and L.ooc_factor_bytes(16, 0, ooc.PREC_FP64) == 0


def test_static_entry_size_limit_needs_no_gpu(ooc):
    """ooc_dpotrf_L_static checks the size against its 64 MiB array before any device call:
    the first panel needs 2*ceil(n/nb) tiles, so at nb=256 (128 tiles of 512 KiB) n=16384
    (64 tile columns) passes the check and n=16385 (65) is rejected."""
    L = ooc.load()
    info = ctypes.c_int(-1)
    dummy = (ctypes.c_double * 1)()
    rc = L.ooc_dpotrf_L_static(dummy, 16385, 16385, 256, None, ctypes.byref(info))
    assert rc == ooc.OOC_ERR_BUDGET
    msg = L.ooc_last_error_string()
    assert b"128 tiles" in msg and b"at least 130 needed" in msg, msg
    if not gpu_available():
        # past the size check the call needs a device, and says so
        rc = L.ooc_dpotrf_L_static(dummy, 16384, 16384, 256, None, ctypes.byref(info))
        assert rc == ooc.OOC_ERR_NODEVICE
