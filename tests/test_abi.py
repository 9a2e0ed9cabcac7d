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
