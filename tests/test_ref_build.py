"""The oracle and the library's panel schedule against the reference's own code.

``oracle/_ref/oocdag_ref`` is the reference's ``oocdag.cpp`` (``Cholesky``, ``find_Yn``)
and ``oocquark.cpp`` (task generators and bodies) compiled unmodified by
``oracle/ref_build.py``, with host stand-ins for QUARK (program order), cuBLAS v2 and
MKL ``dpotrf_`` (SciPy's OpenBLAS).  It exists only where the reference tree does, so
these tests skip elsewhere.
"""
import json
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import ref_build

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

PANEL = re.compile(r"^bb (\d+) jb (\d+) YM (\d+) YN (\d+) Ym (\d+) Yn (\d+) ")
TASKS = re.compile(r"^tasks H2D (\d+) D2H (\d+) potrf (\d+) trsm (\d+) syrk (\d+) gemm (\d+)$")


@pytest.fixture(scope="module")
def ref_bin():
    if not ref_build.available():
        pytest.skip("reference tree not present: the compiled reference is built only where it is")
    return ref_build.build_ref()


def _parse(out: str):
    panels, tasks, info = [], None, None
    for line in out.splitlines():
        m = PANEL.match(line)
        if m:
            bb, jb, YM, YN, Ym, Yn = map(int, m.groups())
            panels.append((jb, Ym, Yn))
        m = TASKS.match(line)
        if m:
            tasks = dict(zip(("H2D", "D2H", "potrf", "trsm", "syrk", "gemm"), map(int, m.groups())))
        if line.startswith("info "):
            info = int(line.split()[1])
    return panels, tasks, info


def ref_plan(ref_bin, n, nb, memsize):
    r = subprocess.run([ref_bin, "plan", str(n), str(nb), str(memsize)], capture_output=True, text=True,
                       check=True, timeout=120)
    return _parse(r.stdout)


def ref_run(ref_bin, oracle_mod, A, nb, memsize):
    """Factor A (Fortran order) with the compiled reference; returns (A out, tasks, info)."""
    lda, n = A.shape
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "a.f64"), os.path.join(d, "l.f64")
        np.asarray(A, dtype=np.float64).T.tofile(fin)  # column-major bytes
        r = subprocess.run([ref_bin, "run", str(n), str(nb), str(lda), str(memsize), oracle_mod.openblas_path(),
                            "scipy_", fin, fout], capture_output=True, text=True, check=True, timeout=600)
        out = np.fromfile(fout, dtype=np.float64).reshape(n, lda).T.copy(order="F")
    _, tasks, info = _parse(r.stdout)
    return out, tasks, info


def test_reference_panel_plans_equal_golden_and_library(ref_bin, ooc):
    """find_Yn and the panel loop as compiled from oocdag.cpp:18-66,478-492."""
    plans = json.load(open(os.path.join(GOLDEN, "panel_plans.json")))
    for label, v in plans.items():
        got, _, _ = ref_plan(ref_bin, v["N"], v["NB"], v["memsize"])
        want = [tuple(p) for p in v["panels"]]
        assert got == want, label
        assert ooc.panel_plan(v["N"], v["NB"], v["memBlock"], nx=1) == want, label


def test_reference_task_counts_at_the_largest_geometry(ref_bin):
    # n=163840, nb=1024, a 24e9-byte budget: five panels, 669,920 gemm and 12,720 syrk
    # tasks, one potrf per tile column.
    panels, tasks, _ = ref_plan(ref_bin, 163840, 1024, 24_000_000_000)
    assert panels[:3] == [(0, 160, 17), (17, 143, 20), (37, 123, 24)] and panels[-1] == (94, 66, 66)
    assert tasks["gemm"] == 669_920 and tasks["syrk"] == 12_720
    assert tasks["potrf"] == 160 and tasks["trsm"] == 160 * 159 // 2


CASES = [  # (n, nb, budget in tiles, generator): one panel, several, ragged last tiles
    (96, 32, 10, "pdmatgen"),
    (300, 64, 14, "uniform"),
    (1000, 64, 40, "pdmatgen"),
    (1001, 128, 30, "uniform"),
    (777, 100, 30, "uniform"),
]


def _matrix(oracle_mod, n, kind):
    return oracle_mod.gen_pdmatgen(n, 100) if kind == "pdmatgen" else oracle_mod.gen_uniform(n, 100, float(n))


@pytest.mark.parametrize("n,nb,tiles,kind", CASES)
def test_oracle_equals_compiled_reference_bitwise(ref_bin, oracle_mod, n, nb, tiles, kind):
    """The oracle's threaded task graph gives the reference's factor bit for bit.

    Both run the same BLAS calls (one thread each) on the same tiles in an order that
    respects every tile's data hazards, so every tile sees the same operation sequence.
    """
    A = _matrix(oracle_mod, n, kind)
    mem = tiles * nb * nb * 8
    L_ref, tasks, info = ref_run(ref_bin, oracle_mod, A, nb, mem)
    assert info == 0
    for nthreads in (0, 4):
        L_orc = A.copy(order="F")
        _, info_o, _ = oracle_mod.cholesky(L_orc, nb, mem, nthreads, 2)
        assert info_o == 0
        np.testing.assert_array_equal(L_orc, L_ref)
    # the upper triangle is untouched, the lower one is a Cholesky factor
    np.testing.assert_array_equal(np.triu(L_ref, 1), np.triu(A, 1))
    Lr = np.tril(L_ref)
    assert np.abs(Lr @ Lr.T - A).max() <= 1e-12 * np.abs(A).max()


def test_compiled_reference_reports_not_positive_definite(ref_bin, oracle_mod):
    n, nb = 300, 64
    A = oracle_mod.gen_uniform(n, 3, float(n))
    A[200, 200] = -1.0
    _, _, info = ref_run(ref_bin, oracle_mod, A, nb, 14 * nb * nb * 8)
    # the reference prints the tile's info and carries on (oocquark.cpp:95); the first
    # failing tile is column block 3, whose local leading minor of order 9 fails
    assert info == 200 - 3 * nb + 1
    B = A.copy(order="F")
    _, info_o, _ = oracle_mod.cholesky(B, nb, 14 * nb * nb * 8, 0, 2)
    assert info_o == 201
