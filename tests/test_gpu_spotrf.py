"""GPU tests of the FP32 entry ooc_spotrf_L and of the command-line driver.

FP32 factor: compared with the FP64 LAPACK factor of the same (FP32-representable)
matrix to FP32 accuracy, 2e-5 relative to max |L| at these sizes; LAPACK info exact for a
planted non-positive pivot; the upper triangle untouched.  Odd orders and leading
dimensions exercise the unaligned-panel path of the FP32 trailing update.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-5


def _spd32(n, seed):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n))
    return (M @ M.T / n + np.eye(n)).astype(np.float32)


@pytest.mark.parametrize("n,lda,nb", [(1001, 1001, 128), (1536, 1540, 256), (700, 703, 512), (64, 64, 64)])
def test_spotrf_device_matches_lapack(handle, n, lda, nb):
    import torch

    A = _spd32(n, n)
    Ap = np.full((n, lda), 7.0, dtype=np.float32)  # row i of Ap = column i of the column-major matrix
    Ap[:, :n] = A  # symmetric
    T = torch.from_numpy(Ap).cuda()
    r = handle.spotrf_L(T, n, lda, nb)
    assert r.info == 0
    got = T.cpu().numpy()[:, :n].T  # column-major view
    want = np.linalg.cholesky(A.astype(np.float64))
    assert np.abs(np.tril(got) - want).max() <= TOL * np.abs(want).max()
    np.testing.assert_array_equal(np.triu(got, 1), np.triu(A, 1))  # strict upper untouched
    np.testing.assert_array_equal(T.cpu().numpy()[:, n:], 7.0)  # padding untouched


def test_spotrf_host_and_info(handle):
    import scipy.linalg as sla

    n, nb = 900, 256
    A = np.asfortranarray(_spd32(n, 3))
    L = A.copy(order="F")
    r = handle.spotrf_L(L, n, n, nb)
    assert r.info == 0 and r.stats["seconds"] > 0
    want = np.linalg.cholesky(A.astype(np.float64))
    assert np.abs(np.tril(L) - want).max() <= TOL * np.abs(want).max()
    B = A.copy(order="F")
    B[500, 500] = -1.0
    r = handle.spotrf_L(B, n, n, nb)
    assert r.info == sla.lapack.spotrf(B, lower=1)[1] == 501


def test_cli_reference_interface():
    from oocdag_gb300 import build

    exe = build.CLI
    assert os.path.exists(exe)
    out = subprocess.run([exe, "3000", "256", "16", "--verify"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[0] == "N NB memsize(MB) streams time Gflops"
    f = lines[1].split()
    assert f[0] == "3000" and f[1] == "256" and float(f[4]) > 0 and float(f[5]) > 0
    res = float(lines[-1].split("=")[-1])
    assert res < 10.0  # the scaled residual of an FP64 factor is O(1)
    bad = subprocess.run([exe, "3000"], capture_output=True, text=True)
    assert bad.returncode == 1 and "invalid arguments" in bad.stderr


@pytest.mark.parametrize("n,lda,nb,budget_mb", [(3000, 3000, 256, 12), (2500, 2511, 128, 5), (2000, 2000, 512, 14)])
def test_spotrf_host_out_of_core(oracle_mod, handle, n, lda, nb, budget_mb):
    """A host FP32 matrix larger than the device budget: left-looking panels streamed
    through it, against the oracle's FP64 factor of the same matrix at FP32 accuracy."""
    A64 = oracle_mod.gen_uniform(n, 17, float(n)).astype(np.float32).astype(np.float64)
    Ap = np.full((lda, n), 5.0, dtype=np.float32, order="F")
    Ap[:n] = A64
    budget = budget_mb << 20
    assert n * n * 4 > budget  # really out of core
    r = handle.spotrf_L(Ap, n, lda, nb, budget)
    assert r.info == 0 and r.stats["npanels"] >= 2, r.stats
    Lo = A64.copy(order="F")
    oracle_mod.cholesky(Lo, nb, 1 << 40, 4, 2)
    Lo = np.tril(Lo)
    got = np.tril(Ap[:n].astype(np.float64))
    assert np.abs(got - Lo).max() <= TOL * np.abs(Lo).max()
    np.testing.assert_array_equal(np.triu(Ap[:n], 1), np.triu(A64.astype(np.float32), 1))
    assert np.all(Ap[n:] == 5.0)  # padding rows untouched
    # non-positive pivot found out of core: LAPACK info
    B = np.asfortranarray(A64.astype(np.float32))
    B[n - 300, n - 300] = -1.0
    assert handle.spotrf_L(B, n, n, nb, budget).info == n - 299


def test_spotrf_out_of_core_budget_too_small(handle, ooc):
    n, nb = 2000, 256
    A = np.asfortranarray(_spd32(n, 5))
    with pytest.raises(ooc.OocError) as e:
        handle.spotrf_L(A, n, n, nb, 3 * n * nb * 4 - 1)
    assert e.value.code == ooc.OOC_ERR_BUDGET


def test_pspotrf_descriptor_form(oracle_mod, handle, ooc, monkeypatch):
    """The FP32 descriptor entry on a sub-matrix (ia = ja = 2 of a larger array), with the
    budget from OOC_DEVICE_BUDGET_MB forcing the out-of-core path."""
    n, nb = 1500, 256
    A64 = oracle_mod.gen_uniform(n, 23, float(n)).astype(np.float32).astype(np.float64)
    big = np.zeros((n + 3, n + 3), dtype=np.float32, order="F")
    big[1:n + 1, 1:n + 1] = A64
    monkeypatch.setenv("OOC_DEVICE_BUDGET_MB", "6")
    desc = [1, 0, n + 3, n + 3, nb, nb, 0, 0, n + 3]
    assert ooc.pspotrf("L", n, big, 2, 2, desc) == 0
    L = np.tril(big[1:n + 1, 1:n + 1].astype(np.float64))
    want = np.linalg.cholesky(A64)
    assert np.abs(L - want).max() <= TOL * np.abs(want).max()
    assert big[0].max() == 0 and big[:, 0].max() == 0  # outside the sub-matrix untouched
    assert ooc.pspotrf("U", n, big, 2, 2, desc) == -1
