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
