"""GPU tests of the batched persistent factor + solve (A = M M^T/n + I, n in [16, 512], small batches).

Each matrix is compared with the per-matrix FP64 path (LAPACK via numpy on the same
matrix): factor entries to FACT_TOL relative, solution to SOL_TOL relative; FP32 to the
looser FP32 bounds.  LAPACK info must match exactly for a planted non-SPD matrix, and
its neighbours must be unaffected.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": (1e-12, 1e-11), "fp32": (2e-5, 2e-4)}


def _make_batch(ns, seed, dtype):
    rng = np.random.default_rng(seed)
    mats, rhs, a_off, b_off = [], [], [], []
    ao = bo = 0
    for n in ns:
        M = rng.standard_normal((n, n))
        A = M @ M.T / n + np.eye(n)
        b = rng.standard_normal(n)
        mats.append(A)
        rhs.append(b)
        a_off.append(ao)
        b_off.append(bo)
        ao += n * n
        bo += n
    Aflat = np.concatenate([np.asfortranarray(A).ravel(order="F") for A in mats]).astype(dtype)
    Bflat = np.concatenate(rhs).astype(dtype)
    return mats, rhs, a_off, b_off, Aflat, Bflat


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batched_matches_per_matrix_fp64(handle, prec):
    import torch

    rng = np.random.default_rng(5)
    ns = list(rng.integers(16, 513, size=120)) + [1, 2, 3, 15, 16, 17, 31, 32, 33, 63, 64, 65, 511, 512]
    dtype = np.float64 if prec == "fp64" else np.float32
    mats, rhs, a_off, b_off, Af, Bf = _make_batch(ns, 9, dtype)
    Ad = torch.from_numpy(Af).cuda()
    Bd = torch.from_numpy(Bf).cuda()
    info, sec = handle.batched_posv(prec, ns, a_off, b_off, Ad, Bd)
    assert all(i == 0 for i in info) and sec > 0
    Ah, Bh = Ad.cpu().numpy(), Bd.cpu().numpy()
    ftol, stol = TOL[prec]
    for i, n in enumerate(ns):
        L = Ah[a_off[i]:a_off[i] + n * n].reshape((n, n), order="F").astype(np.float64)
        Lref = np.linalg.cholesky(mats[i])
        assert np.abs(np.tril(L) - Lref).max() <= ftol * np.abs(Lref).max(), (i, n)
        x = Bh[b_off[i]:b_off[i] + n].astype(np.float64)
        xref = np.linalg.solve(mats[i], rhs[i])
        assert np.abs(x - xref).max() <= stol * np.abs(xref).max(), (i, n)


def test_batched_reports_info_per_matrix(handle):
    import torch

    ns = [100, 300, 50, 200]
    mats, rhs, a_off, b_off, Af, Bf = _make_batch(ns, 3, np.float64)
    bad = 1  # plant a non-positive pivot in the second matrix (n=300) at column 120
    A = mats[bad].copy()
    A[120, 120] = -1.0
    Af[a_off[bad]:a_off[bad] + 300 * 300] = np.asfortranarray(A).ravel(order="F")
    Ad = torch.from_numpy(Af).cuda()
    Bd = torch.from_numpy(Bf).cuda()
    info, _ = handle.batched_posv("fp64", ns, a_off, b_off, Ad, Bd)
    import scipy.linalg as sla

    want = sla.lapack.dpotrf(A, lower=1)[1]
    assert info[bad] == want == 121
    assert [info[i] for i in (0, 2, 3)] == [0, 0, 0]
    Bh = Bd.cpu().numpy()
    for i in (0, 2, 3):
        n = ns[i]
        xref = np.linalg.solve(mats[i], rhs[i])
        assert np.abs(Bh[b_off[i]:b_off[i] + n] - xref).max() <= 1e-11 * np.abs(xref).max()


def test_batched_block_table_does_not_change_results(handle):
    import torch

    ns = [37, 100, 250, 400]
    mats, rhs, a_off, b_off, Af, Bf = _make_batch(ns, 4, np.float64)
    outs = []
    for blk in (8, 16, 32):
        Ad = torch.from_numpy(Af.copy()).cuda()
        Bd = torch.from_numpy(Bf.copy()).cuda()
        info, _ = handle.batched_posv("fp64", ns, a_off, b_off, Ad, Bd, blk_table=[blk] * 16)
        assert info == [0, 0, 0, 0]
        outs.append(Bd.cpu().numpy())
    for o in outs[1:]:
        assert np.abs(o - outs[0]).max() <= 1e-11 * np.abs(outs[0]).max()


@pytest.mark.parametrize("blk", [8, 16, 32])
def test_batched_every_width_all_buckets(handle, blk):
    import torch

    ns = list(range(16, 513, 7)) + [288, 289, 295, 300, 311, 319, 320]
    mats, rhs, a_off, b_off, Af, Bf = _make_batch(ns, 17, np.float64)
    Ad = torch.from_numpy(Af).cuda()
    Bd = torch.from_numpy(Bf).cuda()
    info, _ = handle.batched_posv("fp64", ns, a_off, b_off, Ad, Bd, blk_table=[blk] * 16)
    bad = [(ns[i], info[i]) for i in range(len(ns)) if info[i]]
    assert not bad, bad
    Bh = Bd.cpu().numpy()
    for i, n in enumerate(ns):
        xref = np.linalg.solve(mats[i], rhs[i])
        assert np.abs(Bh[b_off[i]:b_off[i] + n] - xref).max() <= 1e-11 * np.abs(xref).max(), (blk, n)
