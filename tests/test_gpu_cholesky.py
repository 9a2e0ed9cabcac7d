"""GPU parity tests: the CUDA library against the CPU oracle on the same seeded inputs.

Parity bar (floating point): the scaled residual ||A - L L^T||_F / (n eps ||A||_F) of the
GPU factor must be within a factor RESID_RATIO of the oracle's on the same input, and the
factors must agree entrywise to ATOL_REL * max|L|.  Integer outputs (LAPACK info, panel
plans) and the generators must match exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RESID_RATIO = 10.0
ATOL_REL = 1e-12


def _to_dev(A):
    import torch

    return torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # (n, lda) row-major == column-major A


def _from_dev(T):
    return np.asfortranarray(T.cpu().numpy().T)


def _oracle_factor(oracle_mod, A, nb, tiles=None):
    n = A.shape[1]
    B = A.copy(order="F")
    mem = (tiles if tiles else 1 << 20) * nb * nb * 8
    _, info, _ = oracle_mod.cholesky(B, nb, mem, 4, 2)
    return B, info


def _check_parity(oracle_mod, Lg, Lo, kind, seed, alpha):
    n = Lg.shape[1]
    np.testing.assert_allclose(np.tril(Lg[:n]), np.tril(Lo[:n]), rtol=0,
                               atol=ATOL_REL * np.abs(np.tril(Lo[:n])).max())
    rg = oracle_mod.residual(Lg, kind, seed, alpha, tile=256)
    ro = oracle_mod.residual(Lo, kind, seed, alpha, tile=256)
    assert rg <= RESID_RATIO * ro and ro <= RESID_RATIO * rg, (rg, ro)
    return rg, ro


@pytest.mark.parametrize("n,nb", [(512, 128), (1000, 128), (1024, 1024), (777, 100), (300, 33), (64, 64), (1, 8)])
def test_incore_device_matches_oracle(oracle_mod, handle, n, nb):
    A = oracle_mod.gen_uniform(n, 100, float(n))
    Lo, info_o = _oracle_factor(oracle_mod, A, nb)
    T = _to_dev(A)
    r = handle.dpotrf_L(T, n, n, nb, 0)
    assert r.info == 0 == info_o and r.stats["npanels"] == 1
    Lg = _from_dev(T)
    _check_parity(oracle_mod, Lg, Lo, "uniform", 100, float(n))
    np.testing.assert_array_equal(np.triu(Lg, 1), np.triu(A, 1))


def test_incore_padded_leading_dimension(oracle_mod, handle):
    n, lda, nb = 700, 733, 128
    A = np.asfortranarray(np.zeros((lda, n)))
    A[:n] = oracle_mod.gen_uniform(n, 5, float(n))
    A[n:] = 7.0  # padding rows must be left alone
    Lo, _ = _oracle_factor(oracle_mod, A[:n].copy(order="F"), nb)
    T = _to_dev(A)
    assert handle.dpotrf_L(T, n, lda, nb, 0).info == 0
    Lg = _from_dev(T)
    assert np.all(Lg[n:] == 7.0)
    _check_parity(oracle_mod, Lg[:n].copy(order="F"), Lo, "uniform", 5, float(n))


@pytest.mark.parametrize("n,nb,tiles", [(1024, 128, 30), (1000, 128, 40), (1536, 256, 20), (2048, 256, 26)])
def test_ooc_host_matches_oracle_and_is_schedule_invariant(oracle_mod, handle, ooc, n, nb, tiles):
    A = oracle_mod.gen_uniform(n, 100, float(n))
    Lo, _ = _oracle_factor(oracle_mod, A, nb, tiles)
    results = []
    for xb in (1, 2):
        handle.set_option(ooc.OPT_X_BUFFERS, xb)
        for mult in (1, 3):
            H = A.copy(order="F")
            r = handle.dpotrf_L(H, n, n, nb, tiles * mult * nb * nb * 8)
            assert r.info == 0
            results.append((r.stats["npanels"], H))
    handle.set_option(ooc.OPT_X_BUFFERS, 2)
    assert max(p for p, _ in results) >= 2  # really out of core
    for _, H in results[1:]:
        np.testing.assert_array_equal(H, results[0][1])  # bitwise across schedules
    # and bitwise equal to the in-core device factorization
    T = _to_dev(A)
    handle.dpotrf_L(T, n, n, nb, 0)
    np.testing.assert_array_equal(_from_dev(T), results[0][1])
    _check_parity(oracle_mod, results[0][1], Lo, "uniform", 100, float(n))
    np.testing.assert_array_equal(np.triu(results[0][1], 1), np.triu(A, 1))


def test_ooc_matches_compiled_reference_fixture(oracle_mod, handle, ooc):
    """The library's factor against the reference's own output (tests/golden/ref_run.npz,
    made by the reference's oocdag.cpp/oocquark.cpp compiled unmodified), with the
    reference's panel schedule (one X buffer, its budget) and the library's default."""
    import os

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_run.npz"))
    names = [k for k in z.files if not k.endswith("_meta")]
    assert len(names) >= 3
    for name in names:
        n, nb, tiles, kind, seed, npanels = (int(v) for v in z[name + "_meta"])
        A = oracle_mod.gen_uniform(n, seed, float(n)) if kind == 0 else oracle_mod.gen_pdmatgen(n, seed)
        Lref = np.zeros((n, n))
        Lref[np.tril_indices(n)] = z[name]
        for ref_schedule in (1, 0):
            handle.set_option(ooc.OPT_REF_SCHEDULE, ref_schedule)
            handle.set_option(ooc.OPT_X_BUFFERS, 1 if ref_schedule else 2)
            try:
                H = A.copy(order="F")
                r = handle.dpotrf_L(H, n, n, nb, tiles * nb * nb * 8)
            finally:
                handle.set_option(ooc.OPT_REF_SCHEDULE, 0)
                handle.set_option(ooc.OPT_X_BUFFERS, 2)
            assert r.info == 0
            if ref_schedule:
                assert r.stats["npanels"] == npanels, name
            np.testing.assert_allclose(np.tril(H), Lref, rtol=0, atol=ATOL_REL * np.abs(Lref).max(), err_msg=name)
            np.testing.assert_array_equal(np.triu(H, 1), np.triu(A, 1))
            k = "uniform" if kind == 0 else "pdmatgen"
            alpha = float(n) if kind == 0 else 0.0
            rg = oracle_mod.residual(H, k, seed, alpha, tile=64)
            rr = oracle_mod.residual(np.asfortranarray(Lref), k, seed, alpha, tile=64)
            assert rg <= RESID_RATIO * rr and rr <= RESID_RATIO * rg, (name, rg, rr)


def test_ooc_wide_tiles_several_panels(oracle_mod, handle):
    """nb=1024 (the largest configuration's tile) streamed through a budget that forces at
    least three panels, against the oracle at the same tile width."""
    n, nb, tiles = 5120, 1024, 15  # three panels: (0,5,1), (1,4,2), (3,2,2)
    A = oracle_mod.gen_uniform(n, 100, float(n))
    Lo, info_o = _oracle_factor(oracle_mod, A, nb, tiles)
    H = A.copy(order="F")
    r = handle.dpotrf_L(H, n, n, nb, tiles * nb * nb * 8)
    assert r.info == 0 == info_o and r.stats["npanels"] >= 3, r.stats
    _check_parity(oracle_mod, H, Lo, "uniform", 100, float(n))
    np.testing.assert_array_equal(np.triu(H, 1), np.triu(A, 1))


def test_config0_in_core_host(oracle_mod, handle):
    # n=4096, nb=256, 24 GB budget: one panel through host memory.
    n, nb = 4096, 256
    A = oracle_mod.gen_uniform(n, 100, float(n))
    Lo, _ = _oracle_factor(oracle_mod, A, nb)
    H = A.copy(order="F")
    r = handle.dpotrf_L(H, n, n, nb, 24_000_000_000)
    assert r.info == 0 and r.stats["npanels"] == 1
    rg, ro = _check_parity(oracle_mod, H, Lo, "uniform", 100, float(n))
    assert rg < 5.0


def test_pdmatgen_matrix_ooc(oracle_mod, handle):
    n, nb = 1100, 128
    A = oracle_mod.gen_pdmatgen(n, 100)
    Lo, _ = _oracle_factor(oracle_mod, A, nb, 35)
    H = A.copy(order="F")
    assert handle.dpotrf_L(H, n, n, nb, 35 * nb * nb * 8).info == 0
    _check_parity(oracle_mod, H, Lo, "pdmatgen", 100, 0.0)


@pytest.mark.parametrize("where", ["host", "device"])
def test_non_spd_reports_lapack_info(oracle_mod, handle, where):
    n, nb = 900, 128
    A = oracle_mod.gen_uniform(n, 5, float(n))
    A[613, 613] = -3.0
    _, info_o = _oracle_factor(oracle_mod, A, nb, 30)
    assert info_o == 614
    if where == "host":
        H = A.copy(order="F")
        r = handle.dpotrf_L(H, n, n, nb, 30 * nb * nb * 8)
    else:
        T = _to_dev(A)
        r = handle.dpotrf_L(T, n, n, nb, 0)
    assert r.info == 614


def test_generators_match_oracle_bitwise(oracle_mod, handle):
    import torch

    for n in (1, 7, 300, 1031):
        U = oracle_mod.gen_uniform(n, 77, 12.5)
        P = oracle_mod.gen_pdmatgen(n, 100)
        Hu = np.asfortranarray(np.empty((n, n)))
        handle.matgen_uniform(Hu, n, n, 77, 12.5)
        np.testing.assert_array_equal(Hu, U)
        Hp = np.asfortranarray(np.empty((n, n)))
        handle.matgen_pdmatgen(Hp, n, n, 100)
        np.testing.assert_array_equal(Hp, P)
        T = torch.empty((n, n), dtype=torch.float64, device="cuda")
        handle.matgen_uniform(T, n, n, 77, 12.5)
        np.testing.assert_array_equal(_from_dev(T), U)
        handle.matgen_pdmatgen(T, n, n, 100)
        np.testing.assert_array_equal(_from_dev(T), P)


def test_device_residual_matches_oracle(oracle_mod, handle):
    n, nb = 1500, 256
    A = oracle_mod.gen_uniform(n, 3, float(n))
    Lo, _ = _oracle_factor(oracle_mod, A, nb)
    ro = oracle_mod.residual(Lo, "uniform", 3, float(n), tile=256)
    rg_host = handle.residual(Lo, n, n, "uniform", 3, float(n))
    rg_dev = handle.residual(_to_dev(Lo), n, n, "uniform", 3, float(n))
    assert abs(rg_host - ro) <= 0.05 * ro + 1e-3
    assert abs(rg_dev - ro) <= 0.05 * ro + 1e-3
    Lbad = Lo.copy(order="F")
    Lbad[1000, 3] += 1e-8  # planted in the oracle's factor, on the CPU
    assert handle.residual(Lbad, n, n, "uniform", 3, float(n)) > 100 * ro


def test_reference_shaped_entries(oracle_mod, handle, ooc):
    n, nb = 640, 64
    A = oracle_mod.gen_uniform(n, 100, float(n))
    Lo, _ = _oracle_factor(oracle_mod, A, nb, 30)
    H = A.copy(order="F")
    t = ooc.Cholesky(H, n, nb, n, 30 * nb * nb * 8)
    assert t > 0
    _check_parity(oracle_mod, H, Lo, "uniform", 100, float(n))
    # ScaLAPACK descriptor form on a sub-matrix (ia = ja = 1), LLD = n
    H2 = A.copy(order="F")
    desc = [1, 0, n, n, nb, nb, 0, 0, n]
    assert ooc.pdpotrf("L", n, H2, 1, 1, desc) == 0
    np.testing.assert_array_equal(H2, H)
    assert ooc.pdpotrf("U", n, H2, 1, 1, desc) == -1


def test_budget_too_small_errors(oracle_mod, handle, ooc):
    n, nb = 1024, 128
    H = oracle_mod.gen_uniform(n, 1, float(n))
    with pytest.raises(ooc.OocError) as e:
        handle.dpotrf_L(H, n, n, nb, 10 * nb * nb * 8)
    assert e.value.code == ooc.OOC_ERR_BUDGET


def test_profile_stats(oracle_mod, handle, ooc):
    n, nb = 2048, 256
    H = oracle_mod.gen_uniform(n, 1, float(n))
    handle.set_option(ooc.OPT_PROFILE, 1)
    try:
        r = handle.dpotrf_L(H, n, n, nb, 30 * nb * nb * 8)
    finally:
        handle.set_option(ooc.OPT_PROFILE, 0)
    s = r.stats
    assert s["npanels"] >= 2 and s["update_launches"] > 0 and s["update_ms"] > 0 and s["factor_ms"] > 0
    assert s["update_flops"] > 0.5 * s["flops"]
    assert s["h2d_bytes"] >= n * (n + 1) / 2 * 8 * 0.99 and s["d2h_bytes"] >= n * (n + 1) / 2 * 8 * 0.99


def test_fp64_peak_probe(handle):
    tf = handle.fp64_peak(50.0)
    assert 0.3 < tf < 5.0


@pytest.mark.parametrize("where,nrhs,nb", [("host", 1, 256), ("host", 16, 128), ("device", 3, 200)])
def test_solve_with_the_out_of_core_factor(oracle_mod, handle, where, nrhs, nb):
    """ooc_dpotrs_L: the reference's VERIFY solve (dpotrs on the factored matrix,
    oocdag.cpp:436-439) with the factor left by the out-of-core factorization -- a host L
    streamed through the device panel by panel, or a device L -- against LAPACK dpotrs on
    the oracle's factor."""
    import torch

    n = 2900
    A = oracle_mod.gen_uniform(n, 31, float(n))
    tiles = 3 * ((n + nb - 1) // nb) + 6  # a few panels
    Lh = A.copy(order="F")
    r = handle.dpotrf_L(Lh, n, n, nb, tiles * nb * nb * 8)
    assert r.info == 0 and r.stats["npanels"] >= 2
    Lo, _ = _oracle_factor(oracle_mod, A, nb, tiles)
    B = np.asfortranarray(np.random.default_rng(nrhs).standard_normal((n, nrhs)))
    Xo = oracle_mod.potrs(Lo, B)
    if where == "host":
        X = B.copy(order="F")
        handle.dpotrs_L(Lh, n, n, nb, X, n, nrhs, budget=2 * n * nb * 8 + (8 << 20))
    else:
        Ld = _to_dev(Lh)
        Xd = _to_dev(B)
        handle.dpotrs_L(Ld, n, n, nb, Xd, n, nrhs)
        X = _from_dev(Xd)
    assert np.abs(X - Xo).max() / np.abs(Xo).max() < 1e-12

    def berr(Y):  # normwise backward error, worst column
        nA = np.abs(A).sum(axis=1).max()
        return max(np.abs(B[:, q] - A @ Y[:, q]).max() / (nA * np.abs(Y[:, q]).max() + np.abs(B[:, q]).max())
                   for q in range(nrhs))

    assert berr(X) <= 1e-14 and berr(X) <= 10 * berr(Xo) + 1e-16, (berr(X), berr(Xo))


def test_out_of_core_solve_rejects_a_small_budget(oracle_mod, handle, ooc):
    n, nb = 1000, 128
    L = np.asfortranarray(np.eye(n))
    B = np.asfortranarray(np.ones((n, 1)))
    with pytest.raises(ooc.OocError) as e:
        handle.dpotrs_L(L, n, n, nb, B, n, 1, budget=n * nb * 8)
    assert e.value.code == ooc.OOC_ERR_BUDGET
