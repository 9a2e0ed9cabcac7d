"""GPU tests of the mixed-precision factor and the FP64 solve / iterative refinement.

Bars: the plain-precision factor object reproduces the plain path bit for bit; solves
agree with the oracle's FP64 solve (LAPACK dpotrs on the oracle factor) to a forward
error of FWD_TOL; refinement reaches the normwise backward error BERR_TOL (1e-14) for
every precision and every conditioning of the generator A = (R+R^T)/2 + alpha I,
alpha = 0.5774 sqrt(n) (1+delta).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BERR_TOL = 1e-14
FWD_TOL = 1e-11


def _dev(M):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(M).T)).cuda()


def _host(T):
    return np.asfortranarray(T.cpu().numpy().T)


def _c2_matrix(oracle_mod, n, delta, seed=7):
    alpha = 0.5774 * math.sqrt(n) * (1 + delta)
    return oracle_mod.gen_uniform(n, seed, alpha), alpha


def _berr(A, X, B):
    R = B - A @ X
    nA = np.abs(A).sum(axis=1).max()
    return max(np.abs(R[:, q]).max() / (nA * np.abs(X[:, q]).max() + np.abs(B[:, q]).max()) for q in range(B.shape[1]))


def test_fp64_factor_object_matches_plain_path(oracle_mod, handle):
    # The factor object solves each column with the diagonal tile's inverse (one DMMA
    # product) where the plain path substitutes; both are FP64 and agree to rounding.
    n, nb = 1500, 256
    A = oracle_mod.gen_uniform(n, 3, float(n))
    T = _dev(A)
    handle.dpotrf_L(T, n, n, nb, 0)
    F = handle.factor(_dev(A), n, n, nb, "fp64")
    assert F.info == 0
    L = np.asfortranarray(np.empty((n, n)))
    F.copy_L(L, n)
    Lp = np.tril(_host(T))
    assert np.abs(np.tril(L) - Lp).max() <= 1e-12 * np.abs(Lp).max()
    r_obj = oracle_mod.residual(L, "uniform", 3, float(n), tile=256)
    r_plain = oracle_mod.residual(_host(T), "uniform", 3, float(n), tile=256)
    assert r_obj <= 10 * r_plain and r_plain <= 10 * r_obj
    F.close()


@pytest.mark.parametrize("nrhs", [1, 16])
def test_fp64_solve_matches_oracle(oracle_mod, handle, nrhs):
    n, nb = 1300, 256
    A = oracle_mod.gen_uniform(n, 5, float(n))
    Lo = A.copy(order="F")
    oracle_mod.cholesky(Lo, nb, 1 << 30, 4, 2)
    B = np.asfortranarray(np.random.default_rng(2).standard_normal((n, nrhs)))
    Xo = oracle_mod.potrs(Lo, B)
    with handle.factor(A, n, n, nb, "fp64") as F:  # host A
        Bd = _dev(B)
        F.solve(Bd, n, nrhs)
        X = _host(Bd)
    assert np.abs(X - Xo).max() / np.abs(Xo).max() < FWD_TOL
    assert _berr(A, X, B) < BERR_TOL


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x3"])
@pytest.mark.parametrize("delta", [1.0, 0.1, 0.01])
@pytest.mark.parametrize("nrhs", [1, 16])
def test_refinement_reaches_backward_error(oracle_mod, handle, prec, delta, nrhs):
    n, nb = 2048, 256
    A, alpha = _c2_matrix(oracle_mod, n, delta)
    B = np.asfortranarray(np.random.default_rng(11).standard_normal((n, nrhs)))
    Lo = A.copy(order="F")
    oracle_mod.cholesky(Lo, nb, 1 << 30, 4, 2)
    Xo = oracle_mod.potrs(Lo, B)  # the FP64 oracle solve
    Ad = _dev(A)
    Bd = _dev(B)
    import torch

    Xd = torch.empty_like(Bd)
    with handle.factor(Ad, n, n, nb, prec) as F:
        assert F.info == 0
        it, be = F.refine(Ad, n, Bd, n, Xd, n, nrhs, BERR_TOL, 30)
    X = _host(Xd)
    assert be <= BERR_TOL, (prec, delta, it, be)
    assert _berr(A, X, B) <= 2 * BERR_TOL  # recomputed on the host
    fwd = np.abs(X - Xo).max() / np.abs(Xo).max()
    assert fwd < FWD_TOL, fwd
    if prec != "fp64":
        assert 1 <= it <= 10  # the reduced-precision factor needs (and gets) a few corrections


def test_fp32_factor_is_less_accurate_but_close(oracle_mod, handle):
    # The FP32 trailing updates perturb the factor at FP32 level: its residual is well
    # above the FP64 factor's, and well below O(1).
    n, nb = 2048, 256
    A, alpha = _c2_matrix(oracle_mod, n, 0.1)
    L64 = np.asfortranarray(np.empty((n, n)))
    L32 = np.asfortranarray(np.empty((n, n)))
    with handle.factor(A, n, n, nb, "fp64") as F:
        F.copy_L(L64, n)
    with handle.factor(A, n, n, nb, "fp32") as F:
        F.copy_L(L32, n)
    L16 = np.asfortranarray(np.empty((n, n)))
    with handle.factor(A, n, n, nb, "bf16x3") as F:
        F.copy_L(L16, n)
    r64 = oracle_mod.residual(L64, "uniform", 7, alpha, tile=256)
    r32 = oracle_mod.residual(L32, "uniform", 7, alpha, tile=256)
    r16 = oracle_mod.residual(L16, "uniform", 7, alpha, tile=256)
    assert r64 < 10 and 1e3 < r32 < 1e10 and 1e3 < r16 < 1e12, (r64, r32, r16)


def test_non_spd_factor_refuses_to_solve(oracle_mod, handle, ooc):
    n, nb = 700, 128
    A = oracle_mod.gen_uniform(n, 1, float(n))
    A[400, 400] = -5.0
    with handle.factor(A, n, n, nb, "fp32") as F:
        assert F.info == 401
        import torch

        B = torch.zeros((1, n), dtype=torch.float64, device="cuda")
        with pytest.raises(ooc.OocError):
            F.solve(B, n, 1)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("fp32", 3e-6), ("bf16x3", 1e-4)])
@pytest.mark.parametrize("n,k", [(1, 64), (100, 64), (128, 128), (129, 100), (300, 512), (1000, 256)])
def test_dsyrk_kernels_against_fp64(handle, prec, tol, n, k):
    # C := C - A A^T on the lower triangle; the relative error is measured against the
    # size of the product, since C itself is an arbitrary offset.
    rng = np.random.default_rng(n * 1000 + k)
    A = np.asfortranarray(rng.standard_normal((n, k)))
    C = np.asfortranarray(rng.standard_normal((n, n)))
    want = C - A @ A.T
    Ad, Cd = _dev(A), _dev(C)
    handle.dsyrk_ln(prec, n, k, Ad, n, Cd, n)
    got = _host(Cd)
    lo = np.tril(np.ones((n, n), dtype=bool))
    scale = np.abs(A @ A.T).max()
    err = np.abs(got - want)[lo].max() / scale
    assert err < tol, (prec, n, k, err)
    np.testing.assert_array_equal(got[~lo], C[~lo])  # strict upper untouched


@pytest.mark.parametrize("prec", ["bf16x3", "fp64"])
def test_generated_factor_and_refinement(oracle_mod, handle, prec):
    # A generated in place (no copy kept) and regenerated inside the residual: the factor is
    # bit-identical to factoring a stored copy of the same matrix; refinement reaches the bar.
    import torch

    n, nb = 1536, 256
    alpha = 0.5774 * math.sqrt(n) * 1.1
    A = oracle_mod.gen_uniform(n, 21, alpha)
    Fg = handle.factor_gen(n, 21, alpha, nb, prec)
    Fs = handle.factor(A, n, n, nb, prec)
    Lg = np.asfortranarray(np.empty((n, n)))
    Ls = np.asfortranarray(np.empty((n, n)))
    Fg.copy_L(Lg, n)
    Fs.copy_L(Ls, n)
    np.testing.assert_array_equal(np.tril(Lg), np.tril(Ls))
    Bd = torch.empty((4, n), dtype=torch.float64, device="cuda")
    handle.gen_normal(Bd, n, n, 4, 5)
    Xd = torch.empty_like(Bd)
    it, be = Fg.refine_gen(Bd, n, Xd, n, 4, BERR_TOL, 30)
    assert be <= BERR_TOL
    X = _host(Xd)
    B = _host(Bd)
    assert _berr(A, X, B) <= 2 * BERR_TOL
    assert abs(B.mean()) < 0.1 and 0.9 < B.std() < 1.1  # the N(0,1) generator
    Fg.close()
    Fs.close()


def test_reduced_factor_keeps_only_fp32(oracle_mod, handle, ooc):
    # A reduced-precision factor is the FP32 working matrix (half the FP64 factor's memory,
    # no FP64 copy); copy_L widens it exactly (every value an FP32 number), zeros above.
    n, nb = 1100, 256
    assert ooc.factor_bytes(65536, 512, "bf16x3") < 0.51 * ooc.factor_bytes(65536, 512, "fp64")
    A, alpha = _c2_matrix(oracle_mod, n, 0.1)
    with handle.factor(A, n, n, nb, "bf16x3") as F:
        L = np.asfortranarray(np.full((n, n), np.nan))
        F.copy_L(L, n)
    assert np.all(np.triu(L, 1) == 0)
    low = np.tril(L)
    np.testing.assert_array_equal(low.astype(np.float32).astype(np.float64), low)
    Lo = A.copy(order="F")
    oracle_mod.cholesky(Lo, nb, 1 << 30, 4, 2)
    assert np.abs(low - np.tril(Lo)).max() <= 1e-3 * np.abs(np.tril(Lo)).max()


@pytest.mark.parametrize("where,keep", [("host", 1), ("host", 0), ("device", 0)])
def test_refine_reads_only_the_lower_triangle(oracle_mod, handle, ooc, where, keep):
    # The factor and the refinement read only A's lower triangle (the residual and the
    # norm use A's symmetry): NaN above the diagonal must not reach the solution.  A host
    # A is copied once, lower triangle only; with OOC_OPT_KEEP_A the refinement reuses the
    # factor's device copy instead of copying it again.
    import torch

    n, nb, r = 1100, 256, 3
    A, _ = _c2_matrix(oracle_mod, n, 0.1)
    An = A.copy(order="F")
    An[np.triu_indices(n, 1)] = np.nan
    B = np.asfortranarray(np.random.default_rng(2).standard_normal((n, r)))
    if where == "host":
        Ain = torch.from_numpy(np.ascontiguousarray(An.T)).pin_memory()  # column-major storage
    else:
        Ain = _dev(An)
    Bd, Xd = _dev(B), _dev(np.zeros((n, r)))
    handle.set_option(ooc.OPT_KEEP_A, keep)
    try:
        with handle.factor(Ain, n, n, nb, "bf16x3") as F:
            assert F.info == 0
            it, be = F.refine(Ain, n, Bd, n, Xd, n, r, BERR_TOL, 30)
    finally:
        handle.set_option(ooc.OPT_KEEP_A, 0)
    assert be <= BERR_TOL and it <= 5
    X = _host(Xd)
    assert np.isfinite(X).all()
    assert _berr(A, X, B) <= 2 * BERR_TOL


@pytest.mark.parametrize("nb,tail", [(256, 0), (256, 600), (256, 32768), (512, 600)])
def test_tail_panels_schedule(oracle_mod, handle, ooc, nb, tail):
    # Split-BF16 factors switch to nb/2-wide panels for the last `tail` orders (rounded to
    # a multiple of nb): uniform (0), a switch at column 512 with a ragged last panel (600
    # at n=1100, nb=256) and all panels narrow (32768).  The factor, the kept diagonal
    # inverses and the solves follow the same schedule; nb=512 with the switch at column 512
    # mixes 512- and 256-wide diagonal tiles in one factorization.
    n, r = 1100, 2
    A, _ = _c2_matrix(oracle_mod, n, 0.1)
    B = np.asfortranarray(np.random.default_rng(5).standard_normal((n, r)))
    Bd, Xd = _dev(B), _dev(np.zeros((n, r)))
    handle.set_option(ooc.OPT_TAIL_ORDER, tail)
    try:
        with handle.factor(_dev(A), n, n, nb, "bf16x3") as F:
            assert F.info == 0
            L = np.asfortranarray(np.full((n, n), np.nan))
            F.copy_L(L, n)
            it, be = F.refine(_dev(A), n, Bd, n, Xd, n, r, BERR_TOL, 30)
    finally:
        handle.set_option(ooc.OPT_TAIL_ORDER, 24576)
    Lo = A.copy(order="F")
    oracle_mod.cholesky(Lo, nb, 1 << 30, 4, 2)
    assert np.abs(np.tril(L) - np.tril(Lo)).max() <= 1e-3 * np.abs(np.tril(Lo)).max()
    assert be <= BERR_TOL and it <= 5
    assert _berr(A, _host(Xd), B) <= 2 * BERR_TOL


def test_pooled_buffers_give_identical_factors(oracle_mod, handle, ooc):
    # Factor objects take their device buffers from the handle's cache and return them
    # when destroyed; a factor built in reused buffers is bit-identical to one built in
    # fresh ones (OOC_OPT_POOL_BYTES = 0: no caching), and the cap can be read back.
    n, nb = 1100, 256
    A, _ = _c2_matrix(oracle_mod, n, 0.1)
    Ad = _dev(A)

    def factor_L():
        with handle.factor(Ad, n, n, nb, "bf16x3") as F:
            assert F.info == 0
            L = np.asfortranarray(np.full((n, n), np.nan))
            F.copy_L(L, n)
        return L

    cap = handle.get_option(ooc.OPT_POOL_BYTES)
    assert cap > 0
    first = factor_L()
    again = [factor_L() for _ in range(2)]  # sizes repeat: buffers come from the cache
    handle.set_option(ooc.OPT_POOL_BYTES, 0)
    try:
        fresh = factor_L()
    finally:
        handle.set_option(ooc.OPT_POOL_BYTES, cap)
    for L in again + [fresh]:
        np.testing.assert_array_equal(L, first)


@pytest.mark.parametrize("tail", [24576, 8192])
def test_split_bf16_at_bench_tile_width_n16384(oracle_mod, handle, ooc, tail):
    # The benchmark's tile width (nb=512) at n=16384: the default tail schedule (every
    # panel 256 wide here, diagonal tiles in shared memory) and a switch at order 8192
    # (512-wide panels and their diagonal kernel first).  The trailing updates run the
    # persistent 256x128 tcgen05 kernel up to m ~ 16k.  Against the oracle's FP64 solve.
    import os

    import torch

    n, nb = 16384, 512
    A, alpha = _c2_matrix(oracle_mod, n, 0.1)
    B = np.asfortranarray(np.random.default_rng(16).standard_normal((n, 1)))
    Lo = A.copy(order="F")
    _, info_o, _ = oracle_mod.cholesky(Lo, nb, 8 << 30, max(4, (os.cpu_count() or 8) - 2), 2)
    assert info_o == 0
    Xo = oracle_mod.potrs(Lo, B)
    del Lo
    Ad, Bd = _dev(A), _dev(B)
    Xd = torch.empty_like(Bd)
    handle.set_option(ooc.OPT_TAIL_ORDER, tail)
    try:
        with handle.factor(Ad, n, n, nb, "bf16x3") as F:
            assert F.info == 0
            it, be = F.refine(Ad, n, Bd, n, Xd, n, 1, BERR_TOL, 30)
    finally:
        handle.set_option(ooc.OPT_TAIL_ORDER, 24576)
    X = _host(Xd)
    assert be <= BERR_TOL and 1 <= it <= 5, (it, be)
    assert _berr(A, X, B) <= 2 * BERR_TOL
    fwd = np.abs(X - Xo).max() / np.abs(Xo).max()
    assert fwd < FWD_TOL, fwd


@pytest.mark.parametrize("where,keep,nb,bcols,n", [
    ("host", 1, 512, -1, 10000),   # default: page-locked host matrix in 4096-column blocks
    ("host", 0, 256, 1024, 5000),  # ragged last panel, staging instead of a kept copy
    ("device", 0, 512, 2048, 9000),
    ("device", 0, 256, 256, 2100),  # one panel per block
])
def test_left_looking_blocks(oracle_mod, handle, ooc, where, keep, nb, bcols, n):
    # Split-BF16 factors over left-looking column blocks (OOC_OPT_BLOCK_COLS): each block is
    # filled (copied from a page-locked host matrix while earlier blocks are factored, or
    # converted from the device matrix), caught up with every finished panel by one long-K
    # update from the plane store, then factored inside itself.  Against the oracle's FP64
    # factor at the split-BF16 level, close to the right-looking factor of the same matrix,
    # and refinement to the FP64 backward-error bar.
    import torch

    r = 2
    A, _ = _c2_matrix(oracle_mod, n, 0.1)
    B = np.asfortranarray(np.random.default_rng(8).standard_normal((n, r)))
    Bd, Xd = _dev(B), _dev(np.zeros((n, r)))
    Ain = torch.from_numpy(np.ascontiguousarray(A.T)).pin_memory() if where == "host" else _dev(A)
    Lb = np.asfortranarray(np.full((n, n), np.nan))
    Lr = np.asfortranarray(np.full((n, n), np.nan))
    handle.set_option(ooc.OPT_KEEP_A, keep)
    try:
        handle.set_option(ooc.OPT_BLOCK_COLS, bcols)
        with handle.factor(Ain, n, n, nb, "bf16x3") as F:
            assert F.info == 0
            F.copy_L(Lb, n)
            it, be = F.refine(Ain, n, Bd, n, Xd, n, r, BERR_TOL, 30)
        handle.set_option(ooc.OPT_BLOCK_COLS, 0)
        with handle.factor(Ain, n, n, nb, "bf16x3") as F:
            F.copy_L(Lr, n)
    finally:
        handle.set_option(ooc.OPT_BLOCK_COLS, -1)
        handle.set_option(ooc.OPT_KEEP_A, 0)
    Lo = A.copy(order="F")
    oracle_mod.cholesky(Lo, nb, 1 << 40, 4, 2)
    Lo = np.tril(Lo)
    scale = np.abs(Lo).max()
    assert np.abs(np.tril(Lb) - Lo).max() <= 1e-3 * scale
    assert np.abs(np.tril(Lb) - np.tril(Lr)).max() <= 1e-4 * scale
    assert np.all(np.triu(Lb, 1) == 0)
    assert be <= BERR_TOL and it <= 5, (it, be)
    assert _berr(A, _host(Xd), B) <= 2 * BERR_TOL


def test_copy_streams_do_not_change_the_factor(oracle_mod, handle, ooc):
    # A page-locked host matrix streamed into the left-looking factor over one or two
    # host-to-device streams (OOC_OPT_COPY_STREAMS): the copies only move bytes, so the
    # factors are identical bit for bit, and both refine to the FP64 bar.
    import torch

    n, nb = 9000, 512
    A, _ = _c2_matrix(oracle_mod, n, 0.1)
    Ah = torch.from_numpy(np.ascontiguousarray(A.T)).pin_memory()
    B = np.asfortranarray(np.random.default_rng(4).standard_normal((n, 1)))
    Ls = []
    handle.set_option(ooc.OPT_KEEP_A, 1)
    handle.set_option(ooc.OPT_BLOCK_COLS, 2048)
    try:
        for cs in (1, 2):
            handle.set_option(ooc.OPT_COPY_STREAMS, cs)
            assert handle.get_option(ooc.OPT_COPY_STREAMS) == cs
            L = np.asfortranarray(np.full((n, n), np.nan))
            Bd, Xd = _dev(B), _dev(np.zeros((n, 1)))
            with handle.factor(Ah, n, n, nb, "bf16x3") as F:
                assert F.info == 0
                F.copy_L(L, n)
                it, be = F.refine(Ah, n, Bd, n, Xd, n, 1, BERR_TOL, 30)
            assert be <= BERR_TOL and it <= 5, (cs, it, be)
            Ls.append(L)
    finally:
        handle.set_option(ooc.OPT_COPY_STREAMS, 2)
        handle.set_option(ooc.OPT_BLOCK_COLS, -1)
        handle.set_option(ooc.OPT_KEEP_A, 0)
    np.testing.assert_array_equal(Ls[0], Ls[1])


def test_left_looking_blocks_report_lapack_info(oracle_mod, handle, ooc):
    import torch

    n, nb = 3000, 256
    A = oracle_mod.gen_uniform(n, 1, float(n))
    A[2222, 2222] = -5.0
    Ah = torch.from_numpy(np.ascontiguousarray(A.T)).pin_memory()
    handle.set_option(ooc.OPT_BLOCK_COLS, 512)
    try:
        with handle.factor(Ah, n, n, nb, "bf16x3") as F:
            assert F.info == 2223
    finally:
        handle.set_option(ooc.OPT_BLOCK_COLS, -1)
