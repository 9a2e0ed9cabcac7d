"""CPU tests of the oracle: pinned against the golden fixtures, LAPACK and itself."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_pdmatgen_closed_form_matches_literal_loops(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "pdmatgen_literal.npz"))
    assert len(g.files) >= 7
    for k in g.files:
        n = int(k.split("_")[0][1:])
        seed = int(k.split("seed")[1])
        A = oracle_mod.gen_pdmatgen(n, seed)
        np.testing.assert_array_equal(A, g[k], err_msg=k)


def test_pdmatgen_symmetric_and_dominant(oracle_mod):
    n = 200
    A = oracle_mod.gen_pdmatgen(n, 100)
    np.testing.assert_array_equal(A, A.T)
    off = np.abs(A - np.diag(np.diag(A)))
    assert np.all(np.diag(A) >= n) and off.max() <= 1.0


def test_panel_plans_match_literal_find_yn(oracle_mod):
    plans = json.load(open(os.path.join(GOLDEN, "panel_plans.json")))
    for label, v in plans.items():
        got = oracle_mod.panel_plan(v["N"], v["NB"], v["memBlock"])
        assert got == [tuple(p) for p in v["panels"]], label
    # n=163840, nb=1024, 24e9-byte budget: five panels starting (0,160,17),(17,143,20),(37,123,24).
    c1 = plans["c1_n163840_nb1024_24e9B"]["panels"]
    assert len(c1) == 5 and [tuple(p) for p in c1[:3]] == [(0, 160, 17), (17, 143, 20), (37, 123, 24)]
    assert tuple(c1[-1]) == (94, 66, 66)


def test_find_yn_state_only_grows(oracle_mod):
    # The reference keeps Yn in a function-local static (oocdag.cpp:480): a narrow
    # later panel is never chosen, except for the last.
    yn, st = oracle_mod.find_Yn(40, 256, 0, 0)
    yn2, st2 = oracle_mod.find_Yn(40, 256, 5, st)
    assert yn == 5 and yn2 >= yn


def test_oracle_matches_program_order_fixture(oracle_mod):
    c = np.load(os.path.join(GOLDEN, "chol_program_order.npz"))
    for n, nb, t in [(96, 32, 10), (100, 32, 12)]:
        A = c[f"A_n{n}_nb{nb}"].copy(order="F")
        L = c[f"L_n{n}_nb{nb}_tiles{t}"]
        _, info, npan = oracle_mod.cholesky(A, nb, t * nb * nb * 8, 4, 2)
        assert info == 0 and npan >= 1
        np.testing.assert_allclose(A, L, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("n,nb,tiles", [(256, 64, 12), (300, 64, 14), (513, 128, 11), (777, 100, 30), (64, 64, 4)])
def test_oracle_vs_lapack(oracle_mod, n, nb, tiles):
    A = oracle_mod.gen_uniform(n, 7, float(n))
    A0 = A.copy(order="F")
    _, info, npan = oracle_mod.cholesky(A, nb, tiles * nb * nb * 8, 3, 1)
    assert info == 0
    Lref = np.linalg.cholesky(A0)
    np.testing.assert_allclose(np.tril(A), Lref, rtol=0, atol=1e-12 * np.abs(Lref).max())
    np.testing.assert_array_equal(np.triu(A, 1), np.triu(A0, 1))  # upper untouched


def test_oracle_threaded_equals_program_order_bitwise(oracle_mod):
    n, nb = 600, 64
    A = oracle_mod.gen_uniform(n, 3, float(n))
    B = A.copy(order="F")
    oracle_mod.cholesky(A, nb, 25 * nb * nb * 8, 4, 2)
    oracle_mod.cholesky(B, nb, 25 * nb * nb * 8, 0, 0)
    np.testing.assert_array_equal(A, B)


def test_oracle_schedule_invariance_bitwise(oracle_mod):
    # The same tile operations in the same order reach every tile whatever the panel
    # split, so L is bit-identical across budgets.
    n, nb = 640, 64
    A0 = oracle_mod.gen_uniform(n, 11, float(n))
    outs = []
    for tiles in [22, 40, 90, 1000]:
        A = A0.copy(order="F")
        _, info, npan = oracle_mod.cholesky(A, nb, tiles * nb * nb * 8, 4, 2)
        outs.append((npan, A))
    assert len({p for p, _ in outs}) >= 3
    for _, A in outs[1:]:
        np.testing.assert_array_equal(A, outs[0][1])


def test_oracle_non_spd_info(oracle_mod):
    n, nb = 300, 64
    A = oracle_mod.gen_uniform(n, 5, float(n))
    A[170, 170] = -1.0
    _, info, _ = oracle_mod.cholesky(A, nb, 14 * nb * nb * 8, 3, 1)
    assert info == 171


def test_oracle_budget_too_small(oracle_mod):
    A = oracle_mod.gen_uniform(256, 1, 256.0)
    _, info, _ = oracle_mod.cholesky(A, 64, 4 * 64 * 64 * 8, 2, 1)
    assert info == -6


def test_residual_small_and_catches_planted_error(oracle_mod):
    n, nb = 384, 64
    A = oracle_mod.gen_uniform(n, 9, float(n))
    oracle_mod.cholesky(A, nb, 20 * nb * nb * 8, 3, 1)
    r = oracle_mod.residual(A, "uniform", 9, float(n), tile=128)
    assert r < 1.0
    B = A.copy(order="F")
    B[200, 100] += 1e-9  # a mistake planted in the oracle's factor
    assert oracle_mod.residual(B, "uniform", 9, float(n), tile=128) > 100 * r


def test_residual_pdmatgen(oracle_mod):
    n, nb = 256, 64
    A = oracle_mod.gen_pdmatgen(n, 100)
    oracle_mod.cholesky(A, nb, 12 * nb * nb * 8, 3, 1)
    assert oracle_mod.residual(A, "pdmatgen", 100, tile=100) < 1.0


def test_uniform_generator_properties(oracle_mod):
    n = 300
    A = oracle_mod.gen_uniform(n, 42, 0.0)
    np.testing.assert_array_equal(A, A.T)
    assert np.abs(A).max() < 0.5
    # the block generator agrees with the whole-matrix generator
    B = oracle_mod.gen_uniform_block(n, 42, 0.0, 17, 33, 100, 50)
    np.testing.assert_array_equal(B, A[17:117, 33:83])
    # different seeds differ; mean of R is near zero
    C = oracle_mod.gen_uniform(n, 43, 0.0)
    assert not np.array_equal(A, C)
    assert abs(A.mean()) < 0.01


def test_potrs_solves(oracle_mod):
    n = 200
    A = oracle_mod.gen_uniform(n, 2, float(n))
    A0 = A.copy(order="F")
    oracle_mod.cholesky(A, 64, 12 * 64 * 64 * 8, 2, 1)
    b = np.random.default_rng(0).standard_normal((n, 3))
    x = oracle_mod.potrs(A, b)
    np.testing.assert_allclose(A0 @ x, b, rtol=0, atol=1e-10)
