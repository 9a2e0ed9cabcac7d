"""Generate the golden fixtures in tests/golden from literal restatements.

The reference project (efdazedo/oocdag) ships no tests, fixtures or known answers,
and it cannot be built in this environment.  These fixtures are therefore produced by
restatements that follow the reference's own loops statement by statement, in plain
Python, so that the closed forms used by the oracle and by the GPU library can be
checked against them:

* ``pdmatgen_literal.npz`` -- the symmetric, diagonally dominant test matrix of
  LIN/pdmatgen.f (lower pass :223-303, upper pass :307-378, diagonal :516-543) on a
  1 x 1 process grid, driven by the 31-bit LCG helpers of LIN/pmatgeninc.f (LADD :5-34,
  LMUL :40-78 with 32-bit integer wrap-around, XJUMPM :84-135, SETRAN :141-176,
  JUMPIT :182-217, PDRAND :271-313).
* ``panel_plans.json`` -- the (jb, Ym, Yn) panel sequence of the driver loop
  (oocdag.cpp:59-66) with the panel sizing of oocdag.cpp:478-492, for the problem sizes
  used by the tests and the benchmark.
* ``chol_program_order.npz`` -- the reference task list (oocquark.cpp:253-421 driven by
  oocdag.cpp:59-87) executed one task at a time in program order on SciPy's BLAS, for a
  small matrix and a budget that forces several panels.

Run:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# ----------------------------------------------------------------------------------
# 31-bit LCG helpers (LIN/pmatgeninc.f), with Fortran default-integer (32-bit) wrap.
# ----------------------------------------------------------------------------------
IPOW15, IPOW16, IPOW30 = 2 ** 15, 2 ** 16, 2 ** 30


def _i32(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= (1 << 31) else v


def _fix(v: int) -> int:
    # IF( KT.LT.0 ) KT = (KT+IPOW30) + IPOW30   (pmatgeninc.f:65,68,70)
    if v < 0:
        v = _i32(_i32(v + IPOW30) + IPOW30)
    return v


def ladd(j, k):
    s = k[0] + j[0]
    return [s % IPOW16, (s // IPOW16 + k[1] + j[1]) % IPOW15]


def lmul(k, j):
    kt = _fix(_i32(k[0] * j[0]))
    i0 = kt % IPOW16
    lt = _fix(_i32(_i32(k[0] * j[1]) + _i32(k[1] * j[0])))
    kt = _fix(_i32(kt // IPOW16 + lt))
    return [i0, kt % IPOW15]


def xjumpm(jumpm, mult, iadd, irann, iam=None, icm=None):
    """Returns (iranm, iam, icm)."""
    if jumpm > 0:
        iam = list(mult)
        icm = list(iadd)
        for _ in range(jumpm - 1):
            iam = lmul(iam, mult)
            icm = ladd(iadd, lmul(icm, mult))
        iranm = ladd(lmul(irann, iam), icm)
        return iranm, iam, icm
    return list(irann), iam, icm


class Rng:
    """The /RANCOM/ common block with SETRAN, JUMPIT and PDRAND."""

    def __init__(self):
        self.irand = [0, 0]
        self.ias = [0, 0]
        self.ics = [0, 0]

    def setran(self, iran, ia, ic):
        self.irand, self.ias, self.ics = list(iran), list(ia), list(ic)

    def jumpit(self, mult, iadd, irann):
        iranm = ladd(lmul(irann, mult), iadd)
        self.irand = list(iranm)
        return iranm

    def pdrand(self):
        v = (float(self.irand[0]) + 65536.0 * float(self.irand[1])) / 2147483648.0
        self.irand = ladd(lmul(self.irand, self.ias), self.ics)
        return v


def pdmatgen_symm_diag(n: int, nb: int, iseed: int) -> np.ndarray:
    """PDMATGEN('Symm', 'Diag', M=N, MB=NB) on a 1 x 1 grid, offsets 0, full extent."""
    M = N = n
    MB = NB = nb
    mult0, mult1, iadd0, iadd1 = 20077, 16838, 12345, 0
    A = np.zeros((n + 1, n + 1))  # 1-based indexing; row/col 0 unused
    rng = Rng()
    IRNUM = ICNUM = n
    MOFF = NOFF = 0
    MEND = -(-IRNUM // MB) + MOFF
    NEND = -(-ICNUM // NB) + NOFF
    NPMB, NQNB, MRROW, MRCOL = MB, NB, 0, 0

    # ---- lower triangular part (with diagonal block), pdmatgen.f:223-303
    mult, iadd, jseed = [mult0, mult1], [iadd0, iadd1], [iseed, 0]
    iran1, ia1, ic1 = xjumpm(1, mult, iadd, jseed)
    _, ia2, ic2 = xjumpm(NPMB, mult, iadd, iran1)
    _, ia3, ic3 = xjumpm(M, mult, iadd, iran1)
    _, ia4, ic4 = xjumpm(NQNB, ia3, ic3, iran1)
    _, ia5, ic5 = xjumpm(NB, ia3, ic3, iran1)
    itmp3, _, _ = xjumpm(MRCOL, ia5, ic5, iran1)
    iran1, _, _ = xjumpm(MB * MRROW, mult, iadd, itmp3)
    itmp1, _, _ = xjumpm(NOFF, ia4, ic4, iran1)
    iran1, _, _ = xjumpm(MOFF, ia2, ic2, itmp1)
    rng.setran(iran1, ia1, ic1)
    ib1, ib2, ib3 = list(iran1), list(iran1), list(iran1)
    JK = 1
    done = False
    for IC in range(NOFF + 1, NEND + 1):
        IOFFC = ((IC - 1) * 1 + MRCOL) * NB
        for I in range(1, NB + 1):
            if JK > ICNUM:
                done = True
                break
            IK = 1
            for IR in range(MOFF + 1, MEND + 1):
                IOFFR = ((IR - 1) * 1 + MRROW) * MB
                stop = False
                if IOFFR > IOFFC:
                    for _J in range(1, MB + 1):
                        if IK > IRNUM:
                            stop = True
                            break
                        A[IK, JK] = 1.0 - 2.0 * rng.pdrand()
                        IK += 1
                elif IOFFC == IOFFR:
                    IK = IK + I - 1
                    if IK > IRNUM:
                        stop = True
                    else:
                        for _J in range(1, I):
                            A[IK, JK] = 1.0 - 2.0 * rng.pdrand()
                        A[IK, JK] = 1.0 - 2.0 * rng.pdrand()
                        for J in range(1, MB - I + 1):
                            if IK + J > IRNUM:
                                stop = True
                                break
                            A[IK + J, JK] = 1.0 - 2.0 * rng.pdrand()
                            A[IK, JK + J] = A[IK + J, JK]
                        if not stop:
                            IK = IK + MB - I + 1
                else:
                    IK += MB
                if stop:
                    break
                ib1 = rng.jumpit(ia2, ic2, ib1)
            JK += 1
            iran3 = rng.jumpit(ia3, ic3, ib2)
            ib1, ib2 = list(iran3), list(iran3)
        if done:
            break
        iran4 = rng.jumpit(ia4, ic4, ib3)
        ib1, ib2, ib3 = list(iran4), list(iran4), list(iran4)

    # ---- upper triangular part, pdmatgen.f:307-378
    mult, iadd, jseed = [mult0, mult1], [iadd0, iadd1], [iseed, 0]
    iran1, ia1, ic1 = xjumpm(1, mult, iadd, jseed)
    _, ia2, ic2 = xjumpm(NQNB, mult, iadd, iran1)
    _, ia3, ic3 = xjumpm(N, mult, iadd, iran1)
    _, ia4, ic4 = xjumpm(NPMB, ia3, ic3, iran1)
    _, ia5, ic5 = xjumpm(MB, ia3, ic3, iran1)
    itmp3, _, _ = xjumpm(MRROW, ia5, ic5, iran1)
    iran1, _, _ = xjumpm(NB * MRCOL, mult, iadd, itmp3)
    itmp1, _, _ = xjumpm(MOFF, ia4, ic4, iran1)
    iran1, _, _ = xjumpm(NOFF, ia2, ic2, itmp1)
    rng.setran(iran1, ia1, ic1)
    ib1, ib2, ib3 = list(iran1), list(iran1), list(iran1)
    IK = 1
    done = False
    for IR in range(MOFF + 1, MEND + 1):
        IOFFR = ((IR - 1) * 1 + MRROW) * MB
        for _J in range(1, MB + 1):
            if IK > IRNUM:
                done = True
                break
            JK = 1
            for IC in range(NOFF + 1, NEND + 1):
                IOFFC = ((IC - 1) * 1 + MRCOL) * NB
                stop = False
                if IOFFC > IOFFR:
                    for _I in range(1, NB + 1):
                        if JK > ICNUM:
                            stop = True
                            break
                        A[IK, JK] = 1.0 - 2.0 * rng.pdrand()
                        JK += 1
                else:
                    JK += NB
                if stop:
                    break
                ib1 = rng.jumpit(ia2, ic2, ib1)
            IK += 1
            iran3 = rng.jumpit(ia3, ic3, ib2)
            ib1, ib2 = list(iran3), list(iran3)
        if done:
            break
        iran4 = rng.jumpit(ia4, ic4, ib3)
        ib1, ib2, ib3 = list(iran4), list(iran4), list(iran4)

    # ---- diagonal dominance, pdmatgen.f:516-543
    MAXMN = max(M, N)
    JK = 1
    for IC in range(NOFF + 1, NEND + 1):
        IOFFC = ((IC - 1) * 1 + MRCOL) * NB
        IK = 1
        for IR in range(MOFF + 1, MEND + 1):
            IOFFR = ((IR - 1) * 1 + MRROW) * MB
            if IOFFC == IOFFR:
                stop = False
                for J in range(0, MB):
                    if IK > IRNUM:
                        stop = True
                        break
                    A[IK, JK + J] = abs(A[IK, JK + J]) + MAXMN
                    IK += 1
                if stop:
                    break
            else:
                IK += MB
        JK += NB
    return np.asfortranarray(A[1:, 1:])


# ----------------------------------------------------------------------------------
# Panel sizing and the panel loop (oocdag.cpp:59-66, 478-492).
# ----------------------------------------------------------------------------------
def find_yn(bb: int, mem_block: int, jb: int, state: list) -> int:
    Yn = state[0]
    Ym = bb - jb
    if Ym * (Ym + 1) <= (mem_block - Ym) * 2:
        Yn = Ym
    else:
        while (mem_block - Ym) * 2 >= (2 * Ym - Yn) * (Yn + 1):
            if Yn == Ym:
                break
            Yn += 1
    state[0] = Yn
    return Yn


def panel_plan(N: int, NB: int, memsize: int):
    bb = (N + NB - 1) // NB
    mem_block = memsize // 8 // NB // NB
    state = [0]
    out = []
    JB = jb = 0
    while JB < N:
        Ym = bb - jb
        Yn = find_yn(bb, mem_block, jb, state)
        YN = min((jb + Yn) * NB, N) - jb * NB
        out.append((jb, Ym, Yn))
        JB += YN
        jb += Yn
    return mem_block, out


PLAN_CASES = [
    # (label, N, NB, memsize bytes)
    ("c0_n4096_nb256_24GB", 4096, 256, 24_000_000_000),
    ("c1_n163840_nb1024_24e9B", 163840, 1024, 24_000_000_000),
    ("c1_n163840_nb1024_24GiB", 163840, 1024, 24 << 30),
    ("c2_n65536_nb512_24GiB", 65536, 512, 24 << 30),
    ("bench_n40960_nb1024_2GiB", 40960, 1024, 2 << 30),
    ("small_n1000_nb64_40tiles", 1000, 64, 40 * 64 * 64 * 8),
    ("small_n96_nb32_10tiles", 96, 32, 10 * 32 * 32 * 8),
    ("ragged_n1001_nb128_30tiles", 1001, 128, 30 * 128 * 128 * 8),
]


# ----------------------------------------------------------------------------------
# Program-order execution of the reference task list on SciPy's BLAS.
# ----------------------------------------------------------------------------------
def chol_program_order(A: np.ndarray, NB: int, memsize: int) -> tuple[np.ndarray, int]:
    from scipy.linalg import blas, lapack

    N = A.shape[1]
    LDA = A.shape[0]
    A = A.copy(order="F")
    flat = A.reshape(-1, order="F")
    bb = (N + NB - 1) // NB
    mem_block = memsize // 8 // NB // NB
    Y = np.zeros(mem_block * NB * NB)

    def hview(off, m, n):  # strided host block at flat offset `off`
        return np.lib.stride_tricks.as_strided(flat[off:], shape=(m, n), strides=(8, 8 * LDA))

    def dview(buf, off, m, n):  # packed tile, ld = NB
        return np.lib.stride_tricks.as_strided(buf[off:], shape=(m, n), strides=(8, 8 * NB))

    def yoff(ib, jb, Ym):
        return (ib + jb * Ym - (jb * (jb + 1)) // 2) * NB * NB

    def syrk(Xbuf, xoff0, Ybuf, yoff0, H, K):
        Ym = (H + NB - 1) // NB
        for jb, JB in enumerate(range(0, K, NB)):
            LN = min(JB + NB, K) - JB
            xt = dview(Xbuf, xoff0 + jb * NB * NB, LN, NB)
            ct = dview(Ybuf, yoff0 + yoff(jb, jb, Ym), LN, LN)
            r = blas.dsyrk(-1.0, np.asfortranarray(xt), beta=1.0, c=np.asfortranarray(ct), lower=1)
            ct[:, :] = np.where(np.tri(LN, dtype=bool), r, ct)  # dsyrk('L') updates the lower triangle
            for ib, IB in zip(range(jb + 1, 10 ** 9), range(JB + NB, H, NB)):
                LM = min(IB + NB, H) - IB
                at = dview(Xbuf, xoff0 + ib * NB * NB, LM, NB)
                bt = dview(Xbuf, xoff0 + jb * NB * NB, LN, NB)
                cc = dview(Ybuf, yoff0 + yoff(ib, jb, Ym), LM, LN)
                cc[:, :] = blas.dgemm(-1.0, np.asfortranarray(at), np.asfortranarray(bt), beta=1.0,
                                      c=np.asfortranarray(cc), trans_b=1)

    info = 0
    JB = jb = 0
    state = [0]
    while JB < N:
        Ym = bb - jb
        Yn = find_yn(bb, mem_block, jb, state)
        YM = N - JB
        YN = min((jb + Yn) * NB, N) - jb * NB
        xoff = (mem_block - Ym) * NB * NB
        base = jb * NB * LDA + jb * NB
        # A2Y
        for jj, JJ in enumerate(range(0, YN, NB)):
            LN = min(JJ + NB, YN) - JJ
            for ii, II in zip(range(jj, 10 ** 9), range(JJ, YM, NB)):
                LM = min(II + NB, YM) - II
                dview(Y, yoff(ii, jj, Ym), LM, LN)[:, :] = hview(base + jj * NB * LDA + ii * NB, LM, LN)
        for jjb in range(jb):
            src = jjb * NB * LDA + jb * NB
            for ii, II in enumerate(range(0, YM, NB)):
                LM = min(II + NB, YM) - II
                dview(Y, xoff + ii * NB * NB, LM, NB)[:, :] = hview(src + ii * NB, LM, NB)
            syrk(Y, xoff, Y, 0, YM, YN)
        # in-core
        for jj, JJ in enumerate(range(0, YN, NB)):
            LN = min(JJ + NB, YN) - JJ
            dtile = dview(Y, yoff(jj, jj, Ym), LN, LN)
            hdiag = hview(base + jj * NB * LDA + jj * NB, LN, LN)
            hdiag[:, :] = dtile
            c, inf = lapack.dpotrf(np.asfortranarray(hdiag), lower=1, clean=0)
            hdiag[:, :] = c
            if inf > 0 and info == 0:
                info = JB + JJ + inf
            dtile[:, :] = hdiag
            for ii, II in zip(range(jj + 1, 10 ** 9), range(JJ + NB, YM, NB)):
                LM = min(II + NB, YM) - II
                bt = dview(Y, yoff(ii, jj, Ym), LM, LN)
                bt[:, :] = blas.dtrsm(1.0, np.asfortranarray(dtile), np.asfortranarray(bt), side=1, lower=1,
                                      trans_a=1, diag=0)
                hview(base + jj * NB * LDA + ii * NB, LM, LN)[:, :] = bt
            if JJ + NB < YN:
                H = YM - JJ - NB
                K = YN - JJ - NB
                syrk(Y, yoff(jj + 1, jj, Ym), Y, yoff(jj + 1, jj + 1, Ym), H, K)
        JB += YN
        jb += Yn
    return A, info


def main():
    cases = [(8, 3, 100), (9, 3, 100), (7, 7, 100), (10, 4, 100), (16, 5, 100), (33, 8, 100), (12, 4, 7)]
    arrs = {}
    for n, nb, seed in cases:
        arrs[f"n{n}_nb{nb}_seed{seed}"] = pdmatgen_symm_diag(n, nb, seed)
    np.savez_compressed(os.path.join(HERE, "pdmatgen_literal.npz"), **arrs)

    plans = {}
    for label, N, NB, mem in PLAN_CASES:
        mb, plan = panel_plan(N, NB, mem)
        plans[label] = {"N": N, "NB": NB, "memsize": mem, "memBlock": mb, "panels": plan}
    with open(os.path.join(HERE, "panel_plans.json"), "w") as f:
        json.dump(plans, f, indent=1)

    # Program-order run on a small uniform-generator matrix: n=96, nb=32, 10 tiles
    # (three panels), and a ragged case n=100, nb=32.
    import sys

    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    import oracle  # generator only (closed form checked separately)

    out = {}
    for n, nb, tiles in [(96, 32, 10), (100, 32, 12)]:
        A = oracle.gen_uniform(n, 100, float(n))
        L, info = chol_program_order(A, nb, tiles * nb * nb * 8)
        out[f"A_n{n}_nb{nb}"] = A
        out[f"L_n{n}_nb{nb}_tiles{tiles}"] = L
        assert info == 0
    np.savez_compressed(os.path.join(HERE, "chol_program_order.npz"), **out)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
