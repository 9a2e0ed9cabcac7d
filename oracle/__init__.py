"""CPU oracle for the out-of-core left-looking tiled Cholesky (test infrastructure).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
use this package, and only to check or time the GPU library: the product never
imports it.  The C++ restatement lives in ``ooc_oracle.cpp``; this module builds it
(``build()``), loads it with ctypes and wraps it for numpy arrays.

Parity status: pinned to the reference's own code.  ``ref_build.py`` compiles the
reference's ``oocdag.cpp`` and ``oocquark.cpp`` unmodified into ``oracle/_ref`` with host
stand-ins for its absent dependencies (QUARK in program order, cuBLAS v2 and MKL
``dpotrf_`` on SciPy's OpenBLAS); ``tests/test_ref_build.py`` shows the oracle's factor
equal to the compiled reference's bit for bit and its panel plans and task counts equal.
The generator is pinned to the literal-loop restatement of ``LIN/pdmatgen.f`` in
``tests/golden`` (the reference's Fortran is not compiled: no Fortran compiler), and the
tile arithmetic is host BLAS standing in for the reference's MKL/cuBLAS calls.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libooc_oracle.so")
_SRC = os.path.join(_HERE, "ooc_oracle.cpp")

_lib = None


def openblas_path() -> str:
    """Path of SciPy's bundled OpenBLAS (exports ``scipy_d*`` Fortran symbols)."""
    import scipy

    base = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    hits = sorted(glob.glob(os.path.join(base, "libscipy_openblas*.so")))
    if not hits:
        raise RuntimeError("SciPy's bundled OpenBLAS was not found next to scipy")
    return os.path.realpath(hits[0])


def build(force: bool = False) -> str:
    """Compile the C++ oracle into ``oracle/_build`` (host compiler, no GPU)."""
    os.makedirs(_BUILD, exist_ok=True)
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(_SRC):
        return _SO
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", _SRC, "-o", _SO + ".tmp", "-ldl"]
    subprocess.run(cmd, check=True)
    os.replace(_SO + ".tmp", _SO)
    return _SO


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = ctypes.CDLL(_SO)
    c_i64, c_u64, c_dbl, c_int = ctypes.c_int64, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
    P = ctypes.c_void_p
    L.orc_init_blas.argtypes = [ctypes.c_char_p]
    L.orc_init_blas.restype = c_int
    L.orc_set_blas_threads.argtypes = [c_int]
    L.orc_find_Yn.argtypes = [c_int, c_int, c_int, ctypes.POINTER(c_int)]
    L.orc_find_Yn.restype = c_int
    L.orc_panel_plan.argtypes = [c_int, c_int, c_i64, ctypes.POINTER(c_int), c_int]
    L.orc_panel_plan.restype = c_int
    L.orc_cholesky.argtypes = [P, c_int, c_int, c_int, ctypes.c_size_t, c_int, c_int,
                               ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.orc_cholesky.restype = c_dbl
    L.orc_seed_key.argtypes = [c_u64]
    L.orc_seed_key.restype = c_u64
    L.orc_gen_uniform_block.argtypes = [P, c_i64, c_i64, c_u64, c_dbl, c_i64, c_i64, c_i64, c_i64]
    L.orc_gen_pdmatgen_block.argtypes = [P, c_i64, c_i64, c_int, c_i64, c_i64, c_i64, c_i64]
    L.orc_residual.argtypes = [P, c_i64, c_i64, c_int, c_u64, c_dbl, c_int,
                               ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]
    L.orc_residual.restype = c_dbl
    L.orc_potrs.argtypes = [P, c_int, c_int, P, c_int, c_int]
    L.orc_potrs.restype = c_int
    rc = L.orc_init_blas(openblas_path().encode())
    if rc != 0:
        raise RuntimeError(f"oracle: host BLAS init failed ({rc})")
    _lib = L
    return L


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def set_blas_threads(n: int) -> None:
    lib().orc_set_blas_threads(int(n))


def find_Yn(bb: int, memBlock: int, jb: int, state: int) -> tuple[int, int]:
    """Panel width (oocdag.cpp:478-492); returns (Yn, new_state)."""
    s = ctypes.c_int(state)
    yn = lib().orc_find_Yn(bb, memBlock, jb, ctypes.byref(s))
    return yn, s.value


def panel_plan(n: int, nb: int, mem_block: int) -> list[tuple[int, int, int]]:
    """The (jb, Ym, Yn) sequence of the panel loop (oocdag.cpp:59-66)."""
    cap = 4096
    buf = (ctypes.c_int * (3 * cap))()
    np_ = lib().orc_panel_plan(n, nb, mem_block, buf, cap)
    if np_ < 0:
        raise ValueError(f"panel plan failed ({np_})")
    return [(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]) for i in range(np_)]


def gen_uniform(n: int, seed: int, alpha: float, lda: int | None = None) -> np.ndarray:
    """A = (R + R^T)/2 + alpha I, column-major (Fortran order), R from SplitMix64."""
    lda = n if lda is None else lda
    A = np.empty((lda, n), dtype=np.float64, order="F")
    lib().orc_gen_uniform_block(_ptr(A), lda, n, seed, float(alpha), 0, 0, n, n)
    return A


def gen_uniform_block(n: int, seed: int, alpha: float, r0: int, c0: int, m: int, nc: int) -> np.ndarray:
    B = np.empty((m, nc), dtype=np.float64, order="F")
    lib().orc_gen_uniform_block(_ptr(B), m, n, seed, float(alpha), r0, c0, m, nc)
    return B


def gen_pdmatgen(n: int, seed: int = 100, lda: int | None = None) -> np.ndarray:
    """pdmatgen('Symm','Diag') on a 1x1 grid (closed form of LIN/pdmatgen.f)."""
    lda = n if lda is None else lda
    A = np.empty((lda, n), dtype=np.float64, order="F")
    lib().orc_gen_pdmatgen_block(_ptr(A), lda, n, seed, 0, 0, n, n)
    return A


def cholesky(A: np.ndarray, nb: int, memsize: int, nthreads: int = 4, ncomm: int = 2):
    """Run the reference algorithm in place on A (Fortran order, lower).

    Returns (seconds, info, npanels).  ``nthreads=0`` executes every task inline in
    program order (no worker threads).
    """
    assert A.dtype == np.float64 and A.flags.f_contiguous
    n = A.shape[1]
    info = ctypes.c_int(0)
    npan = ctypes.c_int(0)
    t = lib().orc_cholesky(_ptr(A), n, nb, A.shape[0], memsize, nthreads, ncomm,
                           ctypes.byref(info), ctypes.byref(npan))
    return t, info.value, npan.value


def residual(L: np.ndarray, kind: str, seed: int, alpha: float = 0.0, tile: int = 512):
    """Scaled residual ||A - L L^T||_F / (n eps ||A||_F) with A regenerated from its seed.

    ``kind`` is ``"uniform"`` (with ``alpha``) or ``"pdmatgen"``.  Only the lower
    triangle of L is read.
    """
    n = L.shape[1]
    nA = ctypes.c_double(0)
    nR = ctypes.c_double(0)
    k = 0 if kind == "uniform" else 1
    r = lib().orc_residual(_ptr(L), n, L.shape[0], k, seed, float(alpha), tile,
                           ctypes.byref(nA), ctypes.byref(nR))
    return r


def potrs(L: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Solve A X = B given the lower factor L (LAPACK dpotrs)."""
    X = np.array(B, dtype=np.float64, order="F", copy=True)
    if X.ndim == 1:
        X = X.reshape(-1, 1, order="F")
    info = lib().orc_potrs(_ptr(L), L.shape[1], L.shape[0], _ptr(X), X.shape[1], X.shape[0])
    if info != 0:
        raise RuntimeError(f"dpotrs info={info}")
    return X
