"""ctypes binding of the tile-offload interface (include/ooc_offload.h).

Mirrors the reference's ``offload_*`` calls (ooc_offload.h:28-64) one to one: device
pointers are plain integers from ``Alloc``, scalars are passed by reference where the
reference passes them by reference (the Fortran-style BLAS arguments).
"""
from __future__ import annotations

import ctypes

from . import _ptr, load

_I = ctypes.c_int
_D = ctypes.c_double
_P = ctypes.c_void_p
_bound = False


def _lib():
    global _bound
    L = load()
    if not _bound:
        PI, PD = ctypes.POINTER(_I), ctypes.POINTER(_D)
        L.offload_init.argtypes = [PI, PI]
        L.offload_destroy.argtypes = []
        L.offload_Alloc.argtypes = [ctypes.c_size_t, _I]
        L.offload_Alloc.restype = ctypes.c_int64
        L.offload_touch.argtypes = [_P, ctypes.c_size_t, _I]
        L.offload_Free.argtypes = [_P, _I]
        for name in ("offload_dSetVector", "offload_dGetVector"):
            getattr(L, name).argtypes = [_I, _P, _I, _P, _I, _I]
        L.offload_dcopy.argtypes = [_I, _P, _I, _P, _I, _I]
        for name in ("offload_dSetMatrix", "offload_dGetMatrix"):
            getattr(L, name).argtypes = [_I, _I, _P, _I, _P, _I, _I]
        for name in ("offload_dtrSetMatrix", "offload_dtrGetMatrix"):
            getattr(L, name).argtypes = [ctypes.c_char, _I, _I, _P, _I, _P, _I, _I]
        L.offload_dgemm.argtypes = [ctypes.c_char_p, ctypes.c_char_p, PI, PI, PI, PD, _P, PI, _P, PI, PD, _P, PI, _I]
        L.offload_dsyrk.argtypes = [ctypes.c_char_p, ctypes.c_char_p, PI, PI, PD, _P, PI, PD, _P, PI, _I]
        L.offload_dtrsm.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, PI, PI, PD,
                                    _P, PI, _P, PI, _I]
        L.offload_dpotrf.argtypes = [ctypes.c_char_p, PI, _P, PI, PI, _I]
        L.ooc_offload_last_error.restype = _I
        _bound = True
    return L


def _i(v):
    return ctypes.byref(_I(int(v)))


def _d(v):
    return ctypes.byref(_D(float(v)))


def init(rank: int = 0) -> int:
    dev = _I(-1)
    _lib().offload_init(ctypes.byref(_I(rank)), ctypes.byref(dev))
    return dev.value


def destroy() -> None:
    _lib().offload_destroy()


def last_error() -> int:
    return _lib().ooc_offload_last_error()


def Alloc(size: int, r: int = 0) -> int:
    return int(_lib().offload_Alloc(size, r))


def touch(p: int, size: int, r: int = 0) -> None:
    _lib().offload_touch(p, size, r)


def Free(p: int, r: int = 0) -> None:
    _lib().offload_Free(p, r)


def dSetVector(n, x, incx, y, incy, r=0):
    _lib().offload_dSetVector(n, _ptr(x), incx, _ptr(y), incy, r)


def dGetVector(n, x, incx, y, incy, r=0):
    _lib().offload_dGetVector(n, _ptr(x), incx, _ptr(y), incy, r)


def dcopy(n, x, incx, y, incy, r=0):
    _lib().offload_dcopy(n, _ptr(x), incx, _ptr(y), incy, r)


def dSetMatrix(rows, cols, A, lda, B, ldb, r=0):
    _lib().offload_dSetMatrix(rows, cols, _ptr(A), lda, _ptr(B), ldb, r)


def dGetMatrix(rows, cols, A, lda, B, ldb, r=0):
    _lib().offload_dGetMatrix(rows, cols, _ptr(A), lda, _ptr(B), ldb, r)


def dtrSetMatrix(uplo, rows, cols, A, lda, B, ldb, r=0):
    _lib().offload_dtrSetMatrix(uplo.encode(), rows, cols, _ptr(A), lda, _ptr(B), ldb, r)


def dtrGetMatrix(uplo, rows, cols, A, lda, B, ldb, r=0):
    _lib().offload_dtrGetMatrix(uplo.encode(), rows, cols, _ptr(A), lda, _ptr(B), ldb, r)


def dgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, r=0):
    _lib().offload_dgemm(transa.encode(), transb.encode(), _i(m), _i(n), _i(k), _d(alpha), _ptr(a), _i(lda), _ptr(b),
                         _i(ldb), _d(beta), _ptr(c), _i(ldc), r)


def dsyrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc, r=0):
    _lib().offload_dsyrk(uplo.encode(), trans.encode(), _i(n), _i(k), _d(alpha), _ptr(a), _i(lda), _d(beta), _ptr(c),
                         _i(ldc), r)


def dtrsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb, r=0):
    _lib().offload_dtrsm(side.encode(), uplo.encode(), transa.encode(), diag.encode(), _i(m), _i(n), _d(alpha),
                         _ptr(a), _i(lda), _ptr(b), _i(ldb), r)


def dpotrf(uplo, n, a, lda, r=0) -> int:
    info = _I(0)
    _lib().offload_dpotrf(uplo.encode(), _i(n), _ptr(a), _i(lda), ctypes.byref(info), r)
    return info.value
