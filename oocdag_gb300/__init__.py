"""oocdag_gb300: GB300-native out-of-core left-looking tiled Cholesky.

Python mirror of the library's C-ABI (``include/oocdag_gb300.h``).  The compute path is
the CUDA shared library ``_build/liboocdag_gb300.so`` built by ``build.py``; there is no
CPU fallback: if the library is missing or no GPU is present, the calls raise.

Matrices are column-major.  Host matrices are numpy arrays in Fortran order (or any
object with ``ctypes.data``); device matrices are torch CUDA tensors whose storage is
column-major (``t.stride() == (1, lda)``, e.g. ``torch.empty(n, lda).T[:n]``... or simply
a contiguous (n, lda) tensor read as its transpose).  Pointers may also be passed as
plain integers.
"""
from __future__ import annotations

import ctypes
import os
import re
from dataclasses import dataclass

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None

OOC_OK = 0
OOC_ERR_NOMEM = -101
OOC_ERR_CUDA = -102
OOC_ERR_TIMEOUT = -103
OOC_ERR_BUDGET = -104
OOC_ERR_INTERNAL = -105
OOC_ERR_NODEVICE = -106
OOC_ERR_UNSUPPORTED = -107

OPT_X_BUFFERS = 1
OPT_TIMEOUT_MS = 2
OPT_PROFILE = 3
OPT_PIN_HOST = 4
OPT_REF_SCHEDULE = 5
OPT_KEEP_A = 6
OPT_TAIL_ORDER = 7
OPT_POOL_BYTES = 8
OPT_BLOCK_COLS = 9
OPT_COPY_STREAMS = 10

PREC_FP64 = 0
PREC_FP32 = 1
PREC_BF16X3 = 2
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "bf16x3": PREC_BF16X3}


class OocError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = _lib.ooc_last_error_string().decode() if _lib is not None else ""
        super().__init__(f"{where} failed with status {code}" + (f": {msg}" if msg else ""))
        self.code = code


class OocStats(ctypes.Structure):
    _fields_ = [
        ("seconds", ctypes.c_double),
        ("flops", ctypes.c_double),
        ("h2d_bytes", ctypes.c_double),
        ("d2h_bytes", ctypes.c_double),
        ("npanels", ctypes.c_int),
        ("info", ctypes.c_int),
        ("kernel_launches", ctypes.c_int64),
        ("update_ms", ctypes.c_double),
        ("update_launches", ctypes.c_int64),
        ("update_flops", ctypes.c_double),
        ("factor_ms", ctypes.c_double),
        ("h2d_ms", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib_path() -> str:
    from . import build as _b

    return _b.LIB


def header_functions() -> list[str]:
    """Names of the functions declared in include/*.h (for export checks)."""
    inc = os.path.join(os.path.dirname(_HERE), "include")
    names = []
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = re.sub(r"^\s*#[^\n]*", "", text, flags=re.M)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.append(name)
    return sorted(set(names))


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first if needed).  Raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _b

    if build_if_missing and not _b.up_to_date():
        _b.build()
    if not os.path.exists(_b.LIB):
        raise RuntimeError("oocdag_gb300 CUDA library is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(_b.LIB)
    P, I, I64, U64, D, SZ = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64,
                             ctypes.c_double, ctypes.c_size_t)
    L.ooc_create.argtypes = [ctypes.POINTER(P), I]
    L.ooc_destroy.argtypes = [P]
    L.ooc_set_option.argtypes = [P, I, I64]
    L.ooc_get_option.argtypes = [P, I, ctypes.POINTER(I64)]
    L.ooc_last_error_string.restype = ctypes.c_char_p
    L.ooc_last_info.argtypes = [P]
    L.ooc_dpotrf_L.argtypes = [P, P, I64, I64, I, SZ, ctypes.POINTER(I), ctypes.POINTER(OocStats)]
    L.ooc_spotrf_L.argtypes = [P, P, I64, I64, I, SZ, ctypes.POINTER(I), ctypes.POINTER(OocStats)]
    L.ooc_dpotrs_L.argtypes = [P, P, I64, I64, I, SZ, P, I64, I]
    L.Cholesky.argtypes = [P, P, I, I, I, SZ]
    L.Cholesky.restype = D
    L.ooc_pdpotrf_.argtypes = [ctypes.c_char_p, ctypes.POINTER(I), P, ctypes.POINTER(I), ctypes.POINTER(I),
                               ctypes.POINTER(I), ctypes.POINTER(I)]
    L.ooc_pdpotrf_.restype = None
    L.ooc_pspotrf_.argtypes = [ctypes.c_char_p, ctypes.POINTER(I), P, ctypes.POINTER(I), ctypes.POINTER(I),
                               ctypes.POINTER(I), ctypes.POINTER(I)]
    L.ooc_pspotrf_.restype = None
    L.ooc_dmatgen_pdmatgen.argtypes = [P, P, I64, I64, I]
    L.ooc_dmatgen_uniform.argtypes = [P, P, I64, I64, U64, D]
    L.ooc_dresidual.argtypes = [P, P, I64, I64, I, U64, D, ctypes.POINTER(D)]
    L.ooc_fp64_peak_probe.argtypes = [P, D, ctypes.POINTER(D)]
    L.ooc_panel_plan.argtypes = [I64, I, I64, I, ctypes.POINTER(I), I]
    L.ooc_get_stream.argtypes = [P, I, ctypes.POINTER(P)]
    L.ooc_dpotrf_L_static.argtypes = [P, I64, I64, I, P, ctypes.POINTER(I)]
    L.ooc_factor_create.argtypes = [P, P, I64, I64, I, I, ctypes.POINTER(P), ctypes.POINTER(I),
                                    ctypes.POINTER(OocStats)]
    L.ooc_factor_destroy.argtypes = [P]
    L.ooc_dsyrk_ln.argtypes = [P, I, I, I, P, I64, P, I64]
    L.ooc_factor_create_gen.argtypes = [P, I64, U64, D, I, I, ctypes.POINTER(P), ctypes.POINTER(I),
                                        ctypes.POINTER(OocStats)]
    L.ooc_solve_refine_gen.argtypes = [P, P, U64, D, P, I64, P, I64, I, D, I, ctypes.POINTER(I), ctypes.POINTER(D)]
    L.ooc_factor_bytes.argtypes = [I64, I, I]
    L.ooc_factor_bytes.restype = I64
    L.ooc_gen_normal.argtypes = [P, P, I64, I64, I, U64]
    for name in ("ooc_batched_dposv", "ooc_batched_sposv"):
        getattr(L, name).argtypes = [P, I, ctypes.POINTER(I), ctypes.POINTER(I64), ctypes.POINTER(I64), P, P,
                                     ctypes.POINTER(I), ctypes.POINTER(I), I, ctypes.POINTER(D)]
    L.ooc_factor_copy_L.argtypes = [P, P, I64]
    L.ooc_factor_solve.argtypes = [P, P, P, I64, I]
    L.ooc_solve_refine.argtypes = [P, P, P, I64, P, I64, P, I64, I, D, I, ctypes.POINTER(I), ctypes.POINTER(D)]
    _lib = L
    return L


def _ptr(x) -> int:
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    raise TypeError(f"cannot take a device/host pointer of {type(x)}")


def _check(rc: int, where: str) -> None:
    if rc != OOC_OK:
        raise OocError(rc, where)


def panel_plan(n: int, nb: int, mem_block: int, nx: int = 1) -> list[tuple[int, int, int]]:
    """(jb, Ym, Yn) panels of the left-looking loop; nx X buffers counted (1 = reference)."""
    L = load()
    cap = 8192
    buf = (ctypes.c_int * (3 * cap))()
    rc = L.ooc_panel_plan(n, nb, mem_block, nx, buf, cap)
    if rc < 0:
        raise OocError(rc, "ooc_panel_plan")
    return [(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]) for i in range(rc)]


@dataclass
class Result:
    info: int
    stats: dict


class Handle:
    """One library handle (streams, status word, pooled device panel buffer)."""

    def __init__(self, device: int = 0):
        L = load()
        h = ctypes.c_void_p()
        _check(L.ooc_create(ctypes.byref(h), device), "ooc_create")
        self._h = h
        self.device = device

    @property
    def ptr(self) -> ctypes.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            load().ooc_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _after_torch(self, *xs) -> None:
        """The library runs on the handle's own streams.  When an argument is a CUDA tensor,
        torch work that produced it may still be in flight on torch's current stream: make
        the handle's compute and host-to-device streams wait for it (an event, no host
        synchronisation).  Every call returns after its own streams finished, so results are
        ready for torch afterwards."""
        for x in xs:
            if getattr(x, "is_cuda", False):
                import torch

                ev = torch.cuda.Event()
                ev.record(torch.cuda.current_stream(x.device))
                if getattr(self, "_ext_streams", None) is None:
                    self._ext_streams = [torch.cuda.ExternalStream(self.stream(w), device=x.device) for w in (0, 1)]
                for st in self._ext_streams:
                    st.wait_event(ev)
                return

    def stream(self, which: int = 0) -> int:
        """cudaStream_t of the handle (0 compute, 1 host-to-device, 2 device-to-host)."""
        p = ctypes.c_void_p()
        _check(load().ooc_get_stream(self._h, which, ctypes.byref(p)), "ooc_get_stream")
        return p.value or 0

    def set_option(self, key: int, value: int) -> None:
        _check(load().ooc_set_option(self._h, key, int(value)), "ooc_set_option")

    def get_option(self, key: int) -> int:
        v = ctypes.c_int64()
        _check(load().ooc_get_option(self._h, key, ctypes.byref(v)), "ooc_get_option")
        return v.value

    def dpotrf_L(self, A, n: int, lda: int, nb: int, budget: int) -> Result:
        """Lower Cholesky in place (host A: out of core through `budget` bytes; device A:
        in core).  Returns the LAPACK info and the call's statistics."""
        info = ctypes.c_int(0)
        st = OocStats()
        self._after_torch(A)
        rc = load().ooc_dpotrf_L(self._h, _ptr(A), n, lda, nb, budget, ctypes.byref(info), ctypes.byref(st))
        _check(rc, "ooc_dpotrf_L")
        return Result(info.value, st.as_dict())

    def dpotrs_L(self, L, n: int, ldl: int, nb: int, B, ldb: int, nrhs: int, budget: int = 0) -> None:
        """B := A^{-1} B with the lower factor L (host or device, as dpotrf_L leaves it); a
        host L is streamed through the device in nb-wide panels.  B (host or device) holds
        nrhs <= 16 columns of leading dimension ldb."""
        self._after_torch(L, B)
        _check(load().ooc_dpotrs_L(self._h, _ptr(L), n, ldl, nb, budget, _ptr(B), ldb, nrhs), "ooc_dpotrs_L")

    def spotrf_L(self, A, n: int, lda: int, nb: int, budget: int = 0) -> Result:
        """FP32 lower Cholesky in place (device A: in place; host A: on a device copy that
        must fit in `budget` bytes, 0 = 3/4 of free memory)."""
        info = ctypes.c_int(0)
        st = OocStats()
        self._after_torch(A)
        rc = load().ooc_spotrf_L(self._h, _ptr(A), n, lda, nb, budget, ctypes.byref(info), ctypes.byref(st))
        _check(rc, "ooc_spotrf_L")
        return Result(info.value, st.as_dict())

    def matgen_uniform(self, A, n: int, lda: int, seed: int, alpha: float) -> None:
        self._after_torch(A)
        _check(load().ooc_dmatgen_uniform(self._h, _ptr(A), n, lda, seed, float(alpha)), "ooc_dmatgen_uniform")

    def matgen_pdmatgen(self, A, n: int, lda: int, seed: int = 100) -> None:
        self._after_torch(A)
        _check(load().ooc_dmatgen_pdmatgen(self._h, _ptr(A), n, lda, seed), "ooc_dmatgen_pdmatgen")

    def residual(self, L, n: int, lda: int, kind: str, seed: int, alpha: float = 0.0) -> float:
        r = ctypes.c_double()
        k = 0 if kind == "uniform" else 1
        self._after_torch(L)
        _check(load().ooc_dresidual(self._h, _ptr(L), n, lda, k, seed, float(alpha), ctypes.byref(r)),
               "ooc_dresidual")
        return r.value

    def factor(self, A, n: int, lda: int, nb: int, prec="fp64") -> "Factor":
        """In-core factorization with trailing updates in `prec` ('fp64', 'fp32',
        'bf16x3'); A (host or device) is left unchanged."""
        p = PRECISIONS[prec] if isinstance(prec, str) else int(prec)
        F = ctypes.c_void_p()
        info = ctypes.c_int(0)
        st = OocStats()
        self._after_torch(A)
        _check(load().ooc_factor_create(self._h, _ptr(A), n, lda, nb, p, ctypes.byref(F), ctypes.byref(info),
                                        ctypes.byref(st)), "ooc_factor_create")
        return Factor(self, F, n, info.value, st.as_dict())

    def factor_gen(self, n: int, seed: int, alpha: float, nb: int, prec="bf16x3") -> "Factor":
        """Factor the uniform test matrix of `seed` generated in place (no copy of A kept)."""
        p = PRECISIONS[prec] if isinstance(prec, str) else int(prec)
        F = ctypes.c_void_p()
        info = ctypes.c_int(0)
        st = OocStats()
        _check(load().ooc_factor_create_gen(self._h, n, seed, float(alpha), nb, p, ctypes.byref(F),
                                            ctypes.byref(info), ctypes.byref(st)), "ooc_factor_create_gen")
        f = Factor(self, F, n, info.value, st.as_dict())
        f.gen = (seed, float(alpha))
        return f

    def gen_normal(self, B, n: int, ldb: int, nrhs: int, seed: int) -> None:
        self._after_torch(B)
        _check(load().ooc_gen_normal(self._h, _ptr(B), n, ldb, nrhs, seed), "ooc_gen_normal")

    def dsyrk_ln(self, prec, n: int, k: int, A, lda: int, C, ldc: int) -> None:
        """C := C - A A^T (lower) on the device with the given update precision."""
        p = PRECISIONS[prec] if isinstance(prec, str) else int(prec)
        self._after_torch(A, C)
        _check(load().ooc_dsyrk_ln(self._h, p, n, k, _ptr(A), lda, _ptr(C), ldc), "ooc_dsyrk_ln")

    def batched_posv(self, prec: str, ns, a_off, b_off, A, B, blk_table=None, ctas_per_sm: int = 0):
        """Factor and solve len(ns) SPD systems in one persistent launch (A, B on the device,
        matrix i at element offset a_off[i] with ld = ns[i], right-hand side at b_off[i]).
        prec: 'fp64' or 'fp32' (the storage and arithmetic type of A and B).  Returns
        (info list, kernel seconds)."""
        count = len(ns)
        n_arr = (ctypes.c_int * count)(*[int(x) for x in ns])
        ao = (ctypes.c_int64 * count)(*[int(x) for x in a_off])
        bo = (ctypes.c_int64 * count)(*[int(x) for x in b_off])
        info = (ctypes.c_int * count)()
        tbl = None
        if blk_table is not None:
            tbl = (ctypes.c_int * 16)(*[int(x) for x in blk_table])
        sec = ctypes.c_double(0)
        self._after_torch(A, B)
        fn = load().ooc_batched_dposv if prec == "fp64" else load().ooc_batched_sposv
        _check(fn(self._h, count, n_arr, ao, bo, _ptr(A), _ptr(B), info, tbl, ctas_per_sm, ctypes.byref(sec)),
               "ooc_batched_posv")
        return list(info), sec.value

    def fp64_peak(self, ms: float = 200.0) -> float:
        r = ctypes.c_double()
        _check(load().ooc_fp64_peak_probe(self._h, float(ms), ctypes.byref(r)), "ooc_fp64_peak_probe")
        return r.value


def Cholesky(A, N: int, NB: int, LDA: int, memsize: int, handle: Handle | None = None) -> float:
    """Reference-shaped driver entry (oocdag.cpp:18): returns the factorization time in
    seconds.  Raises on a library error; a non-SPD input is reported by last_info()."""
    L = load()
    t = L.Cholesky(handle.ptr if handle else None, _ptr(A), N, NB, LDA, memsize)
    if t < 0:
        raise OocError(int(t), "Cholesky")
    return t


def last_info(handle: Handle) -> int:
    return load().ooc_last_info(handle.ptr)


def pdpotrf(uplo: str, n: int, A, ia: int, ja: int, desca) -> int:
    """ScaLAPACK-style pdpotrf_ on a 1x1 grid; returns info."""
    L = load()
    d = (ctypes.c_int * 9)(*[int(x) for x in desca])
    info = ctypes.c_int(0)
    L.ooc_pdpotrf_(uplo.encode(), ctypes.byref(ctypes.c_int(n)), _ptr(A), ctypes.byref(ctypes.c_int(ia)),
                   ctypes.byref(ctypes.c_int(ja)), d, ctypes.byref(info))
    return info.value


def pspotrf(uplo: str, n: int, A, ia: int, ja: int, desca) -> int:
    """ScaLAPACK-style pspotrf_ (FP32) on a 1x1 grid; returns info.  The device budget is
    the OOC_DEVICE_BUDGET_MB environment variable, else 3/4 of free device memory."""
    L = load()
    d = (ctypes.c_int * 9)(*[int(x) for x in desca])
    info = ctypes.c_int(0)
    L.ooc_pspotrf_(uplo.encode(), ctypes.byref(ctypes.c_int(n)), _ptr(A), ctypes.byref(ctypes.c_int(ia)),
                   ctypes.byref(ctypes.c_int(ja)), d, ctypes.byref(info))
    return info.value


def dpotrf_L_static(A, n: int, lda: int, nb: int, stream: int = 0) -> int:
    """Allocation-free out-of-core Cholesky (ooc_dpotrf_L_static): the panel buffer is the
    library's fixed static device array, the work runs on `stream`.  Returns LAPACK info;
    raises OocError (OOC_ERR_BUDGET) when the matrix does not fit the static buffer."""
    info = ctypes.c_int(0)
    _check(load().ooc_dpotrf_L_static(_ptr(A), n, lda, nb, stream or None, ctypes.byref(info)),
           "ooc_dpotrf_L_static")
    return info.value


class Factor:
    """A factor kept on the device for repeated solves (ooc_factor)."""

    def __init__(self, handle: Handle, ptr, n: int, info: int, stats: dict):
        self.gen = None
        self.handle = handle
        self._f = ptr
        self.n = n
        self.info = info
        self.stats = stats

    def close(self) -> None:
        if self._f:
            load().ooc_factor_destroy(self._f)
            self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def copy_L(self, L, ldl: int) -> None:
        self.handle._after_torch(L)
        _check(load().ooc_factor_copy_L(self._f, _ptr(L), ldl), "ooc_factor_copy_L")

    def solve(self, B, ldb: int, nrhs: int) -> None:
        """B := A^{-1} B in FP64 (device B)."""
        self.handle._after_torch(B)
        _check(load().ooc_factor_solve(self.handle.ptr, self._f, _ptr(B), ldb, nrhs), "ooc_factor_solve")

    def refine_gen(self, B, ldb: int, X, ldx: int, nrhs: int, tol: float = 1e-14, maxiter: int = 30):
        """Refinement for a factor made by Handle.factor_gen: the residual regenerates A."""
        seed, alpha = self.gen
        it = ctypes.c_int(0)
        be = ctypes.c_double(0)
        self.handle._after_torch(B, X)
        _check(load().ooc_solve_refine_gen(self.handle.ptr, self._f, seed, alpha, _ptr(B), ldb, _ptr(X), ldx, nrhs,
                                           float(tol), int(maxiter), ctypes.byref(it), ctypes.byref(be)),
               "ooc_solve_refine_gen")
        return it.value, be.value

    def refine(self, A, lda: int, B, ldb: int, X, ldx: int, nrhs: int, tol: float = 1e-14, maxiter: int = 30):
        """Iterative refinement to backward error <= tol; returns (iterations, backward error)."""
        it = ctypes.c_int(0)
        be = ctypes.c_double(0)
        self.handle._after_torch(A, B, X)
        _check(load().ooc_solve_refine(self.handle.ptr, self._f, _ptr(A), lda, _ptr(B), ldb, _ptr(X), ldx, nrhs,
                                       float(tol), int(maxiter), ctypes.byref(it), ctypes.byref(be)),
               "ooc_solve_refine")
        return it.value, be.value


def factor_bytes(n: int, nb: int, prec="bf16x3") -> int:
    p = PRECISIONS[prec] if isinstance(prec, str) else int(prec)
    return int(load().ooc_factor_bytes(n, nb, p))
