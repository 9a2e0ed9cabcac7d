"""ctypes binding of the serving runtime (ooc_server_* in include/oocdag_gb300.h).

The scheduler, batcher and worker pipelines are native (oocdag_gb300/csrc/server.cu);
this module only mirrors the C structures and calls.
"""
from __future__ import annotations

import ctypes

from . import OocError, PRECISIONS, load


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("workers", ctypes.c_int), ("small_max_n", ctypes.c_int),
                ("nb", ctypes.c_int), ("prec", ctypes.c_int), ("tol", ctypes.c_double),
                ("batch_window_ms", ctypes.c_double), ("hbm_budget", ctypes.c_int64),
                ("ooc_min_n", ctypes.c_int64), ("ooc_budget", ctypes.c_int64)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("n", ctypes.c_int64), ("matrix_seed", ctypes.c_uint64),
                ("rhs_seed", ctypes.c_uint64), ("key", ctypes.c_int64), ("keep_solution", ctypes.c_int)]


class Completion(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int), ("info", ctypes.c_int), ("path", ctypes.c_int),
                ("factor_reused", ctypes.c_int), ("iterations", ctypes.c_int), ("backward_error", ctypes.c_double),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double),
                ("x_sum", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_bound = False


def _lib():
    global _bound
    L = load()
    if not _bound:
        P = ctypes.c_void_p
        L.ooc_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(P)]
        L.ooc_server_submit.argtypes = [P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_int64)]
        L.ooc_server_poll.argtypes = [P, ctypes.POINTER(Completion), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.c_int]
        L.ooc_server_solution.argtypes = [P, ctypes.c_int64, P, ctypes.c_int64]
        L.ooc_server_status.argtypes = [P] + [ctypes.POINTER(ctypes.c_int64)] * 4
        L.ooc_server_now.argtypes = [P]
        L.ooc_server_now.restype = ctypes.c_double
        L.ooc_server_destroy.argtypes = [P]
        L.ooc_server_last_error.argtypes = [P]
        L.ooc_server_last_error.restype = ctypes.c_char_p
        _bound = True
    return L


class Server:
    def __init__(self, device=0, workers=4, small_max_n=512, nb=512, prec="bf16x3", tol=1e-14,
                 batch_window_ms=0.5, hbm_budget=0, ooc_min_n=0, ooc_budget=0):
        cfg = ServerConfig(device, workers, small_max_n, nb, PRECISIONS[prec] if isinstance(prec, str) else prec,
                           tol, batch_window_ms, hbm_budget, ooc_min_n, ooc_budget)
        p = ctypes.c_void_p()
        rc = _lib().ooc_server_create(ctypes.byref(cfg), ctypes.byref(p))
        if rc:
            raise OocError(rc, "ooc_server_create")
        self._s = p
        self._buf = (Completion * 256)()

    def submit(self, n: int, matrix_seed: int, rhs_seed: int, key: int, kind: int = 0, keep_solution: bool = False):
        r = Request(kind, n, matrix_seed, rhs_seed, key, 1 if keep_solution else 0)
        rid = ctypes.c_int64()
        rc = _lib().ooc_server_submit(self._s, ctypes.byref(r), ctypes.byref(rid))
        if rc:
            raise OocError(rc, "ooc_server_submit")
        return rid.value

    def poll(self, wait_ms: int = 0) -> list[dict]:
        cnt = ctypes.c_int(0)
        out = []
        while True:
            rc = _lib().ooc_server_poll(self._s, self._buf, len(self._buf), ctypes.byref(cnt), wait_ms)
            if rc:
                raise OocError(rc, "ooc_server_poll")
            out += [self._buf[i].as_dict() for i in range(cnt.value)]
            if cnt.value < len(self._buf):
                return out
            wait_ms = 0

    def solution(self, rid: int, n: int):
        import numpy as np

        x = np.empty(n)
        rc = _lib().ooc_server_solution(self._s, rid, x.ctypes.data, n)
        if rc:
            raise OocError(rc, "ooc_server_solution")
        return x

    def status(self) -> dict:
        v = [ctypes.c_int64() for _ in range(4)]
        _lib().ooc_server_status(self._s, *[ctypes.byref(x) for x in v])
        return dict(zip(["pending", "running", "resident_bytes", "reserved_bytes"], [x.value for x in v]))

    def last_error(self) -> str:
        return (_lib().ooc_server_last_error(self._s) or b"").decode()

    def now(self) -> float:
        return _lib().ooc_server_now(self._s)

    def close(self) -> None:
        if self._s:
            _lib().ooc_server_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
