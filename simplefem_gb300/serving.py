"""Serving loop with continuous batching (the ``feec_server_*`` part of the C ABI).

``Server.submit`` queues an SPD solve (CSR matrix, right-hand side, tolerance) and
returns at once; worker slots inside the library admit queued requests as soon as a
slot and enough of the device memory budget are free, set them up (upload, Rainbow
coloring, multicolor SSOR layout) and solve each as one thread-block cluster on the
slot's own CUDA stream, so requests overlap on the GPU. ``poll`` returns finished
requests with their solution and timings.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _native
from .solver import _csr, _vec

METHODS = {"cg": _native.METHOD_CG, "rainbow": _native.METHOD_RAINBOW}
MODES = {"fp64": _native.MODE_FP64, "mixed": _native.MODE_MIXED}


class RequestResult(ctypes.Structure):
    _fields_ = [
        ("id", ctypes.c_longlong), ("n", ctypes.c_int), ("status", ctypes.c_int), ("iterations", ctypes.c_int),
        ("outer_iterations", ctypes.c_int), ("cluster_blocks", ctypes.c_int), ("fp64_fallback", ctypes.c_int),
        ("true_relres", ctypes.c_double), ("t_submit_ms", ctypes.c_double), ("t_start_ms", ctypes.c_double),
        ("t_end_ms", ctypes.c_double), ("error_estimate", ctypes.c_double),
    ]


def _declare(L):
    if getattr(L, "_feec_server_declared", False):
        return L
    vp = ctypes.c_void_p
    L.feec_server_create.argtypes = [ctypes.POINTER(vp), ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.feec_server_submit.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_double,
                                     ctypes.POINTER(ctypes.c_longlong)]
    L.feec_server_poll.argtypes = [vp, ctypes.POINTER(RequestResult), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.feec_server_wait.argtypes = [vp, ctypes.c_double]
    L.feec_server_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t),
                                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]
    L.feec_server_destroy.argtypes = [vp]
    L.feec_server_add_operator.argtypes = [vp, ctypes.c_int, vp, vp, vp, ctypes.POINTER(ctypes.c_int)]
    L.feec_server_submit_rhs.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_double, ctypes.POINTER(ctypes.c_longlong)]
    L.feec_server_remove_operator.argtypes = [vp, ctypes.c_int]
    L._feec_server_declared = True
    return L


class Server:
    def __init__(self, hbm_budget_bytes=120 * 10**9, slots=16, method="rainbow", mode="mixed"):
        self._lib = _declare(_native.gpu())
        h = ctypes.c_void_p()
        st = self._lib.feec_server_create(ctypes.byref(h), int(hbm_budget_bytes), int(slots), METHODS[method],
                                          MODES[mode])
        _native.check(st, "feec_server_create")
        self._h = h
        self._live = {}          # id -> arrays kept alive until the request finishes
        self._ops = {}           # resident operator id -> rows
        self._lock = threading.Lock()

    def submit(self, A, C, V, b, precision=1e-10) -> int:
        """Queue A x = b. The host CSR arrays and right-hand side are read by a worker thread
        after this call returns: they are kept alive here until the request is polled, and
        must not be changed before then."""
        n = len(A) - 1
        if n < 1:
            raise ValueError("a request needs at least one row")
        A, C, V = _csr(n, A, C, V)
        b = _vec(b, "b", n)
        x = np.zeros(n)
        rid = ctypes.c_longlong(0)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        with self._lock:
            st = self._lib.feec_server_submit(self._h, len(A) - 1, p(A), p(C), p(V), p(b), p(x), float(precision),
                                              ctypes.byref(rid))
            _native.check(st, "feec_server_submit")
            self._live[rid.value] = (A, C, V, b, x)
        return rid.value

    def add_operator(self, A, C, V) -> int:
        """Upload and prepare a matrix once (coloring, layouts); returns its operator id for
        submit_rhs. Its footprint is reserved in the budget until remove_operator."""
        n = len(A) - 1
        if n < 1:
            raise ValueError("an operator needs at least one row")
        A, C, V = _csr(n, A, C, V)
        op = ctypes.c_int(0)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        _native.check(self._lib.feec_server_add_operator(self._h, n, p(A), p(C), p(V), ctypes.byref(op)),
                      "feec_server_add_operator")
        with self._lock:
            self._ops[op.value] = n
        return op.value

    def submit_rhs(self, op, b, precision=1e-10) -> int:
        """Queue A x = b against a resident operator. The right-hand side is read by a worker
        thread after this call returns: it is kept alive here until the request is polled."""
        with self._lock:
            n = self._ops.get(op)
        if n is None:
            raise ValueError(f"unknown operator {op}")
        b = _vec(b, "b", n)
        x = np.zeros(n)
        rid = ctypes.c_longlong(0)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        with self._lock:
            st = self._lib.feec_server_submit_rhs(self._h, int(op), p(b), p(x), float(precision), ctypes.byref(rid))
            _native.check(st, "feec_server_submit_rhs")
            self._live[rid.value] = (None, None, None, b, x)
        return rid.value

    def remove_operator(self, op) -> None:
        _native.check(self._lib.feec_server_remove_operator(self._h, int(op)), "feec_server_remove_operator")
        with self._lock:
            self._ops.pop(op, None)

    def poll(self, max_out=1024) -> list:
        buf = (RequestResult * max_out)()
        n = ctypes.c_int(0)
        _native.check(self._lib.feec_server_poll(self._h, buf, max_out, ctypes.byref(n)), "feec_server_poll")
        out = []
        with self._lock:
            for i in range(n.value):
                r = buf[i]
                d = {name: getattr(r, name) for name, _ in RequestResult._fields_}
                arrays = self._live.pop(r.id)
                d["x"] = arrays[4]
                d["latency_ms"] = r.t_end_ms - r.t_submit_ms
                d["queue_ms"] = r.t_start_ms - r.t_submit_ms
                out.append(d)
        return out

    def wait(self, timeout_s=600.0) -> bool:
        return self._lib.feec_server_wait(self._h, float(timeout_s)) == _native.FEEC_OK

    def stats(self) -> dict:
        a = ctypes.c_size_t(); p = ctypes.c_size_t(); i = ctypes.c_int(); q = ctypes.c_longlong()
        _native.check(self._lib.feec_server_stats(self._h, ctypes.byref(a), ctypes.byref(p), ctypes.byref(i),
                                                  ctypes.byref(q)), "feec_server_stats")
        return {"bytes_in_use": a.value, "peak_bytes": p.value, "inflight": i.value, "queued": q.value}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.feec_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
