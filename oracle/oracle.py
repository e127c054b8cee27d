"""ORACLE — test infrastructure, not product code.

ctypes binding of ``oracle/_build/libfeec_oracle.so`` (the plain-C restatement of the
reference's CSR Krylov path, ``oracle/feec_oracle.c``). Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (CPU-baseline and reference legs) import
this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfeec_oracle.so")
_lib = None

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(verbose: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, no FMA contraction)."""
    out = subprocess.run(["make", "-C", _HERE, "-s"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if verbose and out.stdout:
        print(out.stdout)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_csr_apply.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, ctypes.c_double]
        L.oracle_csr_diagonal.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p]
        L.oracle_rainbow.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p, _i32p, _i32p]
        L.oracle_rainbow.restype = ctypes.c_int
        L.oracle_cg.argtypes = [ctypes.c_int, _f64p, _f64p, _i32p, _i32p, _f64p, _f64p, ctypes.c_double, ctypes.c_int]
        L.oracle_cg_ssor.argtypes = L.oracle_cg.argtypes + [_f64p, ctypes.c_double]
        L.oracle_cg_rainbow.argtypes = L.oracle_cg_ssor.argtypes + [ctypes.c_int, _i32p, _i32p, _i32p]
        L.oracle_cg_ssor_eisenstat.argtypes = L.oracle_cg_ssor.argtypes
        L.oracle_cg_diag.argtypes = L.oracle_cg.argtypes + [_f64p]
        L.oracle_cg_eisenstat_rainbow.argtypes = L.oracle_cg_rainbow.argtypes
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def csr_apply(A, C, V, src, scaling=1.0):
    dest = np.empty(len(A) - 1)
    lib().oracle_csr_apply(len(A) - 1, A, C, V, np.ascontiguousarray(src, np.float64), dest, float(scaling))
    return dest


def csr_diagonal(A, C, V):
    d = np.empty(len(A) - 1)
    lib().oracle_csr_diagonal(len(A) - 1, A, C, V, d)
    return d


def rainbow(A, C):
    n = len(A) - 1
    F = np.empty(n, np.int32); B = np.empty(n + 1, np.int32); R = np.empty(n, np.int32)
    nc = lib().oracle_rainbow(n, A, C, F, B, R)
    if nc < 0:
        raise RuntimeError("oracle rainbow failed")
    return nc, F, B[: nc + 1].copy(), R


def cg(A, C, V, b, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3)
    return K, x, res


def cg_ssor(A, C, V, b, diag, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_ssor(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                             np.ascontiguousarray(diag, np.float64), float(omega))
    return K, x, res


def cg_rainbow(A, C, V, b, diag, rb, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    nc, F, B, R = rb
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_rainbow(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                                np.ascontiguousarray(diag, np.float64), float(omega), int(nc),
                                np.ascontiguousarray(F, np.int32), np.ascontiguousarray(B, np.int32),
                                np.ascontiguousarray(R, np.int32))
    return K, x, res


def cg_ssor_eisenstat(A, C, V, b, diag, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_ssor_eisenstat(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision),
                                       -3, np.ascontiguousarray(diag, np.float64), float(omega))
    return K, x, res


def cg_eisenstat_rainbow(A, C, V, b, diag, rb, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    nc, F, B, R = rb
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_eisenstat_rainbow(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision),
                                          -3, np.ascontiguousarray(diag, np.float64), float(omega), int(nc),
                                          np.ascontiguousarray(F, np.int32), np.ascontiguousarray(B, np.int32),
                                          np.ascontiguousarray(R, np.int32))
    return K, x, res


def cg_diag(A, C, V, b, precon, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_diag(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                             np.ascontiguousarray(precon, np.float64))
    return K, x, res
