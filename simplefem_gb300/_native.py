"""Loads the package's native libraries with ctypes and declares their C ABI.

There is no Python or CPU fallback: if ``libfeec_gpu.so`` is missing, loading fails
with an error that says how to build it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_gpu = None
_workload = None


class FeecSolveInfo(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("iterations", ctypes.c_int),
        ("outer_iterations", ctypes.c_int),
        ("num_colors", ctypes.c_int),
        ("tolerance", ctypes.c_double),
        ("final_norm", ctypes.c_double),
        ("true_relres", ctypes.c_double),
        ("device_ms", ctypes.c_double),
        ("total_ms", ctypes.c_double),
        ("grid_blocks", ctypes.c_int),
        ("lanes_per_row", ctypes.c_int),
        ("fp64_fallback", ctypes.c_int),
        ("inner_fp64", ctypes.c_int),
        ("error_estimate", ctypes.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


STATUS = {0: "ok", 1: "breakdown", 2: "small_energy", 3: "maxiter", 4: "timeout", 5: "oom", 6: "badarg",
          7: "cuda_error", 8: "no_device"}
FEEC_OK, FEEC_BREAKDOWN, FEEC_SMALL_ENERGY, FEEC_MAXITER, FEEC_TIMEOUT, FEEC_OOM, FEEC_BADARG, FEEC_CUDA_ERROR, \
    FEEC_NO_DEVICE = range(9)
METHOD_CG, METHOD_SSOR, METHOD_RAINBOW, METHOD_SSOR_EISENSTAT, METHOD_RAINBOW_EISENSTAT, METHOD_DIAGONAL = 0, 1, 2, 3, 4, 5
MODE_REFERENCE, MODE_FP64, MODE_MIXED = 0, 1, 2


class FeecError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)} (status {status})")


_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_ip = ctypes.c_int
_dp = ctypes.c_double
_infop = ctypes.POINTER(FeecSolveInfo)


def _load(path):
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build the native libraries with "
                          "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)")
    return ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)


def gpu():
    """The CUDA library (libfeec_gpu.so) with its C ABI declared."""
    global _gpu
    if _gpu is None:
        L = _load(_build.lib_path("libfeec_gpu.so"))
        host = [_ip, _f64p, _f64p, _i32p, _i32p, _f64p, _f64p, _dp, _ip]
        L.feec_cg_csr.argtypes = host + [_infop]
        L.feec_cg_csr_ssor.argtypes = host + [_f64p, _dp, _infop]
        L.feec_cg_csr_rainbow.argtypes = host + [_f64p, _dp, _ip, _i32p, _i32p, _i32p, _infop]
        L.feec_cg_csr_ssor_eisenstat.argtypes = L.feec_cg_csr_ssor.argtypes
        L.feec_cg_csr_diagonal_precon.argtypes = host + [_f64p, _infop]
        L.feec_system_set_diagonal_precon.argtypes = [_vp, _vp, _ip]
        L.feec_cg_csr_eisenstat_rainbow.argtypes = L.feec_cg_csr_rainbow.argtypes
        L.feec_cr_csr.argtypes = host + [_infop]
        L.feec_cr_csr_textbook.argtypes = host + [_infop]
        L.feec_minres_csr.argtypes = host + [_infop]
        L.feec_chebyshev_diag.argtypes = host + [_f64p, _dp, _dp, _infop]
        hodge = [_ip, _ip, _f64p, _f64p] + [_i32p, _i32p, _f64p] * 4 + [_f64p, _dp, _ip, _dp, _ip, _infop]
        for name in ("feec_hodge_cr_csr", "feec_hodge_cr_csr_diagonal", "feec_hodge_cr_csr_ssor",
                     "feec_hodge_cr_csr_textbook"):
            getattr(L, name).argtypes = hodge
        _ip32 = ctypes.POINTER(ctypes.c_int); _dp64 = ctypes.POINTER(ctypes.c_double)
        L.feec_hodge_herzog_soodhalter.argtypes = ([_ip, _ip, _f64p, _f64p, _f64p, _f64p] + [_i32p, _i32p, _f64p] * 4
                                                   + [_dp, _ip] + [_ip32, _ip32, _dp64] * 2 + [_dp, _ip, _infop])
        L.feec_csr_apply.argtypes = [_ip, _ip, _i32p, _i32p, _f64p, _f64p, _f64p, _dp]
        L.feec_csr_diagonal.argtypes = [_ip, _i32p, _i32p, _f64p, _f64p]
        _cp = ctypes.POINTER(ctypes.c_int)
        L.feec_csr_add.argtypes = [_ip, _ip, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _dp, _dp, _i32p, _i32p, _f64p, _cp]
        L.feec_csr_multiply_size.argtypes = [_ip, _ip, _i32p, _i32p, _i32p, ctypes.POINTER(ctypes.c_longlong)]
        L.feec_csr_multiply.argtypes = [_ip, _ip, _ip, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _cp]
        L.feec_csr_transpose.argtypes = [_ip, _ip, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _cp]
        L.feec_coo_to_csr.argtypes = [_ip, _ip, ctypes.c_longlong, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _cp]
        _llp = ctypes.POINTER(ctypes.c_longlong)
        L.feec_coo_multiply_size.argtypes = [_ip, ctypes.c_longlong, _i32p, ctypes.c_longlong, _i32p, _llp]
        L.feec_coo_multiply.argtypes = [_ip, _ip, _ip, ctypes.c_longlong, _i32p, _i32p, _f64p, ctypes.c_longlong,
                                        _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _llp]
        L.feec_rainbow.argtypes = [_ip, _i32p, _i32p, ctypes.POINTER(ctypes.c_int), _i32p, _i32p, _i32p]
        L.feec_csr_check.argtypes = [_ip, _ip, _i32p, _i32p, _f64p]
        L.feec_system_create.argtypes = [ctypes.POINTER(_vp), _ip, _vp, _vp, _vp, _ip, _vp]
        L.feec_system_set_rainbow.argtypes = [_vp, _vp, _dp, _ip, _vp, _vp, _vp, _ip]
        L.feec_system_set_ssor.argtypes = [_vp, _vp, _dp, _ip]
        L.feec_system_solve.argtypes = [_vp, _ip, _ip, _vp, _vp, _vp, _dp, _ip, _infop, _vp]
        L.feec_system_apply.argtypes = [_vp, _vp, _vp, _dp, _vp]
        L.feec_system_apply_f32.argtypes = [_vp, _vp, _vp, ctypes.c_float, _vp]
        L.feec_system_solve_batch.argtypes = [_vp, _ip, _ip, _ip, _vp, _vp, _dp, _ip, _ip, _infop, _vp]
        L.feec_solve_many.argtypes = [_ip, ctypes.POINTER(_vp), _ip, _ip, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                      _dp, _ip, _infop, _vp]
        L.feec_system_tune_batch.argtypes = [_vp, _ip, _ip, _ip, ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_double)]
        L.feec_system_set_batch_config.argtypes = [_vp, _ip, _ip, _ip, _ip, _ip]
        L.feec_batch_create.argtypes = [ctypes.POINTER(_vp), _ip, ctypes.POINTER(_vp), _ip, _ip, ctypes.POINTER(_vp),
                                         ctypes.POINTER(_vp), _dp, _ip, _ip, _vp]
        L.feec_batch_run.argtypes = [_vp, _infop, ctypes.POINTER(ctypes.c_double)]
        L.feec_batch_launch.argtypes = [_vp]
        L.feec_batch_finish.argtypes = [_vp, _infop, ctypes.POINTER(ctypes.c_double)]
        L.feec_batch_destroy.argtypes = [_vp]
        L.feec_system_set_launch.argtypes = [_vp, _ip, _ip]
        L.feec_system_memory.argtypes = [_vp, ctypes.POINTER(ctypes.c_size_t)]
        L.feec_system_destroy.argtypes = [_vp]
        L.feec_kernel_launches.restype = ctypes.c_ulonglong
        L.feec_selftest_wait_timeout.argtypes = [_dp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                 ctypes.POINTER(ctypes.c_double)]
        L.feec_status_string.restype = ctypes.c_char_p
        L.feec_status_string.argtypes = [_ip]
        _gpu = L
    return _gpu


def workload():
    """Host-only synthetic workload library (libfeec_workload.so)."""
    global _workload
    if _workload is None:
        L = _load(_build.lib_path("libfeec_workload.so"))
        L.feec_lattice_size.argtypes = [_ip, _ip, _ip, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
        L.feec_lattice_assemble.argtypes = [_ip, _ip, _ip, ctypes.c_uint64, _i32p, _i32p, _f64p]
        L.feec_lattice_positions.argtypes = [_ip, _ip, _ip, _f64p]
        L.feec_uniform_vector.argtypes = [ctypes.c_uint64, ctypes.c_int64, _dp, _dp, _f64p]
        L.feec_uniform_vector.restype = None
        _workload = L
    return _workload


def check(status, where):
    if status != FEEC_OK:
        raise FeecError(status, where)
