"""Device-resident CSR systems (the ``feec_system_*`` part of the C ABI).

A ``System`` uploads a CSR matrix once, optionally prepares the multicolor or
index-order SSOR layout, and then solves with right-hand sides and iterates that
stay in device memory. Device buffers are torch tensors (used purely as device
allocations); every call runs on torch's current CUDA stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

METHODS = {"cg": _native.METHOD_CG, "ssor": _native.METHOD_SSOR, "rainbow": _native.METHOD_RAINBOW,
           "ssor_eisenstat": _native.METHOD_SSOR_EISENSTAT, "rainbow_eisenstat": _native.METHOD_RAINBOW_EISENSTAT,
           "diagonal": _native.METHOD_DIAGONAL}
MODES = {"reference": _native.MODE_REFERENCE, "fp64": _native.MODE_FP64, "mixed": _native.MODE_MIXED}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("simplefem_gb300.System needs a CUDA device")
    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _device_array(t, name, shape, dtypes=("float64",)):
    """Pointer to a contiguous CUDA tensor of the given shape and an accepted dtype; any
    other argument is a ValueError before the library sees it (a host or mis-sized buffer
    handed to a kernel as a device array would be read out of bounds)."""
    if not (hasattr(t, "is_cuda") and hasattr(t, "data_ptr")):
        raise ValueError(f"{name}: {type(t).__name__}, expected a CUDA tensor")
    dt = str(t.dtype).replace("torch.", "")
    if dt not in dtypes:
        raise ValueError(f"{name}: dtype {dt}, expected {' or '.join(dtypes)}")
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: shape {tuple(t.shape)}, expected {tuple(shape)}")
    if not t.is_contiguous():
        raise ValueError(f"{name}: not contiguous")
    if not t.is_cuda:
        raise ValueError(f"{name}: not a CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class System:
    def __init__(self, A, C, V):
        self._lib = _native.gpu()
        A = np.ascontiguousarray(A, np.int32)
        C = np.ascontiguousarray(C, np.int32)
        V = np.ascontiguousarray(V, np.float64)
        self.n = int(A.shape[0] - 1)
        self.nnz = int(C.shape[0])
        h = ctypes.c_void_p()
        st = self._lib.feec_system_create(ctypes.byref(h), self.n, A.ctypes.data_as(ctypes.c_void_p),
                                          C.ctypes.data_as(ctypes.c_void_p), V.ctypes.data_as(ctypes.c_void_p), 1,
                                          _stream())
        _native.check(st, "feec_system_create")
        self._h = h
        self.prepared = None

    def set_rainbow(self, diagonal, omega, num_colors, F, B, R):
        d = np.ascontiguousarray(diagonal, np.float64)
        F = np.ascontiguousarray(F, np.int32); B = np.ascontiguousarray(B, np.int32); R = np.ascontiguousarray(R, np.int32)
        st = self._lib.feec_system_set_rainbow(self._h, d.ctypes.data_as(ctypes.c_void_p), float(omega), int(num_colors),
                                               F.ctypes.data_as(ctypes.c_void_p), B.ctypes.data_as(ctypes.c_void_p),
                                               R.ctypes.data_as(ctypes.c_void_p), 1)
        _native.check(st, "feec_system_set_rainbow")
        self.prepared = "rainbow"

    def set_diagonal_precon(self, precon):
        """The diagonal preconditioner (z = precon * r) of method="diagonal"."""
        p = np.ascontiguousarray(precon, np.float64)
        st = self._lib.feec_system_set_diagonal_precon(self._h, p.ctypes.data_as(ctypes.c_void_p), 1)
        _native.check(st, "feec_system_set_diagonal_precon")

    def set_ssor(self, diagonal, omega):
        d = np.ascontiguousarray(diagonal, np.float64)
        st = self._lib.feec_system_set_ssor(self._h, d.ctypes.data_as(ctypes.c_void_p), float(omega), 1)
        _native.check(st, "feec_system_set_ssor")
        self.prepared = "ssor"

    def solve(self, b, x, method="rainbow", mode="reference", precision=1e-10, max_iter=0, residual=None,
              raise_on_error=True) -> dict:
        """Solve A x = b with device tensors b, x (float64, length n); x is the initial guess."""
        info = _native.FeecSolveInfo()
        xp, bp = _device_array(x, "x", (self.n,)), _device_array(b, "b", (self.n,))
        rp = None if residual is None else _device_array(residual, "residual", (self.n,))
        st = self._lib.feec_system_solve(self._h, METHODS[method], MODES[mode], xp, bp, rp,
                                         float(precision), int(max_iter), info, _stream())
        out = info.as_dict()
        out["status_name"] = _native.STATUS.get(st, str(st))
        if raise_on_error and st not in (_native.FEEC_OK, _native.FEEC_BREAKDOWN, _native.FEEC_SMALL_ENERGY,
                                         _native.FEEC_MAXITER):
            raise _native.FeecError(st, "feec_system_solve")
        return out

    def solve_batch(self, B, X, method="rainbow", mode="mixed", precision=1e-10, max_iter=0, rhs_per_team=0,
                    raise_on_error=True) -> list:
        """Solve A X[j] = B[j] for every row j of the (nrhs, n) float64 device tensors B, X
        (X holds the initial guesses) with the batched engine; one dict per column."""
        nrhs = int(B.shape[0])
        Bp, Xp = _device_array(B, "B", (nrhs, self.n)), _device_array(X, "X", (nrhs, self.n))
        infos = (_native.FeecSolveInfo * nrhs)()
        st = self._lib.feec_system_solve_batch(self._h, METHODS[method], MODES[mode], nrhs, Xp, Bp,
                                               float(precision), int(max_iter), int(rhs_per_team), infos, _stream())
        if raise_on_error and st not in (_native.FEEC_OK, _native.FEEC_MAXITER, _native.FEEC_BREAKDOWN):
            raise _native.FeecError(st, "feec_system_solve_batch")
        return [i.as_dict() for i in infos]

    def tune_batch(self, method="rainbow", mode="mixed", nrhs_hint=0) -> dict:
        """Run the batched-engine autotuner on this system; the choice is used by solve_batch
        calls with rhs_per_team=0."""
        k = ctypes.c_int(0); t = ctypes.c_int(0); c = ctypes.c_int(0); rate = ctypes.c_double(0.0)
        st = self._lib.feec_system_tune_batch(self._h, METHODS[method], MODES[mode], int(nrhs_hint), ctypes.byref(k),
                                              ctypes.byref(t), ctypes.byref(c), ctypes.byref(rate))
        _native.check(st, "feec_system_tune_batch")
        return {"rhs_per_team": k.value, "team_threads": t.value, "team_blocks": c.value, "rhs_iters_per_s": rate.value}

    def set_batch_config(self, method="rainbow", mode="mixed", rhs_per_team=0, team_threads=256, team_blocks=1):
        """Fix the batched launch configuration used by solve_batch(rhs_per_team=0): K right-hand
        sides per team, and either one-block teams of team_threads threads (team_blocks=1) or
        cluster teams of team_blocks blocks. rhs_per_team=0 returns to the automatic choice."""
        st = self._lib.feec_system_set_batch_config(self._h, METHODS[method], MODES[mode], int(rhs_per_team),
                                                    int(team_threads), int(team_blocks))
        _native.check(st, "feec_system_set_batch_config")

    def apply(self, x, y, scaling=1.0):
        """y = scaling * A x for device tensors (float64, or float32 on the FP32 values)."""
        dt = (str(getattr(x, "dtype", "")).replace("torch.", ""),)
        xp = _device_array(x, "x", (self.n,), ("float64", "float32"))
        yp = _device_array(y, "y", (self.n,), dt)
        if dt == ("float32",):
            st = self._lib.feec_system_apply_f32(self._h, xp, yp, float(scaling), _stream())
        else:
            st = self._lib.feec_system_apply(self._h, xp, yp, float(scaling), _stream())
        _native.check(st, "feec_system_apply")

    def set_launch(self, blocks=0, lanes=0):
        """Override the persistent grid size / lanes per row (0 = automatic)."""
        _native.check(self._lib.feec_system_set_launch(self._h, int(blocks), int(lanes)), "feec_system_set_launch")

    def memory_bytes(self) -> int:
        b = ctypes.c_size_t(0)
        _native.check(self._lib.feec_system_memory(self._h, ctypes.byref(b)), "feec_system_memory")
        return int(b.value)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.feec_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _system_vectors(systems, bs, xs):
    """Host arrays of system handles and of the x, b device pointers (one per system)."""
    n = len(systems)
    if n == 0 or len(bs) != n or len(xs) != n:
        raise ValueError(f"{n} systems, {len(bs)} right-hand sides, {len(xs)} solutions: expected one each")
    hs = (ctypes.c_void_p * n)(*[s._h for s in systems])
    xp = (ctypes.c_void_p * n)(*[_device_array(x, f"xs[{i}]", (s.n,)).value
                                  for i, (s, x) in enumerate(zip(systems, xs))])
    bp = (ctypes.c_void_p * n)(*[_device_array(b, f"bs[{i}]", (s.n,)).value
                                  for i, (s, b) in enumerate(zip(systems, bs))])
    return hs, xp, bp


def solve_many(systems, bs, xs, method="rainbow", mode="mixed", precision=1e-10, max_iter=0,
               raise_on_error=True) -> list:
    """One batched launch over many systems, one right-hand side each (device tensors)."""
    lib = _native.gpu()
    n = len(systems)
    hs, xp, bp = _system_vectors(systems, bs, xs)
    infos = (_native.FeecSolveInfo * n)()
    st = lib.feec_solve_many(n, hs, METHODS[method], MODES[mode], xp, bp, float(precision), int(max_iter), infos,
                             _stream())
    if raise_on_error and st not in (_native.FEEC_OK, _native.FEEC_MAXITER, _native.FEEC_BREAKDOWN):
        raise _native.FeecError(st, "feec_solve_many")
    return [i.as_dict() for i in infos]


class Batch:
    """Many systems, one right-hand side each, solved by one graph-captured batched launch.

    ``bs`` and ``xs`` are device tensors that stay bound to the batch: write new
    right-hand sides into ``bs`` and initial guesses into ``xs`` before each ``run``."""

    def __init__(self, systems, bs, xs, method="rainbow", mode="mixed", precision=1e-10, max_iter=0,
                 team_threads=0):
        self._lib = _native.gpu()
        n = len(systems)
        self.systems, self.bs, self.xs = systems, bs, xs
        hs, xp, bp = _system_vectors(systems, bs, xs)
        h = ctypes.c_void_p()
        st = self._lib.feec_batch_create(ctypes.byref(h), n, hs, METHODS[method], MODES[mode], xp, bp,
                                         float(precision), int(max_iter), int(team_threads), _stream())
        _native.check(st, "feec_batch_create")
        self._h = h
        self.n = n

    def run(self, raise_on_error=True) -> tuple:
        infos = (_native.FeecSolveInfo * self.n)()
        ms = ctypes.c_double(0.0)
        st = self._lib.feec_batch_run(self._h, infos, ctypes.byref(ms))
        if raise_on_error and st not in (_native.FEEC_OK, _native.FEEC_MAXITER, _native.FEEC_BREAKDOWN):
            raise _native.FeecError(st, "feec_batch_run")
        return [i.as_dict() for i in infos], ms.value

    def launch(self):
        """Enqueue a replay after the work on the current stream and return at once
        (the first half of ``run``); ``finish`` waits for it. ``bs`` and ``xs`` must not
        be touched in between."""
        _native.check(self._lib.feec_batch_launch(self._h), "feec_batch_launch")

    def finish(self, raise_on_error=True) -> tuple:
        """Wait for the replay ``launch`` enqueued; returns what ``run`` returns."""
        infos = (_native.FeecSolveInfo * self.n)()
        ms = ctypes.c_double(0.0)
        st = self._lib.feec_batch_finish(self._h, infos, ctypes.byref(ms))
        if raise_on_error and st not in (_native.FEEC_OK, _native.FEEC_MAXITER, _native.FEEC_BREAKDOWN):
            raise _native.FeecError(st, "feec_batch_finish")
        return [i.as_dict() for i in infos], ms.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.feec_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
