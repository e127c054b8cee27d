"""Synthetic workloads with the shapes of the benchmark configurations.

``lattice_matrix(dim, r, L, coef_seed)`` assembles the Lagrange P_r stiffness plus
(coefficient) mass operator on the unit square / cube refined L times — the same
operator the reference's FEEC route builds (tests/solverfem/csrsolver_stiff.cpp:209-243),
numbered lexicographically on the degree-of-freedom lattice (see csrc/lattice_fem.cpp).
``uniform_vector(seed, n)`` draws U[-1, 1) from SplitMix64, reproducible on any host.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


def lattice_size(dim: int, r: int, L: int):
    n = ctypes.c_int64(); nnz = ctypes.c_int64()
    st = _native.workload().feec_lattice_size(dim, r, L, ctypes.byref(n), ctypes.byref(nnz))
    if st != 0:
        raise ValueError(f"unsupported lattice dim={dim} r={r} L={L}")
    return int(n.value), int(nnz.value)


def lattice_matrix(dim: int, r: int, L: int, coef_seed: int = 0):
    """(A, C, V) int32/int32/float64 CSR arrays of the P_r stiffness + mass operator."""
    n, nnz = lattice_size(dim, r, L)
    if nnz >= 2**31:
        raise ValueError("operator too large for int32 CSR")
    A = np.empty(n + 1, np.int32); C = np.empty(nnz, np.int32); V = np.empty(nnz, np.float64)
    st = _native.workload().feec_lattice_assemble(dim, r, L, ctypes.c_uint64(coef_seed), A, C, V)
    if st != 0:
        raise RuntimeError("lattice assembly failed")
    return A, C, V


def lattice_positions(dim: int, r: int, L: int) -> np.ndarray:
    n, _ = lattice_size(dim, r, L)
    pos = np.empty(n * dim, np.float64)
    _native.workload().feec_lattice_positions(dim, r, L, pos)
    return pos.reshape(n, dim)


def uniform_vector(seed: int, n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    out = np.empty(n, np.float64)
    _native.workload().feec_uniform_vector(ctypes.c_uint64(seed), n, lo, hi, out)
    return out


# The benchmark configurations (sizes follow the reference's uniform refinement).
CONFIGS = {
    "cfg1_2d_p1_l6": dict(dim=2, r=1, L=6),     # plain CG, N = 4,225
    "cfg2_3d_p2_l5": dict(dim=3, r=2, L=5),     # Rainbow SSOR-PCG, N = 274,625
    "cfg3_3d_p1_l6": dict(dim=3, r=1, L=6),     # mixed-precision inner sizing, N = 274,625
    "cfg3_3d_p1_l7": dict(dim=3, r=1, L=7),     # mixed-precision target, N = 2,146,689
    "cfg4_2d_p2_l7": dict(dim=2, r=2, L=7),     # largest batched system, N = 66,049
}


def lattice_choices(n_min=1000, n_max=2_000_000, dims=(2, 3), degrees=(1, 2, 3)):
    """All (dim, r, L) whose unknown count (r 2^L + 1)^d lies in [n_min, n_max]."""
    out = []
    for d in dims:
        for r in degrees:
            for L in range(0, 13):
                n = (r * 2 ** L + 1) ** d
                if n > n_max:
                    break
                if n >= n_min:
                    out.append((n, d, r, L))
    return sorted(out)


def serving_requests(count, seed, rate_per_s=200.0, n_min=1000, n_max=2_000_000, tolerances=(1e-8, 1e-10, 1e-12)):
    """A seeded Poisson-arrival request stream: 2D or 3D (50/50), P1-P3, the refinement whose
    unknown count is nearest (in log) to a log-uniform draw in [n_min, n_max], a per-request
    coefficient seed, and a tolerance drawn from `tolerances`."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    choices = {d: [c for c in lattice_choices(n_min, n_max, dims=(d,))] for d in (2, 3)}
    for i in range(count):
        t += rng.exponential(1.0 / rate_per_s)
        d = 2 if rng.random() < 0.5 else 3
        target = np.exp(rng.uniform(np.log(n_min), np.log(n_max)))
        cands = choices[d]
        n, dd, r, L = min(cands, key=lambda c: abs(np.log(c[0]) - np.log(target)))
        reqs.append(dict(t=t, dim=dd, r=r, L=L, n=n, coef_seed=1 + int(rng.integers(0, 2)),
                         rhs_seed=int(rng.integers(1, 2**62)), tol=float(rng.choice(tolerances))))
    return reqs


def batched_uneven_systems(count, seed):
    """The uneven batch: 2D P1 or P2 (50/50), refinement uniform in 3..7, a per-system
    coefficient seed (log-uniform [0.1, 10] cell coefficients on the mass term)."""
    rng = np.random.default_rng(seed)
    return [dict(dim=2, r=int(rng.integers(1, 3)), L=int(rng.integers(3, 8)), coef_seed=1 + i) for i in range(count)]
