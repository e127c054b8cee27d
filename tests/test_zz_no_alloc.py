"""The allocation-free CG entry point (feec_cg_csr_noalloc).

Callers that cannot allocate device memory during a solve (a fixed, pre-reserved
memory budget, or code where a cudaMalloc is not allowed) pass their own device
buffers; the solver's scratch is a fixed array inside the library. These tests call
it through the C ABI twice in a row and compare each result with the existing
drop-in entry point (feec_cg_csr) at the parity tolerance of the other GPU tests:
iteration count within 2% (at least +-1), solution within 1e-9 relative.
This file is collected last so that a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _entry():
    from simplefem_gb300 import _native
    f = _native.gpu().feec_cg_csr_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_int,
                  ctypes.POINTER(_native.FeecSolveInfo), vp]
    f.restype = ctypes.c_int
    return f


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("name", ["fem2d_p1_l6", "fem3d_p2_l3", "lap5_n32"])
def test_noalloc_cg_matches_dropin_twice(cuda, name):
    torch = cuda
    import simplefem_gb300 as S
    from simplefem_gb300 import _native
    g = load_golden(name)
    n = len(g["A"]) - 1
    prec = float(g["precision"])
    x_ref = np.zeros(n); r_ref = np.array(g["b"])
    K_ref = S.ConjugateGradientSolverCSR(n, x_ref, g["b"], g["A"], g["C"], g["V"], r_ref, prec, -3)
    f = _entry()
    dA = torch.from_numpy(np.ascontiguousarray(g["A"], np.int32)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(g["C"], np.int32)).cuda()
    dV = torch.from_numpy(np.ascontiguousarray(g["V"], np.float64)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(g["b"], np.float64)).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        dx = torch.zeros(n, dtype=torch.float64, device="cuda")
        dr = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = _native.FeecSolveInfo()
        st = f(n, _p(dx), _p(db), _p(dA), _p(dC), _p(dV), _p(dr), prec, 0, ctypes.byref(info), stream)
        torch.cuda.synchronize()
        assert st == 0, (call, st)
        K = info.iterations
        assert abs(K - K_ref) <= max(1, int(np.ceil(0.02 * K_ref))), (call, K, K_ref)
        x = dx.cpu().numpy()
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= 1e-9, call
        r = dr.cpu().numpy()
        assert np.linalg.norm(r - r_ref) <= 1e-6 * np.linalg.norm(g["b"]) + 1e-12, call


def test_noalloc_rejects_more_rows_than_its_scratch(cuda):
    torch = cuda
    from simplefem_gb300 import _native
    f = _entry()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    info = _native.FeecSolveInfo()
    n = (1 << 20) + 1
    st = f(n, _p(buf), _p(buf), _p(buf), _p(buf), _p(buf), _p(buf), 1e-10, 0, ctypes.byref(info),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _native.FEEC_BADARG
