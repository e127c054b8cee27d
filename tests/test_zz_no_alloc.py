"""The allocation-free CG entry point (feec_cg_csr_noalloc).

Callers that cannot allocate device memory during a solve (a fixed, pre-reserved
memory budget, or code where a cudaMalloc is not allowed) pass their own device
buffers; the solver's scratch is a fixed array inside the library. These tests call
it through the C ABI twice in a row and compare each result with the reference's own
plain CG output stored in the golden fixture (cg_K, cg_x), at the parity tolerance of
the other drop-in tests: iteration count within 2% (at least +-1), and the solution as
close to the reference's as the reference's own solution is to the exact one (never
looser than 1e-9 relative). The second call must leave the device's free memory
unchanged: the entry point allocates nothing.
This file is collected last so that a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

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
def test_noalloc_cg_matches_reference_twice(cuda, name):
    torch = cuda
    from simplefem_gb300 import _native
    g = load_golden(name)
    n = len(g["A"]) - 1
    prec = float(g["precision"])
    K_ref = int(g["cg_K"])
    x_ref = g["cg_x"]
    M = sp.csr_matrix((g["V"], g["C"], g["A"]), shape=(n, n))
    xs = sla.spsolve(M.tocsc(), g["b"])
    own_err = np.linalg.norm(x_ref - xs) / np.linalg.norm(xs)
    f = _entry()
    dA = torch.from_numpy(np.ascontiguousarray(g["A"], np.int32)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(g["C"], np.int32)).cuda()
    dV = torch.from_numpy(np.ascontiguousarray(g["V"], np.float64)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(g["b"], np.float64)).cuda()
    dx = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(2)]
    dr = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(2)]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    free = []
    for call in range(2):
        free.append(torch.cuda.mem_get_info()[0])
        info = _native.FeecSolveInfo()
        st = f(n, _p(dx[call]), _p(db), _p(dA), _p(dC), _p(dV), _p(dr[call]), prec, 0, ctypes.byref(info), stream)
        torch.cuda.synchronize()
        assert st == 0 and info.status == 0, (call, st, info.status)
        K = info.iterations
        assert abs(K - K_ref) <= max(1, int(np.ceil(0.02 * K_ref))), (call, K, K_ref)
        x = dx[call].cpu().numpy()
        diff = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert diff <= max(1e-9, 2.0 * own_err), (call, diff, own_err)
        # the residual array is the recursive residual; it must describe x
        r = dr[call].cpu().numpy()
        assert np.linalg.norm(r - (g["b"] - M @ x)) <= 1e-6 * np.linalg.norm(g["b"]) + 1e-12, call
    # the first call may load kernels; the second allocates nothing at all
    assert torch.cuda.mem_get_info()[0] == free[1]


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
    assert info.status == _native.FEEC_BADARG


def test_noalloc_bad_arguments_report_their_status(cuda):
    torch = cuda
    from simplefem_gb300 import _native
    f = _entry()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    info = _native.FeecSolveInfo()
    st = f(4, _p(buf), _p(buf), _p(buf), _p(buf), _p(buf), _p(buf), -1.0, 0, ctypes.byref(info),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _native.FEEC_BADARG
    assert info.status == _native.FEEC_BADARG
