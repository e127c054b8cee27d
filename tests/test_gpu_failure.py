"""Failure detection without a GPU fault. Every device-side wait of the solvers is
bounded: a wait that is never satisfied gives up after its limit, records FEEC_TIMEOUT
and the wait site, and every thread leaves, so the host reads an error status and the
GPU context stays usable. Here a kernel waits, through the same bounded wait as the
solvers' grid barrier, on a counter that nothing ever writes (limit 0.25 s); a solve run
right afterwards must still succeed."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_unsatisfied_wait_times_out_and_context_survives(cuda):
    import simplefem_gb300 as S
    from simplefem_gb300 import _native
    lib = _native.gpu()
    st, site, ms = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_double(0.0)
    rc = lib.feec_selftest_wait_timeout(0.25, ctypes.byref(st), ctypes.byref(site), ctypes.byref(ms))
    assert rc == _native.FEEC_OK
    assert st.value == 4                      # FEEC_TIMEOUT recorded by the kernel
    assert site.value == 77                   # the wait site of the self-test kernel
    assert 250.0 <= ms.value < 5000.0, ms.value
    # the context is still usable: a drop-in solve right after gives the reference's answer
    g = load_golden("fem2d_p1_l6")
    n = len(g["A"]) - 1
    x = np.zeros(n); res = np.array(g["b"])
    K = S.ConjugateGradientSolverCSR(n, x, g["b"], g["A"], g["C"], g["V"], res, float(g["precision"]), -3)
    K_ref = int(g["cg_K"])
    assert abs(K - K_ref) <= max(1, int(np.ceil(0.02 * K_ref)))
    assert np.linalg.norm(x - g["cg_x"]) <= 1e-9 * np.linalg.norm(g["cg_x"])


def test_selftest_rejects_bad_limits(cuda):
    from simplefem_gb300 import _native
    lib = _native.gpu()
    st, site, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    for bad in (0.0, -1.0, 11.0):
        assert lib.feec_selftest_wait_timeout(bad, ctypes.byref(st), ctypes.byref(site), ctypes.byref(ms)) == 6
