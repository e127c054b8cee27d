"""Mixed precision (FP32 inner solves inside FP64 defect correction) at the sizes of the
benchmark configurations: every result must reach the requested FP64 relative residual
1e-10 AND be within 1e-9 (relative, 2-norm) of a tight FP64 oracle solve.

The tight oracle is the oracle's restatement of the reference's Rainbow SSOR-PCG
(solver/sparsesolver.cpp:1002-1335) run on the scaled system A (s x) = s b, with s so
large that the reference's absolute floor of 2^-26 (base/base.hpp:127-128) does not
bind, to a relative precision of 1e-13; dividing by s gives x. Its own error is about
1e-12 on these operators, far below the 1e-9 bar.

Cases (the configurations' operators):
* 3D P1 refined 6 times (N = 274,625), the inner sizing operator of the mixed
  configuration: single solves on the whole GPU (Rainbow and plain CG) and a batch;
* a sample of the 512 uneven systems of the batched configuration (2D P1/P2 refined
  3-7 times, coefficient mass), solved together in one batched launch;
* 2D P2 refined 7 times with coefficient mass (N = 66,049): 64 right-hand sides in
  one blocked batch, a sample of the columns checked.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_BAR = 1e-9
PRECISION = 1e-10


def _tight(A, C, V, b, diag, rb):
    from oracle import oracle
    bn = float(np.linalg.norm(b))
    s = max(1.0, 10.0 * 2.0 ** -26 / (1e-13 * bn))
    oracle.set_threads(oracle.max_threads())
    _, x, _ = oracle.cg_rainbow(A, C, V, s * np.asarray(b), diag, rb, 1.0, precision=1e-13)
    return x / s


def _system(dim, r, L, coef_seed=0):
    import simplefem_gb300 as S
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import System
    A, C, V = workloads.lattice_matrix(dim, r, L, coef_seed)
    n = len(A) - 1
    mat = S.MatrixCSR(n, n, A, C, V)
    rb = S.Rainbow(mat)
    diag = mat.getDiagonal().raw()
    sysm = System(A, C, V)
    sysm.set_rainbow(diag, 1.0, rb.num_colors, rb.F, rb.B, rb.R)
    return sysm, (A, C, V, diag, (rb.num_colors, rb.F, rb.B, rb.R))


def _check(x, b, ops, info, what):
    import scipy.sparse as sp
    A, C, V, diag, rb = ops
    n = len(A) - 1
    M = sp.csr_matrix((V, C, A), shape=(n, n))
    relres = np.linalg.norm(b - M @ x) / np.linalg.norm(b)
    assert info["status"] == 0 and relres <= PRECISION, (what, info, relres)
    xt = _tight(A, C, V, b, diag, rb)
    err = np.linalg.norm(x - xt) / np.linalg.norm(xt)
    assert err <= ERR_BAR, (what, err, info)
    return err


@pytest.mark.parametrize("method", ["rainbow", "cg"])
def test_mixed_single_solve_3d_p1_l6_meets_error_bar(cuda, method):
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, ops = _system(3, 1, 6)
    n = sysm.n
    b = workloads.uniform_vector(77, n)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = sysm.solve(torch.from_numpy(b).cuda(), x, method=method, mode="mixed", precision=PRECISION)
    assert info["fp64_fallback"] == 0
    err = _check(x.cpu().numpy(), b, ops, info, method)
    # the solver reports the error bound its stop rule enforced (the oracle checks the real error)
    assert info["error_estimate"] > 0.0, info
    assert err <= 10.0 * max(info["error_estimate"], 1e-12), (err, info["error_estimate"])
    sysm.close()


def test_mixed_batch_3d_p1_l6_meets_error_bar(cuda):
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, ops = _system(3, 1, 6)
    n = sysm.n
    nrhs = 8
    Bh = np.stack([workloads.uniform_vector(300 + j, n) for j in range(nrhs)])
    X = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    infos = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X, method="rainbow", mode="mixed", precision=PRECISION)
    Xh = X.cpu().numpy()
    for j in (0, 5):
        _check(Xh[j], Bh[j], ops, infos[j], ("batch column", j))
    for j in range(nrhs):
        assert infos[j]["error_estimate"] > 0.0, (j, infos[j])
    sysm.close()


def test_mixed_uneven_sample_meets_error_bar(cuda):
    torch = cuda
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import solve_many
    specs = workloads.batched_uneven_systems(512, 4242)
    # every refinement level and both degrees of the configuration, largest systems included
    pick, seen = [], set()
    for i, sp_ in enumerate(specs):
        key = (sp_["r"], sp_["L"])
        if key not in seen:
            seen.add(key)
            pick.append(i)
    systems, opss, bs, xs, bh = [], [], [], [], []
    for i in pick:
        sysm, ops = _system(**specs[i])
        b = workloads.uniform_vector(77 + i, sysm.n)
        systems.append(sysm); opss.append(ops); bh.append(b)
        bs.append(torch.from_numpy(b).cuda())
        xs.append(torch.zeros(sysm.n, dtype=torch.float64, device="cuda"))
    infos = solve_many(systems, bs, xs, method="rainbow", mode="mixed", precision=PRECISION)
    for k, i in enumerate(pick):
        _check(xs[k].cpu().numpy(), bh[k], opss[k], infos[k], ("uneven system", i, specs[i]))
    for s in systems:
        s.close()


def test_mixed_block_64_rhs_2d_p2_l7_meets_error_bar(cuda):
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, ops = _system(2, 2, 7, 1)
    n = sysm.n
    nrhs = 64
    Bh = np.stack([workloads.uniform_vector(4000 + j, n) for j in range(nrhs)])
    X = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    infos = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X, method="rainbow", mode="mixed", precision=PRECISION)
    Xh = X.cpu().numpy()
    for j in (0, 31, 63):
        _check(Xh[j], Bh[j], ops, infos[j], ("block column", j))
    sysm.close()


def test_mixed_kept_directions_stay_bounded_on_ill_conditioned_operator(cuda):
    """2D P1 refined 10 times (N = 1,050,625; condition number x FP32 roundoff near 1e-2) at a
    request of 1e-12 on one block per SM: kept-direction FP32 segments slow down without bound
    here (one such solve took 426,392 iterations), so each gets a bounded share of the
    restarted rate and the solve restarts once one runs out. The whole mixed solve must stay
    within 5x the FP64 solve's iterations (it takes about 3x) and meet the residual and error
    bars."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, ops = _system(2, 1, 10, 1)
    n = sysm.n
    b = workloads.uniform_vector(1429455515942280814, n)
    bd = torch.from_numpy(b).cuda()
    sysm.set_launch(torch.cuda.get_device_properties(0).multi_processor_count, 0)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = sysm.solve(bd, x, method="rainbow", mode="mixed", precision=1e-12, max_iter=50000)   # bounds the test's time
    sysm.set_launch(0, 0)
    x64 = torch.zeros(n, dtype=torch.float64, device="cuda")
    info64 = sysm.solve(bd, x64, method="rainbow", mode="fp64", precision=1e-12)
    assert info["status"] == 0 and info["true_relres"] <= 1e-12, info
    assert info["iterations"] <= 5 * info64["iterations"], (info["iterations"], info64["iterations"])
    # the FP64 solve at 1e-12 is within about 3e-11 of the solution (amplification ~30)
    err = float(torch.linalg.norm(x - x64) / torch.linalg.norm(x64))
    assert err <= ERR_BAR, (err, info)
    sysm.close()


def test_mixed_whole_gpu_solves_measure_both_inner_precisions(cuda):
    """On the whole GPU, a system's first mixed solve runs FP32 inner iterations and its
    second FP64 ones; later solves keep the faster per decade of residual fall and report it
    in inner_fp64. Every one of them meets the residual bar and the error bar against the
    tight oracle, and reports an error estimate."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, ops = _system(3, 1, 5)
    n = sysm.n
    infos = []
    for k in range(3):
        b = workloads.uniform_vector(500 + k, n)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = sysm.solve(torch.from_numpy(b).cuda(), x, method="rainbow", mode="mixed", precision=PRECISION)
        _check(x.cpu().numpy(), b, ops, info, ("solve", k))
        assert info["error_estimate"] > 0.0, info
        infos.append(info)
    assert [i["inner_fp64"] for i in infos[:2]] == [0, 1], infos
    assert infos[2]["inner_fp64"] in (0, 1)
    assert infos[1]["fp64_fallback"] == 0
    sysm.close()
