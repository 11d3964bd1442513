"""GPU parity at the benchmark problem sizes, through the C ABI, against the CPU oracle.

2D SIPG DGQ3 on 64 x 64 cells (65,536 DoFs), additive vertex patches of 8 x 8 DoFs, in both
SIPG penalty modes: the reference's (ip k(k+1)(1/h_l+1/h_r)/2 inside, 2 ip k(k+1)/h on the
boundary, apps/common_integrator.h:30-37) and 2(k+1)^2/h on every face.
  - smoother vmult at damping 0.5: FP64 relative max-norm error <= 1e-12, FP32 <= 2e-5
  - level operator: FP64 <= 1e-12
  - CG + V-cycle at damping 0.5: lambda_max(P A) of these patches is about 5.8, so damping 0.5
    gives smoothing factors |1 - 0.5 lambda| up to 1.9 and an indefinite V-cycle; the oracle
    and the GPU both stop without convergence, and their residual histories agree while CG
    still reduces the residual (first 4 iterations, relative 1e-8)
  - CG + V-cycle at the reference's damping 0.25 (TPSS.h:121-163): iteration counts identical
    to the oracle's, residual histories within 1e-6 relative plus 1e-9 ||r_0|| (the coarse CG
    stops at an absolute 1e-12, so the V-cycle is a slightly variable preconditioner and the
    last residuals of two FP64 implementations drift apart by ~1e-5 relative)
3D SIPG DGQ4 on 64^3 cells (32,768,000 DoFs), FP64, damping 0.15: CG + V-cycle iteration count
identical to the oracle's (tests/golden/mg_large.json, written by
tests/golden/make_golden.py --large, which takes minutes on the CPU).
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
DIM, K, NREP, NC = 2, 3, 2, 64
N2 = NC ** DIM * (K + 1) ** DIM


def philox(seed, n):
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, n)


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def large_cases():
    with open(os.path.join(GOLDEN, "mg_large.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("penalty", ["reference", "kp1sq"])
def test_dgq3_64sq_smoother_and_operator(tpss, oracle, cuda, penalty):
    import torch
    mode = tpss.Penalty.reference if penalty == "reference" else tpss.Penalty.kp1sq
    src = philox(0, N2)
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
        dim=DIM, degree=K, n_cells=(NC, NC), patch_variant=tpss.PatchVariant.vertex))
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    ref = oracle.schwarz_vmult(DIM, K, (NC, NC), src, patch_variant=1, omega=0.5, penalty=penalty)
    for precision, tol in ((tpss.Precision.fp64, 1e-12), (tpss.Precision.fp32, 2e-5)):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=0.5, precision=precision, penalty_mode=mode))
        d = torch.full_like(s, 7.0)
        p.vmult(d, s)
        torch.cuda.synchronize()
        assert rel_err(d.cpu().numpy(), ref) <= tol, (penalty, precision)
    op = tpss.LaplaceOperator(sh, 1.0, penalty_mode=mode)
    d = torch.empty_like(s)
    op.vmult(d, s)
    torch.cuda.synchronize()
    assert rel_err(d.cpu().numpy(), oracle.sipg_vmult(DIM, K, (NC, NC), src, penalty=penalty)) <= 1e-12
    # the two modes give different operators
    if penalty == "kp1sq":
        assert rel_err(d.cpu().numpy(), oracle.sipg_vmult(DIM, K, (NC, NC), src)) > 1e-3


def _solve_raw(tpss, mg, u, f, max_iter):
    """tpss_mg_cg_solve through the C ABI; returns (status, iterations, residual history)."""
    lib = tpss.load()
    hist = np.zeros(max_iter + 1)
    it = C.c_int(0)
    code = lib.tpss_mg_cg_solve(mg._h, C.c_void_p(u.data_ptr()), C.c_void_p(f.data_ptr()), 1e-8,
                                1e-14, max_iter, C.byref(it),
                                hist.ctypes.data_as(C.POINTER(C.c_double)), None)
    return code, it.value, hist


@pytest.mark.parametrize("penalty", ["reference", "kp1sq"])
def test_dgq3_64sq_damping_half_diverges_like_the_oracle(tpss, oracle, cuda, penalty):
    import torch
    mode = tpss.Penalty.reference if penalty == "reference" else tpss.Penalty.kp1sq
    f = philox(0, N2)
    it_ref, _, hist_ref = oracle.mg_cg_solve(DIM, K, NREP, NC, f, omega=0.5, rel_tol=1e-8,
                                             max_iter=40, penalty=penalty)
    assert it_ref == -1
    mg = tpss.MultigridSolver(DIM, K, NREP, NC, relaxation=0.5, coarse_solver=0,
                              penalty_mode=mode)
    u = torch.zeros(N2, dtype=torch.float64, device=cuda)
    ft = torch.tensor(f, dtype=torch.float64, device=cuda)
    torch.cuda.synchronize()
    code, it, hist = _solve_raw(tpss, mg, u, ft, 40)
    torch.cuda.synchronize()
    assert code == 6 and it == -1  # TPSS_ERR_NOT_CONVERGED
    np.testing.assert_allclose(hist[:5], hist_ref[:5], rtol=1e-8)


@pytest.mark.parametrize("penalty", ["reference", "kp1sq"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_dgq3_64sq_iterations_match_oracle(tpss, cuda, penalty, precision):
    import torch
    case = [c for c in large_cases() if c["dim"] == 2 and c["penalty"] == penalty][0]
    mode = tpss.Penalty.reference if penalty == "reference" else tpss.Penalty.kp1sq
    f = torch.tensor(philox(case["rhs_seed"], N2), dtype=torch.float64, device=cuda)
    prec = tpss.Precision.fp64 if precision == "fp64" else tpss.Precision.fp32
    for coarse_solver in (0, 1):
        mg = tpss.MultigridSolver(DIM, K, NREP, NC, relaxation=case["omega"], precision=prec,
                                  coarse_solver=coarse_solver, penalty_mode=mode)
        u = torch.zeros_like(f)
        it, hist = mg.solve(u, f, rel_tol=1e-8)
        ref = np.array(case["residual_history"])
        if precision == "fp64":
            assert it == case["iterations"], (penalty, coarse_solver)
            np.testing.assert_allclose(hist, ref, rtol=1e-6, atol=1e-9 * ref[0])
        else:
            # FP32 smoothers: the rounding of the preconditioner may cost one iteration
            assert abs(it - case["iterations"]) <= 1, (penalty, coarse_solver)


def test_dgq4_64cubed_fp64_iterations_match_oracle(tpss, cuda):
    """The headline problem: 3D DGQ4 64^3, FP64 smoothers, coarse CG (the oracle's solver) and
    the dense coarse solve the benchmark uses; both must give the oracle's iteration count.
    The residual histories agree to 1e-6 relative while the residual is above 1e-3 ||r_0||;
    further down the two FP64 implementations' histories drift apart (tens of percent around
    1e-5 ||r_0||) and meet again at the same stopping iteration. The drift is CG's own
    sensitivity, not a GPU difference: the oracle alone, given f perturbed by 1e-15 relative,
    drifts by 2-5 % below 1e-6 ||r_0|| (16^3 cells) and also stops at the same iteration."""
    import torch
    case = [c for c in large_cases() if c["dim"] == 3][0]
    n = case["n_cells_fine"]
    N = n ** 3 * (case["k"] + 1) ** 3
    f = torch.tensor(philox(case["rhs_seed"], N), dtype=torch.float64, device=cuda)
    ref = np.array(case["residual_history"])
    head = ref >= 1e-3 * ref[0]
    for coarse_solver in (0, 1):
        mg = tpss.MultigridSolver(3, case["k"], case["n_rep"], n, relaxation=case["omega"],
                                  precision=tpss.Precision.fp64, coarse_solver=coarse_solver)
        u = torch.zeros_like(f)
        it, hist = mg.solve(u, f, rel_tol=1e-8)
        assert it == case["iterations"], coarse_solver
        np.testing.assert_allclose(hist[head], ref[head], rtol=1e-6)
        del mg
