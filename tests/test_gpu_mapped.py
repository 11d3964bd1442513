"""GPU parity on distorted (multilinear) meshes against the numpy quadrature oracle.

Tolerances: operator 1e-12 relative max-norm (FP64 assembly and product); CG + V-cycle with
surrogate-patch smoothers: identical iteration counts, solution 1e-8 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def philox(seed, n):
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, n)


@pytest.fixture(scope="module")
def mapped():
    from oracle import np_distorted
    return np_distorted


def _op(tpss, dim, k, nc, X, ip=1.0):
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1,
                                              vertex_coords=X)
    sh = tpss.SubdomainHandler(ad)
    return sh, tpss.LaplaceOperator(sh, ip)


@pytest.mark.parametrize("dim,k,nc,seed,amp", [
    (2, 1, (5, 4), 1, 0.25), (2, 3, (4, 5), 2, 0.25), (2, 7, (3, 2), 3, 0.2),
    (3, 1, (3, 4, 2), 4, 0.25), (3, 2, (3, 3, 3), 5, 0.25), (3, 3, (2, 3, 2), 6, 0.25),
    (3, 4, (2, 2, 3), 7, 0.15)])
def test_mapped_operator_vs_quadrature(tpss, oracle, mapped, cuda, dim, k, nc, seed, amp):
    import torch
    X = oracle.distorted_coords(dim, list(nc), seed, amp)
    ip = 1.3
    A = mapped.sipg_matrix_mapped(dim, k, list(nc), X, ip)
    N = A.shape[0]
    x = philox(seed, N)
    sh, op = _op(tpss, dim, k, nc, X, ip)
    src = torch.tensor(x, dtype=torch.float64, device=cuda)
    dst = torch.full_like(src, 7.0)
    op.vmult(dst, src)
    torch.cuda.synchronize()
    assert rel_err(dst.cpu().numpy(), A @ x) <= 1e-12


@pytest.mark.parametrize("dim,k,nc,seed", [(2, 3, (5, 4), 12), (3, 2, (3, 4, 3), 13)])
def test_mapped_operator_permuted_cells(tpss, oracle, mapped, cuda, dim, k, nc, seed):
    """Distorted level with a permuted cell numbering (cell_dof_start): the product with the
    matrix-free face couplings addresses cells and neighbours through the permutation."""
    import torch
    X = oracle.distorted_coords(dim, list(nc), seed, 0.2)
    A = mapped.sipg_matrix_mapped(dim, k, list(nc), X, 1.0)
    ncell, nd = int(np.prod(nc)), (k + 1) ** dim
    cs = np.random.default_rng(seed).permutation(ncell) * nd
    xp = philox(seed, ncell * nd)
    idx = (cs[:, None] + np.arange(nd)[None, :]).reshape(-1)  # lexicographic DoF -> permuted DoF
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1,
                                              vertex_coords=X, cell_dof_start=cs)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh)
    src = torch.tensor(xp, dtype=torch.float64, device=cuda)
    dst = torch.full_like(src, float("nan"))
    op.vmult(dst, src)
    ref = np.empty_like(xp)
    ref[idx] = A @ xp[idx]
    assert rel_err(dst.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("dim,k,nc,seed,amp", [(2, 3, (4, 5), 2, 0.25), (3, 3, (3, 3, 2), 6, 0.25)])
def test_mapped_operator_fp32(tpss, oracle, mapped, cuda, dim, k, nc, seed, amp):
    """The single-precision product on a distorted level (FP32 copy of the block-sparse matrix)
    against the quadrature matrix: FP32 rounding only (1e-5 relative), and the residual form
    dst = rhs - A src through the single-precision V-cycle is covered by the MG tests."""
    import torch
    X = oracle.distorted_coords(dim, list(nc), seed, amp)
    A = mapped.sipg_matrix_mapped(dim, k, list(nc), X, 1.0)
    x = philox(seed + 10, A.shape[0])
    sh, op = _op(tpss, dim, k, nc, X)
    src = torch.tensor(x, dtype=torch.float64, device=cuda)
    dst = torch.full_like(src, float("nan"))
    op.vmult_fp32(dst, src)
    err = rel_err(dst.cpu().numpy(), A @ x)
    assert 0.0 < err <= 1e-5, err


@pytest.mark.parametrize("dim,k,nc", [(2, 3, (6, 5)), (3, 2, (4, 3, 3))])
def test_mapped_operator_on_cartesian_coords_equals_tensor_operator(tpss, mapped, cuda, dim, k, nc):
    import torch
    X = mapped.cartesian_coords(dim, list(nc))
    _, opm = _op(tpss, dim, k, nc, X)
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc))
    opc = tpss.LaplaceOperator(sh)
    N = sh.n_dofs()
    src = torch.tensor(philox(3, N), dtype=torch.float64, device=cuda)
    a, b = torch.empty_like(src), torch.empty_like(src)
    opm.vmult(a, src)
    opc.vmult(b, src)
    assert rel_err(a.cpu().numpy(), b.cpu().numpy()) <= 1e-12


# amplitude 0.15 for the surrogate smoother: at 0.25 its damped additive sweep is no longer a
# contraction on some patches and CG iteration counts become sensitive to rounding
@pytest.mark.parametrize("dim,k,n_rep,ncf,seed,amp,local", [
    (2, 2, 2, 16, 5, 0.15, "surrogate"), (2, 3, 2, 8, 6, 0.15, "surrogate"),
    (3, 1, 2, 8, 7, 0.15, "surrogate"), (2, 2, 2, 16, 5, 0.25, "ksum"),
    (2, 2, 2, 16, 5, 0.25, "exact"), (3, 1, 2, 8, 7, 0.2, "ksum"), (3, 1, 2, 8, 7, 0.2, "exact")])
def test_mg_cg_on_distorted_mesh(tpss, oracle, mapped, cuda, dim, k, n_rep, ncf, seed, amp, local):
    """CG + V-cycle on a distorted hierarchy: mapped operators on every level, Schwarz
    smoothers with surrogate / Kronecker-sum / exact local solvers, dense coarse solve;
    identical iterations to the numpy oracle."""
    import torch
    X = oracle.distorted_coords(dim, [ncf] * dim, seed, amp)
    N = ncf ** dim * (k + 1) ** dim
    f = philox(seed, N)
    om = oracle.lookup_damping_factor(1, 0, dim)
    it_ref, hist_ref, u_ref = mapped.mg_cg_solve_mapped(dim, k, n_rep, ncf, X, f, om, local=local)
    ls = {"surrogate": tpss.LocalSolver.fd, "ksum": tpss.LocalSolver.ksum, "exact": tpss.LocalSolver.exact}[local]
    mg = tpss.MultigridSolver(dim, k, n_rep, ncf, relaxation=om, coarse_solver=1, vertex_coords=X,
                              local_solver=ls)
    u = torch.zeros(N, dtype=torch.float64, device=cuda)
    ft = torch.tensor(f, dtype=torch.float64, device=cuda)
    it, hist = mg.solve(u, ft)
    assert it == it_ref
    assert rel_err(u.cpu().numpy(), u_ref) <= 1e-8
    assert rel_err(hist, hist_ref) <= 1e-8


@pytest.mark.parametrize("dim,k,ncf,amp,local", [(3, 2, 8, 0.15, "surrogate"), (2, 3, 8, 0.25, "ksum")])
def test_mg_scaled_relaxation_on_distorted_mesh(tpss, oracle, mapped, cuda, dim, k, ncf, amp, local):
    """Spectrum-scaled damping: the per-level lambda_max(P A) estimates and the CG iterations
    match the oracle's; with it the 3D surrogate smoother converges where the reference's fixed
    damping makes the V-cycle indefinite."""
    import torch
    from tpss_gb300.mesh import distorted_cube
    X = distorted_cube(dim, [ncf] * dim, 7, amp)
    N = ncf ** dim * (k + 1) ** dim
    f = philox(7, N)
    om = oracle.lookup_damping_factor(1, 0, dim)
    it_ref, hist_ref, u_ref = mapped.mg_cg_solve_mapped(dim, k, 2, ncf, X, f, om, local=local,
                                                        auto_relaxation=True, max_iter=300)
    w_ref = mapped.mg_cg_solve_mapped.last_omegas
    ls = {"surrogate": tpss.LocalSolver.fd, "ksum": tpss.LocalSolver.ksum}[local]
    mg = tpss.MultigridSolver(dim, k, 2, ncf, relaxation=om, coarse_solver=1, vertex_coords=X,
                              local_solver=ls, auto_relaxation=True)
    for l in range(1, mg.n_levels):
        w, lam = mg.relaxation(l)
        assert abs(w - w_ref[l]) <= 1e-8 * w_ref[l]
    u = torch.zeros(N, dtype=torch.float64, device=cuda)
    it, hist = mg.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda), max_iter=300)
    assert it == it_ref > 0
    assert rel_err(u.cpu().numpy(), u_ref) <= 1e-8


def test_mg_fp32_vcycle_on_distorted_mesh(tpss, oracle, mapped, cuda):
    """Single-precision V-cycle on a distorted hierarchy (FP32 block-sparse level operators and
    transfers, FP32 smoothers): converges within two iterations of the FP64 V-cycle, and the
    returned solution meets the tolerance with the FP64 operator."""
    import torch
    from tpss_gb300.mesh import distorted_cube
    dim, k, ncf = 3, 2, 8
    X = distorted_cube(dim, [ncf] * dim, 7, 0.15)
    N = ncf ** dim * (k + 1) ** dim
    f = torch.tensor(philox(8, N), dtype=torch.float64, device=cuda)
    its = {}
    for vp in (0, 1):
        mg = tpss.MultigridSolver(dim, k, 2, ncf, relaxation=0.15, precision=1, coarse_solver=1,
                                  vertex_coords=X, auto_relaxation=True, vcycle_precision=vp)
        u = torch.zeros(N, dtype=torch.float64, device=cuda)
        it, hist = mg.solve(u, f, rel_tol=1e-8, max_iter=300)
        sh, op = _op(tpss, dim, k, (ncf,) * dim, X)
        r = torch.empty_like(u)
        op.vmult(r, u)
        assert float(torch.linalg.norm(f - r) / torch.linalg.norm(f)) <= 2e-8, vp
        its[vp] = it
    assert its[1] <= its[0] + 2, its
