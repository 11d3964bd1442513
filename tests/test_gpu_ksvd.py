"""GPU low Kronecker-rank approximation (tpss_kronecker_approx) and the rank-2 Kronecker local
solver (TPSS_LOCAL_KSVD), against the numpy ALS restatement (oracle/np_ksvd.py).

Tolerances: ALS factors' Kronecker matrix 1e-10 relative to the numpy ALS from the same start
(the reference's order-3 case: exact recovery, 1e-12); local inverses 1e-8 relative to the
numpy inverse of the numpy-fitted rank-2 matrix; Cartesian 2D patches, where rank 2 is exact:
local inverse error <= 1e-10 and the smoother equal to the surrogate one to 1e-10.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("dim,m,n,rank,iters", [(2, (3, 4), (3, 4), 2, 14), (2, (5, 2), (3, 4), 1, 10),
                                                (3, (3, 2, 4), (3, 2, 4), 2, 14), (3, (2, 3, 2), (4, 2, 3), 2, 7)])
def test_kronecker_approx_matches_numpy_als(tpss, cuda, dim, m, n, rank, iters):
    import torch
    from oracle import np_ksvd
    g = np.random.default_rng(dim * 10 + rank)
    count = 5
    rows, cols = int(np.prod(m)), int(np.prod(n))
    K = g.standard_normal((count, rows, cols))
    init = [g.standard_normal((count, rank, m[d], n[d])) for d in range(dim)]
    got = tpss.kronecker_approx(torch.tensor(K, device=cuda), m, n,
                                [torch.tensor(f, device=cuda) for f in init], iterations=iters)
    for i in range(count):
        ref = np_ksvd.kcp_als(K[i], m, n, [f[i] for f in init], iters)
        Fi = [got[d][i].cpu().numpy() for d in range(dim)]
        assert rel(np_ksvd.kron_matrix(Fi), np_ksvd.kron_matrix(ref)) <= 1e-10, i


def test_kronecker_approx_reference_order3_case(tpss, cuda):
    import torch
    from oracle import np_ksvd
    K, m, n, init = np_ksvd.reference_order3_case()
    got = tpss.kronecker_approx(torch.tensor(K[None], device=cuda), m, n,
                                [torch.tensor(f[None], device=cuda) for f in init], iterations=14)
    F = [got[d][0].cpu().numpy() for d in range(3)]
    assert rel(np_ksvd.kron_matrix(F), K) <= 1e-12


def _surrogate_init(oracle, dim, k, nc, X, lower):
    """Per patch the surrogate 1-D matrices (surrogate widths, boundary flags) and the ALS start
    term 0 = (A_0, M_1[, M_2]), term 1 = (M_0, A_1[, M_2])."""
    hp = oracle.surrogate_h(dim, list(nc), X)
    inits = []
    for p, lo in enumerate(lower):
        Ms, As = [], []
        for d in range(dim):
            M1, A1 = oracle.patch_matrices_1d(k, hp[p, d], lo[d] == 0, lo[d] + 2 == nc[d])
            Ms.append(M1)
            As.append(A1)
        t0 = [As[0], Ms[1]] + ([Ms[2]] if dim == 3 else [])
        t1 = [Ms[0], As[1]] + ([Ms[2]] if dim == 3 else [])
        inits.append([np.stack([t0[d], t1[d]]) for d in range(dim)])
    return inits


@pytest.mark.parametrize("dim,k,nc,seed,amp", [(2, 2, (5, 4), 3, 0.2), (3, 2, (3, 3, 3), 4, 0.15)])
def test_ksvd_local_solver_vs_numpy(tpss, oracle, cuda, dim, k, nc, seed, amp):
    """The solver's local inverses equal the inverses of the numpy ALS fits of the exact patch
    matrices (same start, 14 sweeps), wherever the fit is kept; the local inverse errors
    against the exact inverses are reported for the three separable solvers."""
    from oracle import np_ksvd
    X = oracle.distorted_coords(dim, list(nc), seed, amp, mode="edge")
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc,
                                                                     patch_variant=1, vertex_coords=X))
    op = tpss.LaplaceOperator(sh)
    P = sh.n_subdomains()
    lower, _ = sh.patches()
    K = tpss.local_matrices(sh, op, 0, P, device=cuda).cpu().numpy()
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.5,
                                                                   local_solver=tpss.LocalSolver.ksvd))
    B = tpss.precond_local_inverse(p, 0, P, device=cuda).cpu().numpy()
    n1 = 2 * (k + 1)
    inits = _surrogate_init(oracle, dim, k, nc, X, lower)
    matched = 0
    for j in range(P):
        F = np_ksvd.kcp_als(K[j], [n1] * dim, [n1] * dim, inits[j], 14)
        Xj = np_ksvd.kron_matrix(F)
        if np.linalg.eigvalsh(0.5 * (Xj + Xj.T)).min() <= 0:
            continue  # such a patch keeps the surrogate
        if rel(B[j], np.linalg.inv(Xj)) <= 1e-8:
            matched += 1
    assert matched >= 0.8 * P, (matched, P)
    errs = {}
    for ls in (tpss.LocalSolver.fd, tpss.LocalSolver.ksum, tpss.LocalSolver.ksvd):
        q = tpss.SchwarzPreconditioner()
        q.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.5, local_solver=ls))
        errs[ls] = tpss.local_inverse_error(q, op, 0, P)
    assert np.all(np.isfinite(errs[tpss.LocalSolver.ksvd]))
    if dim == 2:
        # rank 2 holds the whole 2D Kronecker structure: the fit beats the surrogate on average
        assert errs[tpss.LocalSolver.ksvd].mean() < errs[tpss.LocalSolver.fd].mean()


def test_ksvd_local_solver_exact_on_cartesian_2d(tpss, oracle, cuda):
    import torch
    dim, k, nc = 2, 3, (5, 6)
    X = oracle.distorted_coords(dim, list(nc), 1, 0.0)
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc,
                                                                     patch_variant=1, vertex_coords=X))
    op = tpss.LaplaceOperator(sh)
    ps = {}
    for ls in (tpss.LocalSolver.fd, tpss.LocalSolver.ksvd):
        ps[ls] = tpss.SchwarzPreconditioner()
        ps[ls].initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.4, local_solver=ls))
    assert tpss.local_inverse_error(ps[tpss.LocalSolver.ksvd], op, 0, sh.n_subdomains()).max() <= 1e-10
    src = torch.tensor(np.random.default_rng(2).uniform(-1, 1, sh.n_dofs()), dtype=torch.float64, device=cuda)
    a, b = torch.empty_like(src), torch.empty_like(src)
    ps[tpss.LocalSolver.fd].vmult(a, src)
    ps[tpss.LocalSolver.ksvd].vmult(b, src)
    torch.cuda.synchronize()
    assert rel(b.cpu().numpy(), a.cpu().numpy()) <= 1e-10
