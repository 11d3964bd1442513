"""GPU parity of the local solvers built from exact patch matrices, and of the learned solver.

Tolerances: exact patch matrices and FP64 smoothers 1e-12 relative (1e-10 where a 1-D
eigenproblem of a fitted matrix enters); FP32 dense smoother 2e-5; network forward pass and
gradients (FP32 on the GPU against the FP64 numpy restatement) 1e-4 relative to the largest
entry; features and targets (FP32 outputs) 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def philox(seed, n):
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, n)


@pytest.fixture(scope="module")
def nd():
    from oracle import np_distorted
    return np_distorted


@pytest.fixture(scope="module")
def npmlp():
    from oracle import np_mlp
    return np_mlp


def level(tpss, dim, k, nc, X, ip=1.0):
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1,
                                              vertex_coords=X)
    sh = tpss.SubdomainHandler(ad)
    return sh, tpss.LaplaceOperator(sh, ip)


def smoother(tpss, sh, op, cuda, src, local_solver, omega=0.5, precision=0, model=None, ip=1.0):
    import torch
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(
        relaxation=omega, precision=precision, local_solver=local_solver, model=model, ip_factor=ip))
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    d = torch.full_like(s, 5.0)
    p.vmult(d, s)
    torch.cuda.synchronize()
    return d.cpu().numpy()


@pytest.mark.parametrize("dim,k,nc,seed", [(2, 3, (4, 5), 1), (3, 1, (3, 3, 4), 2), (3, 2, (3, 3, 3), 3)])
def test_local_matrices_are_level_submatrices(tpss, oracle, nd, xcheck, cuda, dim, k, nc, seed):
    X = oracle.distorted_coords(dim, list(nc), seed, 0.25)
    A = nd.sipg_matrix_mapped(dim, k, list(nc), X)
    sh, op = level(tpss, dim, k, nc, X)
    P = sh.n_subdomains()
    got = tpss.local_matrices(sh, op, 0, P, device=cuda).cpu().numpy()
    lo_g, _ = sh.patches()
    for p in range(P):
        idx = xcheck.patch_dofs(dim, k, list(nc), lo_g[p][:dim], 2)
        assert rel_err(got[p], A[np.ix_(idx, idx)]) <= 1e-12


@pytest.mark.parametrize("dim,k,nc,seed", [(2, 3, (5, 4), 11), (3, 3, (3, 3, 3), 12)])
def test_local_inverse_error(tpss, oracle, nd, xcheck, cuda, dim, k, nc, seed):
    """tpss_precond_local_inverse and tpss_local_inverse_error against numpy: the dense local
    inverses the preconditioner applies, the relative Frobenius error of each against the FP64
    inverse of the exact patch matrix (1e-8 relative agreement with numpy), zero error (1e-10)
    for the exact local solver and for surrogate patches on an undistorted mesh."""
    X = oracle.distorted_coords(dim, list(nc), seed, 0.25)
    A = nd.sipg_matrix_mapped(dim, k, list(nc), X)
    sh, op = level(tpss, dim, k, nc, X)
    P = sh.n_subdomains()
    lo, _ = sh.patches()
    exact_inv = [np.linalg.inv(A[np.ix_(ix, ix)])
                 for ix in (xcheck.patch_dofs(dim, k, list(nc), lo[p][:dim], 2) for p in range(P))]
    for ls in (tpss.LocalSolver.fd, tpss.LocalSolver.ksum, tpss.LocalSolver.exact):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.5, local_solver=ls))
        B = tpss.precond_local_inverse(p, 0, P, device=cuda).cpu().numpy()
        err = tpss.local_inverse_error(p, op, 0, P)
        ref = np.array([np.linalg.norm(B[j] - exact_inv[j]) / np.linalg.norm(exact_inv[j]) for j in range(P)])
        np.testing.assert_allclose(err, ref, rtol=1e-8, atol=1e-13)
        if ls == tpss.LocalSolver.exact:
            assert err.max() <= 1e-10
        else:
            assert err.min() > 1e-6  # a distorted patch is not separable
    # an undistorted level: surrogate fast diagonalization is the exact local inverse
    Xc = oracle.distorted_coords(dim, list(nc), seed, 0.0)
    shc, opc = level(tpss, dim, k, nc, Xc)
    pc = tpss.SchwarzPreconditioner()
    pc.initialize(shc, opc, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.5))
    assert tpss.local_inverse_error(pc, opc, 0, shc.n_subdomains()).max() <= 1e-10


@pytest.mark.parametrize("dim,k,nc,seed,precision", [(2, 3, (5, 4), 4, 0), (2, 2, (6, 6), 5, 1),
                                                      (3, 1, (4, 3, 3), 6, 0), (3, 3, (3, 3, 3), 13, 0)])
def test_exact_local_solver_vs_dense_patch_solves(tpss, oracle, nd, xcheck, cuda, dim, k, nc, seed, precision):
    X = oracle.distorted_coords(dim, list(nc), seed, 0.25)
    A = nd.sipg_matrix_mapped(dim, k, list(nc), X)
    sh, op = level(tpss, dim, k, nc, X)
    src = philox(seed, A.shape[0])
    got = smoother(tpss, sh, op, cuda, src, tpss.LocalSolver.exact, omega=0.4, precision=precision)
    lo, _, _ = oracle.patches(dim, list(nc), 1)
    ref = xcheck.schwarz_vmult_dense(A, dim, k, list(nc), [l[:dim] for l in lo], 2, 0.4, src)
    assert rel_err(got, ref) <= (1e-12 if precision == 0 else 2e-5)


@pytest.mark.parametrize("dim,k,nc,seed", [(2, 3, (5, 4), 7), (3, 2, (3, 4, 3), 8)])
def test_ksum_local_solver_vs_numpy_fit(tpss, oracle, nd, xcheck, cuda, dim, k, nc, seed):
    X = oracle.distorted_coords(dim, list(nc), seed, 0.25)
    A = nd.sipg_matrix_mapped(dim, k, list(nc), X)
    sh, op = level(tpss, dim, k, nc, X)
    src = philox(seed, A.shape[0])
    got = smoother(tpss, sh, op, cuda, src, tpss.LocalSolver.ksum, omega=0.3)
    ref = np.zeros_like(src)
    for lo, MA, _, _ in nd.patch_problems(dim, k, list(nc), X):
        idx = xcheck.patch_dofs(dim, k, list(nc), lo, 2)
        Ms = [m for m, _ in MA]
        Af = nd.keep_definite(Ms, nd.ksum_fit_closed(A[np.ix_(idx, idx)], Ms), [a for _, a in MA])
        ref[idx] += 0.3 * (nd.fd_inverse(Ms, Af) @ src[idx])
    assert rel_err(got, ref) <= 1e-10


def test_learned_features_and_targets_vs_numpy(tpss, oracle, nd, cuda):
    dim, k, nc = 2, 2, [6, 5]
    X = oracle.distorted_coords(dim, nc, 9, 0.25)
    A = nd.sipg_matrix_mapped(dim, k, nc, X)
    sh, op = level(tpss, dim, k, tuple(nc), X)
    probs = nd.patch_problems(dim, k, nc, X)
    F = tpss.learned_features(sh, device=cuda).cpu().numpy()
    T = tpss.learned_targets(sh, op, device=cuda).cpu().numpy()
    Fr = nd.learned_features(dim, nc, X, probs)
    Tr = nd.learned_targets(dim, k, nc, A, probs)
    assert rel_err(F, Fr) <= 1e-5
    assert rel_err(T, Tr) <= 1e-5


def test_mlp_forward_and_gradient_vs_numpy(tpss, npmlp, cuda):
    import torch
    m = tpss.MLP(11, 5, n_hidden=16, n_hidden_layers=3, seed=3)
    widths = [11, 16, 16, 16, 5]
    p = m.get_params()
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1, (37, 11)).astype(np.float32)
    t = rng.normal(0, 1, (37, 5)).astype(np.float32)
    xd, td = torch.tensor(x, device=cuda), torch.tensor(t, device=cuda)
    y = m.forward(xd).cpu().numpy()
    yr, _ = npmlp.forward(p, widths, x)
    assert rel_err(y, yr) <= 1e-4
    loss, g = m.loss_grad(xd, td)
    lr, gr = npmlp.loss_grad(p, widths, x, t)
    assert abs(loss - lr) <= 1e-5 * lr
    assert rel_err(g, gr) <= 1e-4


def test_mlp_training_is_deterministic_and_reduces_loss(tpss, cuda):
    import torch
    rng = np.random.default_rng(2)
    x = torch.tensor(rng.normal(0, 1, (512, 6)).astype(np.float32), device=cuda)
    t = torch.sin(x[:, :2] * 1.5) + 0.3 * x[:, 2:4]
    runs = []
    for _ in range(2):
        m = tpss.MLP(6, 2, n_hidden=32, n_hidden_layers=2, seed=5)
        l0 = m.loss(x, t.contiguous())
        hist = m.train(x, t.contiguous(), epochs=40, batch=64, lr=3e-3, seed=7)
        runs.append((l0, hist, m.get_params()))
    assert np.array_equal(runs[0][2], runs[1][2])
    assert runs[0][1][-1] < 0.1 * runs[0][0]


def test_learned_solver_with_zero_network_equals_surrogate(tpss, oracle, cuda):
    """A network whose output is zero leaves the surrogate problems unchanged."""
    dim, k, nc = 2, 3, (5, 6)
    X = oracle.distorted_coords(dim, list(nc), 10, 0.25)
    sh, op = level(tpss, dim, k, nc, X)
    n_in, n_out = tpss.learned_sizes(sh)
    m = tpss.MLP(n_in, n_out, n_hidden=8, n_hidden_layers=1, seed=0)
    m.set_params(np.zeros(m.n_params, dtype=np.float32))
    src = philox(10, sh.n_dofs())
    a = smoother(tpss, sh, op, cuda, src, tpss.LocalSolver.learned, omega=0.25, model=m)
    b = smoother(tpss, sh, op, cuda, src, tpss.LocalSolver.fd, omega=0.25)
    assert rel_err(a, b) <= 1e-12


def test_learned_solver_gains_over_surrogate_on_unseen_mesh(tpss, oracle, cuda):
    """Train on patches of eight distorted meshes, then compare CG + V-cycle iterations on a
    ninth: learned corrections must need fewer iterations than the plain surrogate patches,
    and the exact-matrix fit (the network's target) bounds what they can reach."""
    import torch
    dim, k, ncf = 2, 2, 16
    xs, ys = [], []
    for seed in range(21, 29):
        X = oracle.distorted_coords(dim, [ncf] * dim, seed, 0.2)
        sh, op = level(tpss, dim, k, (ncf, ncf), X)
        xs.append(tpss.learned_features(sh, device=cuda))
        ys.append(tpss.learned_targets(sh, op, device=cuda))
    x, y = torch.cat(xs), torch.cat(ys)
    n_in, n_out = x.shape[1], y.shape[1]
    m = tpss.MLP(n_in, n_out, n_hidden=64, n_hidden_layers=3, seed=1)
    l0 = m.loss(x, y)
    hist = m.train(x, y, epochs=300, batch=64, lr=1e-3, seed=3)
    assert hist[-1] < 0.5 * l0
    X = oracle.distorted_coords(dim, [ncf] * dim, 99, 0.2)
    f = philox(99, ncf ** dim * (k + 1) ** dim)
    its = {}
    for name, ls, model in (("surrogate", 0, None), ("learned", 3, m), ("ksum", 2, None)):
        mg = tpss.MultigridSolver(dim, k, 2, ncf, relaxation=0.25, coarse_solver=1, vertex_coords=X,
                                  local_solver=ls, model=model)
        u = torch.zeros(len(f), dtype=torch.float64, device=cuda)
        try:
            its[name], _ = mg.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda), max_iter=200)
        except tpss.TPSSNotConverged:
            its[name] = 10 ** 9
    print("CG iterations on the unseen mesh:", its)
    assert its["ksum"] < its["surrogate"]
    assert its["learned"] < its["surrogate"]
