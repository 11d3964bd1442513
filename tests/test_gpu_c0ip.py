"""GPU parity of the C0IP biharmonic path against the numpy oracle (oracle/np_c0ip.py).

Tolerances: operator, transfer-based V-cycle and FP64 smoothers 1e-12 relative; FP32 smoother
2e-5 relative; CG + V-cycle iteration counts identical to the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def philox(seed, n):
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, n)


@pytest.fixture(scope="module")
def c0():
    from oracle import np_c0ip
    return np_c0ip


@pytest.mark.parametrize("k,nc", [(2, 3), (3, 4), (4, 2), (5, 3), (7, 2)])
def test_c0ip_operator(tpss, c0, cuda, k, nc):
    import torch
    P = tpss.C0IPBiharmonic(k, nc, nc, ip_factor=1.4)
    A = c0.level_matrix(k, nc, 1.4)
    x = philox(k, A.shape[0])
    xs = torch.tensor(x, dtype=torch.float64, device=cuda)
    y = torch.full_like(xs, 3.0)
    P.vmult(y, xs)
    assert rel_err(y.cpu().numpy(), A @ x) <= 1e-12


@pytest.mark.parametrize("k,nc,local,prec", [(2, 6, 1, 0), (3, 4, 1, 0), (3, 4, 0, 0), (4, 4, 0, 0),
                                             (3, 6, 1, 1), (3, 6, 0, 1), (5, 4, 1, 0)])
def test_c0ip_smoother(tpss, c0, cuda, k, nc, local, prec):
    """Fine level of a two-level hierarchy (nc cells per direction)."""
    import torch
    P = tpss.C0IPBiharmonic(k, nc // 2, nc, local_solver=local, precision=prec, relaxation=0.3)
    n = (nc * k - 1) ** 2
    x = philox(10 + k, n)
    xs = torch.tensor(x, dtype=torch.float64, device=cuda)
    y = torch.full_like(xs, 7.0)
    P.smooth(y, xs)
    ref = c0.schwarz_vmult(k, nc, x, 0.3, "exact" if local == 1 else "bilaplacian")
    assert rel_err(y.cpu().numpy(), ref) <= (1e-12 if prec == 0 else 2e-5)


@pytest.mark.parametrize("k,nc", [(2, 4), (3, 3), (5, 2)])
def test_q_poisson_operator(tpss, c0, cuda, k, nc):
    """Poisson with continuous FE_Q(k) (the Q vertex-patch layout): level operator 1e-12."""
    import torch
    P = tpss.C0IPBiharmonic(k, nc, nc, problem=tpss.C0IPBiharmonic.Q_POISSON)
    A = c0.level_matrix(k, nc, problem="poisson")
    x = philox(30 + k, A.shape[0])
    y = torch.full((A.shape[0],), 3.0, dtype=torch.float64, device=cuda)
    P.vmult(y, torch.tensor(x, dtype=torch.float64, device=cuda))
    assert rel_err(y.cpu().numpy(), A @ x) <= 1e-12


@pytest.mark.parametrize("k,nc,local,prec", [(2, 6, 1, 0), (3, 4, 0, 0), (3, 4, 1, 0), (4, 4, 0, 1), (6, 4, 0, 0)])
def test_q_poisson_smoother(tpss, c0, cuda, k, nc, local, prec):
    """Additive Q vertex patches ((2k-1)^2 nodes): exact and fast-diagonalization local solvers
    (identical here), FP64 1e-12 and FP32 2e-5 against the numpy dense patch solves."""
    import torch
    P = tpss.C0IPBiharmonic(k, nc // 2, nc, local_solver=local, precision=prec, relaxation=0.3,
                            problem=tpss.C0IPBiharmonic.Q_POISSON)
    n = (nc * k - 1) ** 2
    x = philox(40 + k, n)
    y = torch.full((n,), 7.0, dtype=torch.float64, device=cuda)
    P.smooth(y, torch.tensor(x, dtype=torch.float64, device=cuda))
    ref = c0.schwarz_vmult(k, nc, x, 0.3, "exact", problem="poisson")
    assert rel_err(y.cpu().numpy(), ref) <= (1e-12 if prec == 0 else 2e-5)


@pytest.mark.parametrize("k,n_rep,ncf,local", [(2, 2, 16, 0), (3, 2, 8, 1), (4, 2, 8, 0)])
def test_q_poisson_cg_mg_iterations(tpss, c0, cuda, k, n_rep, ncf, local):
    """CG + V-cycle with the Q vertex-patch smoother (damping 0.25, TPSS.h:121-163): iteration
    counts identical to the numpy oracle, solution 1e-8."""
    import torch
    n = (ncf * k - 1) ** 2
    f = philox(50 + k, n)
    it_ref, _, u_ref = c0.mg_cg_solve(k, n_rep, ncf, f, 0.25, "exact", problem="poisson")
    P = tpss.C0IPBiharmonic(k, n_rep, ncf, local_solver=local, relaxation=0.25,
                            problem=tpss.C0IPBiharmonic.Q_POISSON)
    u = torch.zeros(n, dtype=torch.float64, device=cuda)
    it, _ = P.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda))
    assert it == it_ref
    assert rel_err(u.cpu().numpy(), u_ref) <= 1e-8


@pytest.mark.parametrize("k,n_rep,ncf,local", [(2, 2, 8, 1), (3, 2, 8, 1), (3, 2, 16, 0), (4, 2, 8, 0)])
def test_c0ip_cg_mg_iterations(tpss, c0, cuda, k, n_rep, ncf, local):
    import torch
    n = (ncf * k - 1) ** 2
    f = philox(20 + k, n)
    loc = "exact" if local == 1 else "bilaplacian"
    it_ref, hist_ref, u_ref = c0.mg_cg_solve(k, n_rep, ncf, f, 0.25, loc)
    P = tpss.C0IPBiharmonic(k, n_rep, ncf, local_solver=local, relaxation=0.25)
    u = torch.zeros(n, dtype=torch.float64, device=cuda)
    it, hist = P.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda))
    assert it == it_ref
    assert rel_err(u.cpu().numpy(), u_ref) <= 1e-8
