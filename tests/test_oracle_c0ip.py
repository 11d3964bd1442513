"""CPU checks of the C0IP oracle (oracle/np_c0ip.py)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def c0():
    from oracle import np_c0ip
    return np_c0ip


@pytest.mark.parametrize("k,nc", [(2, 3), (3, 2), (3, 3), (4, 2)])
def test_kronecker_form_equals_2d_quadrature(c0, k, nc):
    A = c0.level_matrix(k, nc, 1.3)
    Q = c0.matrix_2d_quadrature(k, nc, 1.3)
    assert np.abs(A - Q).max() <= 1e-13 * np.abs(Q).max()


@pytest.mark.parametrize("k,nc", [(2, 3), (3, 2), (4, 3)])
def test_q_poisson_kronecker_form_and_patch_matrices(c0, k, nc):
    """Poisson with continuous FE_Q(k): the Kronecker form M x L + L x M equals a plain 2-D
    quadrature assembly, and every vertex patch matrix of the (2k-1)^2 interior patch nodes (the
    Q layout, TPSS/patch_dof_worker.h:265-300) equals the Kronecker sum of the restricted 1-D
    matrices -- the relation of FDAssemblyVertexPatch / FDInverseVertexPatch for Q
    (tests/apps_laplace_integrator.cc:393-430), so fast diagonalization is the exact local solver."""
    A = c0.level_matrix(k, nc, problem="poisson")
    Q = c0.poisson_q_matrix_quadrature(k, nc)
    assert np.abs(A - Q).max() <= 1e-13 * np.abs(Q).max()
    M, L, _ = c0.matrices_1d(k, [1.0 / nc] * nc)
    m = 2 * k - 1
    for vx, vy, _ in c0.patches(nc):
        idx = c0.patch_indices(k, nc, vx, vy)
        sx = slice((vx - 1) * k, (vx - 1) * k + m)
        sy = slice((vy - 1) * k, (vy - 1) * k + m)
        K = np.kron(M[sy, sy], L[sx, sx]) + np.kron(L[sy, sy], M[sx, sx])
        assert np.abs(A[np.ix_(idx, idx)] - K).max() <= 1e-13 * np.abs(K).max()
        Ki = np.linalg.inv(K)
        assert np.abs(Ki @ K - np.eye(len(idx))).max() <= 1e-10


def test_level_matrix_spd(c0):
    A = c0.level_matrix(3, 4)
    assert np.abs(A - A.T).max() <= 1e-13 * np.abs(A).max()
    assert np.linalg.eigvalsh(A).min() > 0


@pytest.mark.parametrize("k", [2, 3, 5])
def test_prolongation_reproduces_coarse_functions(c0, k):
    """Continuous Q_k on the coarse mesh is Q_k on the refined mesh: prolongation of nodal
    values equals interpolation of the same polynomial-per-cell function at the fine nodes."""
    ncc = 3
    nodes = c0.gll_nodes(k)
    xc = np.concatenate([[(c + z) / ncc for z in nodes[:-1]] for c in range(ncc)] + [[1.0]])
    xf = np.concatenate([[(c + z) / (2 * ncc) for z in nodes[:-1]] for c in range(2 * ncc)] + [[1.0]])
    f = lambda x: np.sin(3 * x) * x * (1 - x)  # vanishes at the boundary
    # coarse nodal values; fine values = the coarse interpolant at the fine nodes
    uc = f(xc)
    _, P, _, _ = c0.basis_1d(k)
    uf_ref = np.zeros(len(xf))
    for i, x in enumerate(xf):
        c = min(int(x * ncc), ncc - 1)
        t = x * ncc - c
        uf_ref[i] = sum(uc[c * k + j] * P[j](t) for j in range(k + 1))
    Pm = c0.prolongation_1d(k, ncc)
    assert np.abs(Pm @ uc[1:-1] - uf_ref[1:-1]).max() <= 1e-12


def test_oracle_mg_converges(c0):
    k, nc = 2, 8
    f = np.random.default_rng(0).uniform(-1, 1, (nc * k - 1) ** 2)
    it, hist, u = c0.mg_cg_solve(k, 2, nc, f, 0.25, "exact")
    assert 0 < it < 40
    A = c0.level_matrix(k, nc)
    assert np.linalg.norm(f - A @ u) <= 1e-8 * np.linalg.norm(f)
