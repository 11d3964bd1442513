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
