"""CPU checks of the distorted-mesh oracles: mapped SIPG assembly, separable fits, numpy MLP."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def nd():
    from oracle import np_distorted
    return np_distorted


@pytest.fixture(scope="module")
def mlp():
    from oracle import np_mlp
    return np_mlp


@pytest.mark.parametrize("dim,k,nc", [(2, 2, [3, 4]), (3, 1, [2, 3, 2]), (2, 3, [2, 2])])
def test_mapped_assembly_on_cartesian_mesh_equals_tensor_assembly(nd, xcheck, dim, k, nc):
    A = nd.sipg_matrix_mapped(dim, k, nc, nd.cartesian_coords(dim, nc), ip=1.7)
    B = xcheck.sipg_matrix(dim, k, nc, ip=1.7)
    assert np.abs(A - B).max() <= 1e-13 * np.abs(B).max()


def test_mapped_assembly_symmetric_positive_definite(nd, oracle):
    X = oracle.distorted_coords(2, [4, 4], 3)
    A = nd.sipg_matrix_mapped(2, 2, [4, 4], X)
    assert np.abs(A - A.T).max() <= 1e-13 * np.abs(A).max()
    assert np.linalg.eigvalsh(A).min() > 0


def test_mapped_local_matrix_is_level_submatrix_of_cartesian_fd(nd, oracle, xcheck):
    """On an undistorted mesh the surrogate patch problems reproduce the exact patch matrix
    (the reference's relation tests/apps_laplace_integrator.cc:55-115)."""
    dim, k, nc = 2, 2, [4, 4]
    X = nd.cartesian_coords(dim, nc)
    A = nd.sipg_matrix_mapped(dim, k, nc, X)
    for lo, MA, _, _ in nd.patch_problems(dim, k, nc, X):
        idx = xcheck.patch_dofs(dim, k, nc, lo, 2)
        K = A[np.ix_(idx, idx)]
        Ks = sum(nd.kron_dirs([MA[e][0] if e != d else MA[d][1] for e in range(dim)]) for d in range(dim))
        assert np.abs(K - Ks).max() <= 1e-12 * np.abs(K).max()


@pytest.mark.parametrize("dim,k", [(2, 2), (3, 1)])
def test_ksum_fit_closed_form_equals_least_squares(nd, oracle, xcheck, dim, k):
    nc = [4] * dim
    X = oracle.distorted_coords(dim, nc, 11, 0.25)
    A = nd.sipg_matrix_mapped(dim, k, nc, X)
    for lo, MA, _, _ in nd.patch_problems(dim, k, nc, X)[:6]:
        idx = xcheck.patch_dofs(dim, k, nc, lo, 2)
        K = A[np.ix_(idx, idx)]
        Ms = [m for m, _ in MA]
        a = nd.ksum_fit_lstsq(K, Ms)
        b = nd.ksum_fit_closed(K, Ms)
        for d in range(dim):
            assert np.abs(a[d] - b[d]).max() <= 1e-9 * np.abs(a[d]).max()


def test_ksum_fit_exact_on_cartesian_patch(nd, xcheck):
    dim, k, nc = 3, 1, [3, 3, 3]
    X = nd.cartesian_coords(dim, nc)
    A = nd.sipg_matrix_mapped(dim, k, nc, X)
    for lo, MA, _, _ in nd.patch_problems(dim, k, nc, X):
        idx = xcheck.patch_dofs(dim, k, nc, lo, 2)
        K = A[np.ix_(idx, idx)]
        Ms = [m for m, _ in MA]
        Af = nd.ksum_fit_closed(K, Ms)
        Kf = sum(nd.kron_dirs([Ms[e] if e != d else Af[d] for e in range(dim)]) for d in range(dim))
        assert np.abs(K - Kf).max() <= 1e-11 * np.abs(K).max()


def test_learned_features_vanish_on_cartesian_mesh(nd):
    dim, nc = 2, [4, 5]
    X = nd.cartesian_coords(dim, nc)
    probs = nd.patch_problems(dim, 2, nc, X)
    F = nd.learned_features(dim, nc, X, probs)
    assert F.shape == (len(probs), 9 * 2 + 4)
    assert np.abs(F[:, :18]).max() <= 1e-12


def test_numpy_mlp_gradient_matches_finite_differences(mlp):
    rng = np.random.default_rng(0)
    widths = [5, 7, 6, 3]
    n = sum(widths[l] * widths[l + 1] + widths[l + 1] for l in range(3))
    p = rng.normal(0, 0.5, n)
    x = rng.normal(0, 1, (9, 5))
    t = rng.normal(0, 1, (9, 3))
    _, g = mlp.loss_grad(p, widths, x, t)
    eps = 1e-6
    fd = np.zeros(n)
    for i in range(n):
        e = np.zeros(n)
        e[i] = eps
        fd[i] = (mlp.loss_grad(p + e, widths, x, t)[0] - mlp.loss_grad(p - e, widths, x, t)[0]) / (2 * eps)
    assert np.abs(g - fd).max() <= 1e-7 * max(1.0, np.abs(fd).max())


def test_product_mesh_generator_matches_oracle_and_keeps_cells_valid(nd, oracle):
    from tpss_gb300.mesh import distorted_cube
    X = distorted_cube(3, [6, 5, 7], 3, 0.25)
    assert np.array_equal(X, oracle.distorted_coords(3, [6, 5, 7], 3, 0.25, mode="edge"))
    nc = [6, 5, 7]
    for c in [(i, j, l) for i in range(6) for j in range(5) for l in range(7)]:
        V = nd.cell_vertices(X, 3, nc, list(c))
        for corner in range(8):
            xi = [(corner >> d) & 1 for d in range(3)]
            assert np.linalg.det(nd.jacobian(V, xi)) > 0
