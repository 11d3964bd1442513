"""The CPU oracle against the reference's own relations and the golden fixtures (no GPU).

Reference tests restated (jwitte08/TPSS, tests/):
  patch_transfer.cc:146-313          gather/scatter partition of unity
  apps_laplace_integrator.cc:55-115  FD local matrix == submatrix of the level matrix
                                     (DGQ vertex patches, ip_factor = 12.34)
  tensor_product_matrix.cc:147-345   Kronecker-sum inverse vs the explicit matrix
  apps_poisson.cc:87-135             CG + GMG iteration upper bounds (AVP, ACP)
Tolerance of the reference helpers: numeric_eps<double> = 10^(log10(eps)/2) ~ 1.5e-8
(tests/test_utilities.h:30); the oracle meets 1e-12 on all of them.
"""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sl

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def kron_sum(Ms, As):
    """sum_d M_{dim-1} x .. x A_d x .. x M_0 (direction 0 fastest)."""
    dim = len(Ms)
    K = 0
    for d in range(dim):
        T = np.ones((1, 1))
        for e in reversed(range(dim)):
            T = np.kron(T, As[e] if e == d else Ms[e])
        K = K + T
    return K


def test_quadrature(oracle, xcheck):
    for n in range(1, 12):
        x, w = oracle.gauss(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        np.testing.assert_allclose(x, 0.5 * (xr + 1), atol=1e-15)
        np.testing.assert_allclose(w, 0.5 * wr, atol=1e-15)
    for k in range(1, 9):
        np.testing.assert_allclose(oracle.gauss_lobatto(k + 1), xcheck.gll_nodes(k), atol=1e-14)


def test_shape_data_partition_of_unity(oracle):
    for k in range(1, 8):
        s = oracle.shape_data(k)
        np.testing.assert_allclose(s["val"].sum(axis=0), 1.0, atol=1e-13)
        np.testing.assert_allclose(s["grad"].sum(axis=0), 0.0, atol=1e-10)
        # nodal (Kronecker delta) property at the Gauss-Lobatto nodes
        np.testing.assert_allclose(s["fval"][0], np.eye(k + 1)[0], atol=1e-14)
        np.testing.assert_allclose(s["fval"][1], np.eye(k + 1)[k], atol=1e-14)


@pytest.mark.parametrize("k", [1, 3, 5, 7])
@pytest.mark.parametrize("ncp", [1, 2])
def test_generalized_eigenproblem(oracle, k, ncp):
    h = [0.1, 0.13][:ncp]
    M, A = oracle.patch_matrices_1d(k, h, 1, 0, ip=1.0)
    S, lam = oracle.gen_eig(A, M)
    n = M.shape[0]
    np.testing.assert_allclose(S.T @ M @ S, np.eye(n), atol=1e-11)
    np.testing.assert_allclose(S.T @ A @ S, np.diag(lam), atol=1e-9 * lam.max())
    np.testing.assert_allclose(lam, sl.eigh(A, M, eigvals_only=True), rtol=1e-11)
    assert np.all(np.diff(lam) >= 0)


@pytest.mark.parametrize("dim,k,nc", [(2, 2, [4, 3]), (2, 4, [3, 3]), (3, 1, [3, 3, 2]),
                                      (3, 2, [2, 3, 2])])
@pytest.mark.parametrize("pv", [0, 1])
def test_local_matrix_is_level_submatrix(oracle, xcheck, dim, k, nc, pv):
    """CheckLocalSolvers: every FD local matrix equals the level matrix restricted to the
    patch DoFs (tests/apps_laplace_integrator.cc:55-115, ip_factor 12.34)."""
    ip = 12.34
    A = xcheck.sipg_matrix(dim, k, nc, ip=ip)
    lowers, _, _ = oracle.patches(dim, nc, pv, 0)
    ncp = 2 if pv else 1
    for lo in lowers:
        idx = xcheck.patch_dofs(dim, k, nc, lo, ncp)
        Ms, As = [], []
        for d in range(dim):
            c0, c1 = lo[d], lo[d] + ncp - 1
            M1, A1 = oracle.patch_matrices_1d(k, [1.0 / nc[d]] * ncp, c0 == 0, c1 == nc[d] - 1, ip)
            Ms.append(M1)
            As.append(A1)
        K = kron_sum(Ms, As)
        Kj = A[np.ix_(idx, idx)]
        assert np.abs(K - Kj).max() <= 1e-12 * np.abs(Kj).max()


@pytest.mark.parametrize("dim,k,nc", [(2, 3, [4, 4]), (2, 2, [3, 4]), (3, 2, [3, 2, 3])])
def test_kp1sq_penalty_matches_quadrature(oracle, xcheck, dim, k, nc):
    """The opt-in penalty 2(k+1)^2/h (interior faces 2(k+1)^2 (1/h_l+1/h_r)/2, Dirichlet faces
    2(k+1)^2/h): the oracle's operator equals the independent quadrature assembly, and every
    vertex-patch FD matrix equals the level submatrix, as in CheckLocalSolvers
    (tests/apps_laplace_integrator.cc:55-115)."""
    A = xcheck.sipg_matrix(dim, k, nc, penalty="kp1sq")
    Aref = xcheck.sipg_matrix(dim, k, nc)
    assert np.abs(A - Aref).max() > 1e-3 * np.abs(Aref).max()  # the mode changes the matrix
    v = np.random.default_rng(11).uniform(-1, 1, A.shape[0])
    got = oracle.sipg_vmult(dim, k, nc, v, penalty="kp1sq")
    assert np.abs(got - A @ v).max() <= 1e-12 * np.abs(A @ v).max()
    lowers, _, _ = oracle.patches(dim, nc, 1, 0)
    for lo in lowers:
        idx = xcheck.patch_dofs(dim, k, nc, lo, 2)
        Ms, As = [], []
        for d in range(dim):
            M1, A1 = oracle.patch_matrices_1d(k, [1.0 / nc[d]] * 2, lo[d] == 0, lo[d] + 1 == nc[d] - 1,
                                              penalty="kp1sq")
            Ms.append(M1)
            As.append(A1)
        Kj = A[np.ix_(idx, idx)]
        assert np.abs(kron_sum(Ms, As) - Kj).max() <= 1e-12 * np.abs(Kj).max()
    # the mode is reset after each call
    np.testing.assert_allclose(oracle.sipg_vmult(dim, k, nc, v), Aref @ v, rtol=0,
                               atol=1e-12 * np.abs(Aref @ v).max())


@pytest.mark.parametrize("dim,k,nc", [(2, 2, [5, 4]), (2, 3, [3, 3]), (3, 1, [3, 4, 3]), (3, 2, [3, 3, 3])])
def test_ras_boolean_weights_vs_dense_restricted_patch_solves(oracle, xcheck, dim, k, nc):
    """RAS boolean weights (rscatter_add, compute_restricted_dofs_impl in
    TPSS/dof_info.templates.h:194-313), restated here with numpy as the reference states it:
    collect for every global DoF all (distance to the patch centre, patch-local index, patch)
    occurrences, sort, and let only the first scatter. The restricted prolongations form a
    partition of unity (every DoF is scattered exactly once)."""
    A = xcheck.sipg_matrix(dim, k, nc)
    N = A.shape[0]
    lowers, _, _ = oracle.patches(dim, nc, 1, 0)
    n = 2 * (k + 1)
    occ = {}
    idxs = []
    for p, lo in enumerate(lowers):
        idx = xcheck.patch_dofs(dim, k, nc, lo, 2)
        idxs.append(idx)
        for i, g in enumerate(idx):
            m = [(i // n ** d) % n for d in range(dim)]
            dist = max(int(abs(n / 2.0 - 0.5 - md)) for md in m)
            occ.setdefault(int(g), []).append((dist, i, p))
    keep = [np.zeros(len(ix), dtype=bool) for ix in idxs]
    for g, lst in occ.items():
        _, i, p = sorted(lst)[0]
        keep[p][i] = True
    count = np.zeros(N)
    for p, ix in enumerate(idxs):
        np.add.at(count, ix[keep[p]], 1.0)
    assert np.all(count == 1.0)
    src = np.random.default_rng(21).uniform(-1, 1, N)
    om = 0.6
    ref = np.zeros(N)
    for p, ix in enumerate(idxs):
        u = om * np.linalg.solve(A[np.ix_(ix, ix)], src[ix])
        ref[ix[keep[p]]] += u[keep[p]]
    got = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=om, use_ras="boolean")
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("dim,n", [(2, 4), (2, 8), (3, 4), (3, 6)])
def test_fd_inverse_matches_explicit(oracle, dim, n):
    """Kronecker-sum apply_inverse against the explicit matrix (tensor_product_matrix.cc)."""
    g = np.random.default_rng(3)
    Ms, As, Ss, Ls = [], [], [], []
    for d in range(dim):
        B = g.standard_normal((n, n))
        M = B @ B.T + n * np.eye(n)
        C = g.standard_normal((n, n))
        A = C @ C.T + np.eye(n)
        S, lam = oracle.gen_eig(A, M)
        Ms.append(M); As.append(A); Ss.append(S); Ls.append(lam)
    K = kron_sum(Ms, As)
    r = g.uniform(-1, 1, n ** dim)
    u = oracle.fd_apply(Ss, Ls, r)
    np.testing.assert_allclose(K @ u, r, atol=1e-10 * np.abs(r).max() * np.linalg.cond(K) ** 0.5)
    np.testing.assert_allclose(u, np.linalg.solve(K, r), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("dim,k", [(2, 1), (2, 3), (3, 2)])
def test_partition_of_unity(oracle, dim, k):
    """sum_j R_j^T R_j v == v for cell patches (3x1(x1) cuboid) and for the single vertex
    patch of a 2^dim mesh (tests/patch_transfer.cc:146-313).  With identity local solvers
    (A_j = I) the Schwarz operator is exactly that sum; we obtain it by solving with the
    mass-free trick: one FD 'solve' with S = I and lambda = 1/dim."""
    g = np.random.default_rng(5)
    for pv, nc in ((0, [3] + [1] * (dim - 1)), (1, [2] * dim)):
        N = int(np.prod(nc)) * (k + 1) ** dim
        v = g.uniform(-1, 1, N)
        lowers, _, _ = oracle.patches(dim, nc, pv, 0)
        ncp = 2 if pv else 1
        from oracle import np_crosscheck as X
        dst = np.zeros(N)
        n = ncp * (k + 1)
        I = [np.eye(n)] * dim
        lam = [np.full(n, 1.0 / dim)] * dim
        for lo in lowers:
            idx = X.patch_dofs(dim, k, nc, lo, ncp)
            dst[idx] += oracle.fd_apply(I, lam, v[idx])
        np.testing.assert_allclose(dst, v, atol=1e-15)


@pytest.mark.parametrize("dim,k,nc,pv", [(2, 3, [5, 4], 1), (2, 2, [4, 4], 0), (3, 2, [3, 3, 3], 1),
                                         (3, 1, [3, 2, 3], 0)])
def test_schwarz_vmult_vs_dense_patch_solves(oracle, xcheck, dim, k, nc, pv):
    ip, om = 1.0, 0.37
    A = xcheck.sipg_matrix(dim, k, nc, ip=ip)
    src = np.random.default_rng(9).uniform(-1, 1, A.shape[0])
    lowers, _, _ = oracle.patches(dim, nc, pv, 0)
    ref = xcheck.schwarz_vmult_dense(A, dim, k, nc, lowers, 2 if pv else 1, om, src)
    got = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=pv, omega=om, ip=ip)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_schwarz_nonuniform_h_and_cell_permutation(oracle, xcheck):
    """Tensor-product meshes with varying h per direction and a permuted cell numbering."""
    dim, k, nc = 2, 2, [4, 3]
    h = [np.array([0.1, 0.3, 0.25, 0.35]), np.array([0.5, 0.2, 0.3])]
    N = 12 * 9
    src = np.random.default_rng(2).uniform(-1, 1, N)
    a = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=1.0, h=h)
    # permute the cell blocks: the result must permute the same way
    perm = np.random.default_rng(4).permutation(12)
    cell_start = perm * 9
    src_p = np.zeros(N)
    for c in range(12):
        src_p[cell_start[c]:cell_start[c] + 9] = src[c * 9:(c + 1) * 9]
    b = oracle.schwarz_vmult(dim, k, nc, src_p, patch_variant=1, omega=1.0, h=h,
                             cell_start=cell_start)
    for c in range(12):
        np.testing.assert_allclose(b[cell_start[c]:cell_start[c] + 9], a[c * 9:(c + 1) * 9],
                                   rtol=1e-14, atol=1e-14)
    # additive Schwarz with exact local solves is symmetric
    y = np.random.default_rng(8).uniform(-1, 1, N)
    Py = oracle.schwarz_vmult(dim, k, nc, y, patch_variant=1, omega=1.0, h=h)
    assert abs(y @ a - src @ Py) <= 1e-12 * abs(y @ a)


def test_sipg_operator_vs_quadrature(oracle, xcheck):
    for dim, k, nc, ip in ((2, 3, [4, 3], 1.0), (3, 2, [2, 3, 2], 2.5)):
        A = xcheck.sipg_matrix(dim, k, nc, ip=ip)
        v = np.random.default_rng(1).uniform(-1, 1, A.shape[0])
        got = oracle.sipg_vmult(dim, k, nc, v, ip=ip)
        assert np.abs(got - A @ v).max() <= 1e-12 * np.abs(A @ v).max()
        assert np.abs(A - A.T).max() <= 1e-12 * np.abs(A).max()
        assert np.linalg.eigvalsh(A).min() > 0


def test_transfer_embedding(oracle, xcheck):
    """Prolongation reproduces coarse polynomials exactly; restriction is its transpose."""
    dim, k, ncc = 2, 3, [2, 3]
    nf = [2 * n for n in ncc]
    nodes = xcheck.gll_nodes(k)
    npt = k + 1

    def interp(nc, fn):
        out = np.zeros(int(np.prod(nc)) * npt ** dim)
        for cy in range(nc[1]):
            for cx in range(nc[0]):
                cell = cx + nc[0] * cy
                for j in range(npt):
                    for i in range(npt):
                        x = (cx + nodes[i]) / nc[0]
                        y = (cy + nodes[j]) / nc[1]
                        out[cell * npt ** 2 + i + npt * j] = fn(x, y)
        return out

    f = lambda x, y: 1 + 2 * x - y + x * y ** 2 + 0.5 * x ** 3  # degree <= 3 per direction
    uc = interp(ncc, f)
    uf = oracle.prolongate_add(dim, k, ncc, uc, np.zeros(int(np.prod(nf)) * npt ** dim))
    np.testing.assert_allclose(uf, interp(nf, f), atol=1e-13)
    g = np.random.default_rng(0)
    a, b = g.standard_normal(uc.size), g.standard_normal(uf.size)
    Pa = oracle.prolongate_add(dim, k, ncc, a, np.zeros(uf.size))
    Rb = oracle.restrict_add(dim, k, ncc, np.zeros(uc.size), b)
    assert abs(Pa @ b - a @ Rb) < 1e-12 * abs(Pa @ b)


@pytest.mark.parametrize("dim,k,bound", [(2, 4, 15.0), (2, 7, 17.0), (3, 2, 21.0)])
def test_cg_gmg_iteration_bounds_avp(oracle, xcheck, dim, k, bound):
    """AVP bounds of tests/apps_poisson.cc:122-133: 2 root cells per direction,
    4-dim initial refinements, 3 cycles, rel. tolerance 1e-6, Gaussian-bell load."""
    for cycle in range(3):
        ncf = 2 * 2 ** (4 - dim + cycle)
        if dim == 3 and cycle == 2:
            ncf = 16
        f = xcheck.bells_load_vector(dim, k, ncf)
        it, _, hist = oracle.mg_cg_solve(dim, k, 2, ncf, f, patch_variant=1, smoother_variant=0,
                                         rel_tol=1e-6)
        n_frac, _ = oracle.fractional_steps(hist, 1e-6)
        assert it > 0 and n_frac < bound, (ncf, it, n_frac)


@pytest.mark.parametrize("dim,k,bound", [(2, 4, 11.0), (3, 2, 12.0)])
def test_cg_gmg_iteration_bounds_acp(oracle, xcheck, dim, k, bound):
    """ACP bounds of tests/apps_poisson.cc:90-97 (additive cell patches, damping 0.7)."""
    for cycle in range(2):
        ncf = 2 * 2 ** (4 - dim + cycle)
        f = xcheck.bells_load_vector(dim, k, ncf)
        it, _, hist = oracle.mg_cg_solve(dim, k, 2, ncf, f, patch_variant=0, smoother_variant=0,
                                         rel_tol=1e-6)
        n_frac, _ = oracle.fractional_steps(hist, 1e-6)
        assert it > 0 and n_frac < bound, (ncf, it, n_frac)


def test_golden_fd1d(oracle):
    g = np.load(os.path.join(GOLDEN, "fd1d.npz"))
    for k in range(1, 8):
        for ncp in (1, 2):
            for lo, hi in ((0, 0), (1, 0), (0, 1), (1, 1)):
                key = f"k{k}_ncp{ncp}_lo{lo}_hi{hi}"
                M, A = oracle.patch_matrices_1d(k, [0.125] * ncp, lo, hi, ip=1.0)
                np.testing.assert_allclose(M, g[key + "_M"], rtol=1e-13, atol=1e-15)
                np.testing.assert_allclose(A, g[key + "_A"], rtol=1e-13, atol=1e-12)
                _, lam = oracle.gen_eig(A, M)
                np.testing.assert_allclose(lam, g[key + "_lam"], rtol=1e-12)


def test_golden_vmult(oracle):
    g = np.load(os.path.join(GOLDEN, "vmult.npz"))
    cases = json.load(open(os.path.join(GOLDEN, "vmult_cases.json")))
    for i, c in enumerate(cases):
        got = oracle.schwarz_vmult(c["dim"], c["k"], c["n_cells"], g[f"c{i}_src"],
                                   patch_variant=c["patch_variant"],
                                   smoother_variant=c["smoother_variant"], omega=c["omega"],
                                   ip=c["ip"])
        ref = g[f"c{i}_dst"]
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max(), i


def test_golden_mg_iterations(oracle, xcheck):
    for c in json.load(open(os.path.join(GOLDEN, "mg_iterations.json"))):
        if c["dim"] == 3 and c["k"] >= 3:
            continue  # the largest case runs in the GPU tests only
        N = c["n_cells_fine"] ** c["dim"] * (c["k"] + 1) ** c["dim"]
        if c["rhs"] == "random":
            f = np.random.Generator(np.random.Philox(c["rhs_seed"])).uniform(-1, 1, N)
        else:
            f = xcheck.bells_load_vector(c["dim"], c["k"], c["n_cells_fine"])
        it, _, _ = oracle.mg_cg_solve(c["dim"], c["k"], c["n_rep"], c["n_cells_fine"], f,
                                      patch_variant=c["patch_variant"],
                                      smoother_variant=c["smoother_variant"], rel_tol=c["rel_tol"])
        assert it == c["iterations"]


@pytest.mark.parametrize("dim,k,nc,pv", [(2, 3, (6, 5), 1), (2, 2, (5, 3), 0), (3, 2, (4, 3, 5), 1),
                                         (3, 4, (4, 4, 4), 1), (3, 3, (3, 2, 4), 0), (3, 7, (2, 3, 2), 1)])
def test_simd_cpu_baseline_matches_oracle(oracle, dim, k, nc, pv):
    """The timed CPU baseline (oracle/simd_baseline.c: 8-lane macro patches, FMA allowed) is the
    same smoother as the strict oracle: relative max-norm error <= 1e-12, full vmult and a
    patch range."""
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = np.random.default_rng(17).uniform(-1, 1, N)
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=pv, omega=0.41)
    h = oracle.SimdSchwarzHandle(dim, k, nc, patch_variant=pv, omega=0.41)
    got = np.full(N, np.nan)
    h.apply(got, src)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    part = np.zeros(N)
    h.apply_range(0, h.n_patches, part, src)
    assert np.abs(part - ref).max() <= 1e-12 * np.abs(ref).max()
    h.close()
