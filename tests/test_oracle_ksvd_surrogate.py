"""KSVD and surrogate-patch parts of the oracle (no GPU).

Known answers of the reference (tests/kroneckersvd.cc:241-250, 274-283): the rank-2 KSVD of
diag(1..12) and of the same diagonal with entries 3 and 8 negated, 4x4 (x) 3x3 factors, first
term to 1e-6 -- signs included.  Rank-1/2 exactness follows tests/kroneckersvd.cc's rank tests.
Surrogate widths (TPSS/mapping_info.templates.h:42-240) are checked on Cartesian and affinely
stretched meshes, where they are exact, and against a numpy restatement on distorted meshes.
"""
import numpy as np
import pytest


def test_ksvd_diagonal_known_answers(oracle):
    B, A = oracle.ksvd_diag(np.arange(1.0, 13.0), 4, 3, 2)
    np.testing.assert_allclose(B[0], [0.710868, 1.735563, 2.760258, 3.784953], atol=1e-6)
    np.testing.assert_allclose(A[0], [2.545889, 2.899023, 3.252157], atol=1e-6)
    d = np.arange(1.0, 13.0)
    d[3], d[8] = -12.0, -33.0
    B, A = oracle.ksvd_diag(d, 4, 3, 2)
    np.testing.assert_allclose(B[0], [-0.422376, -1.250524, 5.699786, -1.457304], atol=1e-6)
    np.testing.assert_allclose(A[0], [1.097814, 0.618112, -5.896291], atol=1e-6)


@pytest.mark.parametrize("rank", [1, 2])
def test_ksvd_recovers_low_kronecker_rank(oracle, rank):
    g = np.random.default_rng(rank)
    M = sum(np.kron(g.standard_normal((4, 3)), g.standard_normal((2, 5))) for _ in range(rank))
    B, A = oracle.ksvd(M, (4, 3), (2, 5), rank)
    R = sum(np.kron(B[r], A[r]) for r in range(rank))
    np.testing.assert_allclose(R, M, atol=1e-11 * np.abs(M).max())


def test_ksvd_is_best_approximation(oracle):
    """Rank-r truncation error equals the tail of the rearranged matrix's singular values."""
    g = np.random.default_rng(7)
    M = g.standard_normal((12, 12))
    B, A = oracle.ksvd(M, (4, 4), (3, 3), 2)
    R = np.zeros((16, 9))
    for k in range(4):
        for l in range(4):
            R[k * 4 + l] = M[k * 3:(k + 1) * 3, l * 3:(l + 1) * 3].reshape(-1)
    s = np.linalg.svd(R, compute_uv=False)
    err = np.linalg.norm(M - np.kron(B[0], A[0]) - np.kron(B[1], A[1]))
    np.testing.assert_allclose(err, np.sqrt(np.sum(s[2:] ** 2)), rtol=1e-10)


def test_als_reproduces_reference_order3_case():
    from oracle import np_ksvd
    K, m, n, init = np_ksvd.reference_order3_case()
    F = np_ksvd.kcp_als(K, m, n, init, 14)  # rank^2 + 10 sweeps, compute_kcp's default
    assert np.abs(np_ksvd.kron_matrix(F) - K).max() <= 1e-12 * np.abs(K).max()


def test_als_rank2_matches_ksvd_of_reference_diagonal(oracle):
    """For two factors the ALS fixed point is the truncated SVD of the reshuffled matrix: on the
    reference's known-answer input diag(1..12) (4x4 (x) 3x3), the rank-2 approximation from ALS
    equals the one from the oracle's KSVD, whose first term is pinned to the reference's numbers."""
    from oracle import np_ksvd
    K = np.diag(np.arange(1.0, 13.0))
    B, A = oracle.ksvd(K, (4, 4), (3, 3), 2)
    ref = sum(np.kron(B[r], A[r]) for r in range(2))
    g = np.random.default_rng(3)
    init = [g.standard_normal((2, 3, 3)), g.standard_normal((2, 4, 4))]
    F = np_ksvd.kcp_als(K, (3, 4), (3, 4), init, 300)
    np.testing.assert_allclose(np_ksvd.kron_matrix(F), ref, atol=1e-9 * np.abs(ref).max())


def test_ksvd_separable_patch_matrix(oracle):
    """A Cartesian 2D FD patch matrix M (x) L + L (x) M has Kronecker rank 2 exactly."""
    M1, L1 = oracle.patch_matrices_1d(3, [0.25, 0.25], 0, 0)
    M2, L2 = oracle.patch_matrices_1d(3, [0.2, 0.3], 1, 0)
    K = np.kron(M2, L1) + np.kron(L2, M1)
    B, A = oracle.ksvd(K, (8, 8), (8, 8), 2)
    np.testing.assert_allclose(np.kron(B[0], A[0]) + np.kron(B[1], A[1]), K, atol=1e-10 * np.abs(K).max())


def _np_surrogate(dim, nc, X, nq=5):
    """numpy restatement: per cell arc lengths on a Gauss-Lobatto grid, averaged per patch."""
    from numpy.polynomial import legendre as L
    z = np.concatenate([[-1.0], np.sort(np.real(L.Legendre.basis(nq - 1).deriv().roots())), [1.0]])
    P = L.Legendre.basis(nq - 1)(z)
    w = 2.0 / (nq * (nq - 1) * P ** 2) / 2.0
    z = 0.5 * (z + 1.0)
    nv = [n + 1 for n in nc]

    def vid(v):
        return v[0] + nv[0] * (v[1] + (nv[1] if dim > 2 else 1) * (v[2] if dim > 2 else 0))

    def cmap(corner, xi):
        x = np.zeros(dim)
        for v in range(2 ** dim):
            wt = np.prod([xi[d] if (v >> d) & 1 else 1 - xi[d] for d in range(dim)])
            vv = [corner[d] + ((v >> d) & 1) for d in range(dim)]
            x += wt * X[vid(vv)]
        return x

    def cell_h(corner):
        h = np.zeros(dim)
        import itertools
        for d in range(dim):
            for face in itertools.product(range(nq), repeat=dim - 1):
                wf = np.prod([w[f] for f in face])
                pts = []
                for i in range(nq):
                    xi, t = [0.0] * dim, 0
                    for e in range(dim):
                        if e == d:
                            xi[e] = z[i]
                        else:
                            xi[e] = z[face[t]]
                            t += 1
                    pts.append(cmap(corner, xi))
                h[d] += wf * sum(np.linalg.norm(pts[i] - pts[i - 1]) for i in range(1, nq))
        return h

    lowers, _, _ = __import__("oracle.oracle", fromlist=["x"]).patches(dim, nc, 1, 0)
    out = np.zeros((len(lowers), dim, 2))
    for p, lo in enumerate(lowers):
        for cn in range(2 ** dim):
            corner = [lo[d] + ((cn >> d) & 1) for d in range(dim)]
            h = cell_h(corner)
            for d in range(dim):
                out[p, d, (cn >> d) & 1] += h[d] / 2 ** (dim - 1)
    return out


def test_surrogate_h_cartesian_and_stretched(oracle):
    for dim, nc in ((2, (4, 3)), (3, (3, 2, 4))):
        X = oracle.distorted_coords(dim, nc, 0, amplitude=0.0)
        hp = oracle.surrogate_h(dim, nc, X)
        for d in range(dim):
            np.testing.assert_allclose(hp[:, d, :], 1.0 / nc[d], rtol=1e-13)
        scale = np.array([2.0, 0.5, 3.0][:dim])
        hp2 = oracle.surrogate_h(dim, nc, X * scale[None, :])
        for d in range(dim):
            np.testing.assert_allclose(hp2[:, d, :], scale[d] / nc[d], rtol=1e-13)


def test_surrogate_h_distorted_vs_numpy(oracle):
    for dim, nc in ((2, (4, 3)), (3, (3, 3, 2))):
        X = oracle.distorted_coords(dim, nc, 3)
        np.testing.assert_allclose(oracle.surrogate_h(dim, nc, X), _np_surrogate(dim, nc, X), rtol=1e-12)


def test_surrogate_vmult_reduces_to_cartesian(oracle):
    dim, k, nc = 3, 2, (4, 3, 3)
    X = oracle.distorted_coords(dim, nc, 0, amplitude=0.0)
    hp = oracle.surrogate_h(dim, nc, X)
    src = np.random.default_rng(1).uniform(-1, 1, int(np.prod(nc)) * (k + 1) ** dim)
    a = oracle.schwarz_vmult_surrogate(dim, k, nc, hp, src, omega=0.7)
    b = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.7)
    np.testing.assert_allclose(a, b, rtol=1e-11, atol=1e-13)
