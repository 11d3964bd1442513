"""Low Kronecker-rank approximation by alternating least squares, restated in numpy.

TEST INFRASTRUCTURE ONLY: tests/ use it as the checker of the GPU approximation
(tpss_kronecker_approx) and of the rank-2 Kronecker local solver; the product never imports it.

Follows compute_kcp (include/solvers_and_preconditioners/TPSS/kroneckersvd.h:501-585): with the
reshuffled tensor T(a_0, .., a_{D-1}), a_d = i_d n_d + j_d, of a matrix
K = sum_r F_{D-1,r} x .. x F_{0,r} (direction 0 fastest), one sweep updates for d = 0..D-1
    F_d <- T_(d) (khatri-rao of the other factors) V^+,   V = hadamard_{e != d} F_e^T F_e.
For two factors the fixed point spans the leading singular pairs of the reshuffled matrix, which
compute_ksvd (kroneckersvd.h:306-402) obtains by Lanczos bidiagonalization.
"""
from __future__ import annotations

import numpy as np


def reshuffle(K, m, n):
    """T[a_0, .., a_{D-1}] with a_d = i_d n_d + j_d for K[(i_{D-1} .. i_0), (j_{D-1} .. j_0)]."""
    D = len(m)
    T = K.reshape(list(reversed(m)) + list(reversed(n)))  # axes i_{D-1}..i_0, j_{D-1}..j_0
    # bring to (i_0, j_0, i_1, j_1, ...)
    axes = []
    for d in range(D):
        axes += [D - 1 - d, 2 * D - 1 - d]
    T = T.transpose(axes)
    return T.reshape([m[d] * n[d] for d in range(D)])


def reference_order3_case():
    """The order-3 case of the reference's tests/kroneckersvd.cc (test_three_dim_kronecker_cp): a
    Kronecker-rank-2 matrix t1 x t2 x t2 + t3 x t4 x t4 + 0.8 t3 x t4 x t4 given by three terms;
    CP/ALS of rank 2 started from the first two terms must reproduce it. Returned with direction
    0 fastest: (K, m = (2, 2, 4), n = (2, 2, 3), initial factors per direction [rank, m_d, n_d])."""
    t1 = np.array([[1, 0, 1], [0, 1, 0.1], [1, 0.1, -7], [0, -1, 0]], dtype=float)
    t2 = np.array([[1, 2], [2, 4]], dtype=float)
    t3 = np.array([[0.5, 3, 2], [3.4, 1, -0.4], [2, -0.5, 0], [0, 0, 0]], dtype=float)
    t4 = np.array([[1, 1], [1, 0]], dtype=float)
    t5 = 0.8 * t3
    K = np.kron(t1, np.kron(t2, t2)) + np.kron(t3, np.kron(t4, t4)) + np.kron(t5, np.kron(t4, t4))
    init = [np.stack([t2, t4]), np.stack([t2, t4]), np.stack([t1, t3])]
    return K, (2, 2, 4), (2, 2, 3), init


def kron_matrix(factors):
    """sum_r F_{D-1,r} x .. x F_{0,r} from factors[d] of shape [rank, m_d, n_d]."""
    D = len(factors)
    out = 0
    for r in range(factors[0].shape[0]):
        t = np.ones((1, 1))
        for d in reversed(range(D)):
            t = np.kron(t, factors[d][r])
        out = out + t
    return out


def kcp_als(K, m, n, init, iters):
    """ALS sweeps from the initial factors init[d] ([rank, m_d, n_d]); returns the factors."""
    D = len(m)
    T = reshuffle(np.asarray(K, dtype=np.float64), m, n)
    F = [np.array(f, dtype=np.float64).reshape(f.shape[0], -1).T.copy() for f in init]  # [m_d n_d, rank]
    R = F[0].shape[1]
    for _ in range(iters):
        for d in range(D):
            others = [e for e in range(D) if e != d]
            V = np.ones((R, R))
            for e in others:
                V = V * (F[e].T @ F[e])
            # G(a_d, r) = sum_{others} T(a) prod_e F_e(a_e, r)
            G = np.zeros((F[d].shape[0], R))
            for r in range(R):
                t = np.moveaxis(T, d, 0)
                for e in reversed(others):
                    # contract the last remaining axis that corresponds to e
                    t = t @ F[e][:, r]
                G[:, r] = t
            if R == 2 and abs(np.linalg.det(V)) > 1e-14 * abs(V[0, 0] * V[1, 1]):
                Vi = np.linalg.inv(V)
            elif R == 1:
                Vi = np.array([[1.0 / V[0, 0] if V[0, 0] != 0 else 0.0]])
            else:
                Vi = np.diag([1.0 / V[i, i] if V[i, i] != 0 else 0.0 for i in range(R)])
            F[d] = G @ Vi
    return [F[d].T.reshape(R, m[d], n[d]) for d in range(D)]
