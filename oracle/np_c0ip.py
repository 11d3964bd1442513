"""C0 interior-penalty biharmonic problem on Cartesian meshes, numpy (TEST INFRASTRUCTURE ONLY).

Restates the reference's clamped C0IP formulation (apps/biharmonic_integrator.h: MW cell, face and
boundary workers 69-350; FD patch matrices 376-535) for FE_Q(k) with Lagrange basis on the
Gauss-Lobatto points, u = 0 strongly on the boundary nodes, the normal derivative weakly:

  a(u, v) = sum_K int_K D^2 u : D^2 v
          + sum_F int_F ( -{d_nn v}[d_n u] - {d_nn u}[d_n v] + sigma [d_n u][d_n v] )

with [w] = w_0 - w_1 and {w} = (w_0 + w_1)/2 on interior faces (n the normal of cell 0), the
one-sided values on boundary faces, sigma = ip gamma (1/h_0 + 1/h_1)/2 inside and 2 ip gamma / h
at the boundary, gamma = k(k+1) (Nitsche::compute_penalty_impl). On a Cartesian mesh
D^2u:D^2v = u_xx v_xx + 2 u_xy v_xy + u_yy v_yy and every face term is a 1-D term times a 1-D
mass, so the level matrix is  B (x) M + 2 L (x) L + M (x) B  with the 1-D FE_Q matrices
M (mass), L (int u'v') and B (int u''v'' plus the C0IP point terms). `matrix_2d_quadrature`
assembles the 2-D matrix directly by quadrature (cells and edges) to pin that separability.
Vectors: interior nodes of the (n k + 1)^2 node grid, lexicographic with x fastest.
"""
from __future__ import annotations

import itertools

import numpy as np
from numpy.polynomial import legendre as npleg

try:
    from .np_crosscheck import gll_nodes
except ImportError:
    from np_crosscheck import gll_nodes


class _Lag:
    """Lagrange basis function i on `nodes` (derivative order 0, 1 or 2) evaluated by the
    product rule over the factors (x - z_a) / (z_i - z_a) -- no monomial coefficients, which
    lose accuracy at high degree."""

    def __init__(self, nodes, i, order):
        self.z, self.i, self.order = nodes, i, order

    def __call__(self, x):
        x = np.asarray(x, dtype=np.float64)
        f, f1, f2 = np.ones_like(x), np.zeros_like(x), np.zeros_like(x)
        for a, za in enumerate(self.z):
            if a == self.i:
                continue
            d = 1.0 / (self.z[self.i] - za)
            f2 = f2 * (x - za) * d + 2.0 * f1 * d
            f1 = f1 * (x - za) * d + f * d
            f = f * (x - za) * d
        return (f, f1, f2)[self.order]


def basis_1d(k):
    """Lagrange basis on the k+1 GLL nodes of [0, 1] and its first and second derivatives, as
    callables."""
    nodes = gll_nodes(k)
    P = [_Lag(nodes, i, 0) for i in range(k + 1)]
    P1 = [_Lag(nodes, i, 1) for i in range(k + 1)]
    P2 = [_Lag(nodes, i, 2) for i in range(k + 1)]
    return nodes, P, P1, P2


def _ev(p, x):
    return p(x)


def matrices_1d(k, h, ip=1.0, keep_boundary=False):
    """Global 1-D FE_Q matrices (M, L, B) on cells of widths h (list); boundary nodes removed
    unless keep_boundary."""
    nc = len(h)
    n = nc * k + 1
    nodes, P, P1, P2 = basis_1d(k)
    qx, qw = npleg.leggauss(k + 1)
    qx, qw = 0.5 * (qx + 1.0), 0.5 * qw
    gamma = 1.0 if k == 0 else k * (k + 1.0)
    M, L, B = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    for c in range(nc):
        idx = np.arange(c * k, c * k + k + 1)
        hc = h[c]
        V = np.array([_ev(p, qx) for p in P])
        D1 = np.array([_ev(p, qx) for p in P1]) / hc
        D2 = np.array([_ev(p, qx) for p in P2]) / hc ** 2
        w = qw * hc
        M[np.ix_(idx, idx)] += (V * w) @ V.T
        L[np.ix_(idx, idx)] += (D1 * w) @ D1.T
        B[np.ix_(idx, idx)] += (D2 * w) @ D2.T

    def point_vals(c, side):
        """first and second derivatives of the cell's basis at its end `side` (0 left, 1 right)"""
        hc = h[c]
        d1 = np.array([_ev(p, float(side)) for p in P1]) / hc
        d2 = np.array([_ev(p, float(side)) for p in P2]) / hc ** 2
        return d1, d2

    # interior nodes between cell c (0) and c + 1 (1), normal +1
    for c in range(nc - 1):
        i0 = np.arange(c * k, c * k + k + 1)
        i1 = np.arange((c + 1) * k, (c + 1) * k + k + 1)
        d1a, d2a = point_vals(c, 1)
        d1b, d2b = point_vals(c + 1, 0)
        idx = np.concatenate([i0, i1])
        jump = np.concatenate([d1a, -d1b])          # [d_n u]
        avg = 0.5 * np.concatenate([d2a, d2b])      # {d_nn u}
        sig = ip * gamma * (1.0 / h[c] + 1.0 / h[c + 1]) / 2.0
        blk = -np.outer(avg, jump) - np.outer(jump, avg) + sig * np.outer(jump, jump)
        for a, ia in enumerate(idx):
            for b, ib in enumerate(idx):
                B[ia, ib] += blk[a, b]
    # boundary nodes: one-sided, outward normal
    for c, side, nrm in ((0, 0, -1.0), (nc - 1, 1, 1.0)):
        idx = np.arange(c * k, c * k + k + 1)
        d1, d2 = point_vals(c, side)
        jump = nrm * d1
        avg = d2
        sig = ip * 2.0 * gamma / h[c]
        B[np.ix_(idx, idx)] += -np.outer(avg, jump) - np.outer(jump, avg) + sig * np.outer(jump, jump)
    if keep_boundary:
        return M, L, B
    s = slice(1, n - 1)
    return M[s, s], L[s, s], B[s, s]


def level_matrix(k, nc, ip=1.0, problem="c0ip"):
    """2-D C0IP matrix on the unit square, nc x nc cells (Kronecker form); problem "poisson": the
    Laplacian of continuous FE_Q(k), M x L + L x M."""
    h = [1.0 / nc] * nc
    M, L, B = matrices_1d(k, h, ip)
    if problem == "poisson":
        return np.kron(M, L) + np.kron(L, M)
    return np.kron(M, B) + 2.0 * np.kron(L, L) + np.kron(B, M)


def poisson_q_matrix_quadrature(k, nc):
    """The FE_Q(k) Laplacian on the unit square by plain 2-D quadrature over the cells (interior
    nodes, x fastest) -- independent of the Kronecker form."""
    h = 1.0 / nc
    nodes, P, P1, _ = basis_1d(k)
    qx, qw = npleg.leggauss(k + 1)
    qx, qw = 0.5 * (qx + 1.0), 0.5 * qw
    V = np.array([[p(x) for x in qx] for p in P])
    D = np.array([[p(x) for x in qx] for p in P1]) / h
    ng = nc * k + 1
    A = np.zeros((ng * ng, ng * ng))
    for cy in range(nc):
        for cx in range(nc):
            ii = np.array([(cy * k + b) * ng + cx * k + a for b in range(k + 1) for a in range(k + 1)])
            Kc = np.zeros((len(ii), len(ii)))
            for qy in range(k + 1):
                for qxi in range(k + 1):
                    w = qw[qy] * qw[qxi] * h * h
                    gx = np.array([D[a, qxi] * V[b, qy] for b in range(k + 1) for a in range(k + 1)])
                    gy = np.array([V[a, qxi] * D[b, qy] for b in range(k + 1) for a in range(k + 1)])
                    Kc += w * (np.outer(gx, gx) + np.outer(gy, gy))
            A[np.ix_(ii, ii)] += Kc
    inner = [j * ng + i for j in range(1, ng - 1) for i in range(1, ng - 1)]
    return A[np.ix_(inner, inner)]


def matrix_2d_quadrature(k, nc, ip=1.0):
    """The same 2-D matrix assembled by plain quadrature over cells and edges (independent of
    the separability argument)."""
    h = 1.0 / nc
    nodes, P, P1, P2 = basis_1d(k)
    qx, qw = npleg.leggauss(k + 1)
    qx, qw = 0.5 * (qx + 1.0), 0.5 * qw
    gamma = 1.0 if k == 0 else k * (k + 1.0)
    ng = nc * k + 1
    A = np.zeros((ng * ng, ng * ng))

    def cell_dofs(cx, cy):
        return [(cy * k + j) * ng + cx * k + i for j in range(k + 1) for i in range(k + 1)]

    def derivs(x, y):
        """value, gradient, Hessian of the (k+1)^2 cell basis functions at reference (x, y)"""
        vx = np.array([_ev(p, x) for p in P]); vy = np.array([_ev(p, y) for p in P])
        dx = np.array([_ev(p, x) for p in P1]) / h; dy = np.array([_ev(p, y) for p in P1]) / h
        ddx = np.array([_ev(p, x) for p in P2]) / h ** 2; ddy = np.array([_ev(p, y) for p in P2]) / h ** 2
        g = np.zeros(((k + 1) ** 2, 2)); H = np.zeros(((k + 1) ** 2, 2, 2))
        a = 0
        for j in range(k + 1):
            for i in range(k + 1):
                g[a] = [dx[i] * vy[j], vx[i] * dy[j]]
                H[a] = [[ddx[i] * vy[j], dx[i] * dy[j]], [dx[i] * dy[j], vx[i] * ddy[j]]]
                a += 1
        return g, H

    for cy in range(nc):
        for cx in range(nc):
            d = cell_dofs(cx, cy)
            for qa, qb in itertools.product(range(k + 1), repeat=2):
                _, H = derivs(qx[qa], qx[qb])
                w = qw[qa] * qw[qb] * h * h
                Hf = H.reshape(len(d), 4)
                A[np.ix_(d, d)] += w * Hf @ Hf.T
    # edges: normal direction e (0: x, 1: y)
    for e in range(2):
        for cy in range(nc):
            for cx in range(nc):
                c = [cx, cy]
                for side in (0, 1):
                    nb = list(c)
                    nb[e] += 1 if side else -1
                    boundary = nb[e] < 0 or nb[e] >= nc
                    if not boundary and side == 0:
                        continue  # interior edges once, from the lower cell
                    nrm = np.zeros(2); nrm[e] = 1.0 if side else -1.0
                    for q in range(k + 1):
                        t = qx[q]
                        pt = [t, t]; pt[e] = float(side)
                        g0, H0 = derivs(*pt)
                        w = qw[q] * h
                        d0 = cell_dofs(*c)
                        if boundary:
                            jump = g0 @ nrm
                            avg = np.einsum("aij,i,j->a", H0, nrm, nrm)
                            sig = ip * 2.0 * gamma / h
                            idx = d0
                        else:
                            pn = [t, t]; pn[e] = 0.0
                            g1, H1 = derivs(*pn)
                            d1 = cell_dofs(*nb)
                            jump = np.concatenate([g0 @ nrm, -(g1 @ nrm)])
                            avg = 0.5 * np.concatenate([np.einsum("aij,i,j->a", H0, nrm, nrm),
                                                        np.einsum("aij,i,j->a", H1, nrm, nrm)])
                            sig = ip * gamma * (2.0 / h) / 2.0
                            idx = d0 + d1
                        blk = w * (-np.outer(avg, jump) - np.outer(jump, avg) + sig * np.outer(jump, jump))
                        ii = np.array(idx)
                        np.add.at(A, (ii[:, None], ii[None, :]), blk)
    inner = [j * ng + i for j in range(1, ng - 1) for i in range(1, ng - 1)]
    return A[np.ix_(inner, inner)]


def patch_indices(k, nc, vx, vy):
    """Interior-node indices (level numbering) of the vertex patch around interior vertex
    (vx, vy), 1 <= vx, vy <= nc-1: (2k-1)^2 nodes, x fastest."""
    n = nc * k - 1
    x0, y0 = (vx - 1) * k, (vy - 1) * k
    return np.array([(y0 + b) * n + x0 + a for b in range(2 * k - 1) for a in range(2 * k - 1)])


def patches(nc):
    """Interior vertices in the smoother's order: colors (vx % 2, vy % 2) -> 0..3, lexicographic
    inside a color."""
    out = []
    for color in range(4):
        for vy in range(1, nc):
            for vx in range(1, nc):
                if (vx % 2) + 2 * (vy % 2) == color:
                    out.append((vx, vy, color))
    return out


def schwarz_vmult(k, nc, src, omega, local="exact", ip=1.0, problem="c0ip"):
    """Additive vertex-patch Schwarz: sum_j omega R_j^T A_j^-1 R_j src with the exact patch
    matrices (local = "exact", LocalSolverVariant::Exact) or their Kronecker sum without the
    mixed-derivative term B (x) M + M (x) B (local = "bilaplacian", solved by fast
    diagonalization in the product). problem "poisson": the FE_Q Laplacian, whose patch matrix
    is the Kronecker sum M x L + L x M of the restricted 1-D matrices (both locals coincide)."""
    A = level_matrix(k, nc, ip, problem)
    h = [1.0 / nc] * nc
    M, L, B = matrices_1d(k, h, ip)
    if problem == "poisson":
        B = L
    out = np.zeros_like(src)
    m = 2 * k - 1
    for vx, vy, _ in patches(nc):
        idx = patch_indices(k, nc, vx, vy)
        if local == "exact":
            K = A[np.ix_(idx, idx)]
        else:
            sx = slice((vx - 1) * k, (vx - 1) * k + m)
            sy = slice((vy - 1) * k, (vy - 1) * k + m)
            K = np.kron(M[sy, sy], B[sx, sx]) + np.kron(B[sy, sy], M[sx, sx])
        out[idx] += omega * np.linalg.solve(K, src[idx])
    return out


def embedding_1d(k):
    """Values of the coarse basis at the fine nodes of the two children: E[s][i, j] =
    phi_j((z_i + s) / 2)."""
    nodes, P, _, _ = basis_1d(k)
    return [np.array([[_ev(P[j], (z + s) / 2.0) for j in range(k + 1)] for z in nodes]) for s in (0, 1)]


def prolongation_1d(k, nc_coarse):
    """Interior-to-interior prolongation of continuous Q_k from nc to 2 nc cells (1-D)."""
    E = embedding_1d(k)
    nfc, ncc = 2 * nc_coarse * k + 1, nc_coarse * k + 1
    Pm = np.zeros((nfc, ncc))
    for c in range(nc_coarse):
        for s in (0, 1):
            fine = np.arange((2 * c + s) * k, (2 * c + s) * k + k + 1)
            coarse = np.arange(c * k, c * k + k + 1)
            Pm[np.ix_(fine, coarse)] = E[s]  # continuous: shared nodes get the same value
    return Pm[1:-1, 1:-1]


def mg_cg_solve(k, n_rep, nc_fine, f, omega, local="exact", rel_tol=1e-8, abs_tol=1e-14,
                max_iter=200, ip=1.0, problem="c0ip"):
    """CG + V-cycle (one pre-/post-step of the additive patch smoother, exact coarse solve)."""
    nl, n = 0, n_rep
    while n <= nc_fine:
        nl += 1
        n *= 2
    ncs = [n_rep << l for l in range(nl)]
    A = [level_matrix(k, c, ip, problem) for c in ncs]
    P = [None] + [np.kron(prolongation_1d(k, ncs[l - 1]), prolongation_1d(k, ncs[l - 1])) for l in range(1, nl)]
    A0inv = np.linalg.inv(A[0])

    def vcycle(l, b):
        if l == 0:
            return A0inv @ b
        x = schwarz_vmult(k, ncs[l], b, omega, local, ip, problem)
        bc = P[l].T @ (b - A[l] @ x)
        x = x + P[l] @ vcycle(l - 1, bc)
        return x + schwarz_vmult(k, ncs[l], b - A[l] @ x, omega, local, ip, problem)

    u = np.zeros_like(f)
    r = f.copy()
    res = np.linalg.norm(r)
    hist = [res]
    tol = max(abs_tol, rel_tol * res)
    z = vcycle(nl - 1, r)
    p = z.copy()
    rz = r @ z
    for it in range(1, max_iter + 1):
        Ap = A[-1] @ p
        alpha = rz / (p @ Ap)
        u += alpha * p
        r -= alpha * Ap
        res = np.linalg.norm(r)
        hist.append(res)
        if res <= tol:
            return it, np.array(hist), u
        z = vcycle(nl - 1, r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return -1, np.array(hist), u
