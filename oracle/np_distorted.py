"""SIPG level matrix on multilinear (bi-/trilinear) meshes, numpy (TEST INFRASTRUCTURE ONLY).

Independent restatement of the reference's matrix-free operator on a general mesh
(apps/laplace_integrator.h:613-743) by plain quadrature, for small meshes:

- cell term  int grad u . grad v  with the multilinear map x(xi) of each cell, Gauss rule
  with k+1 points per direction;
- interior faces  int sigma [u][v] - {d_n u}[v] - [u]{d_n v}, normal pointing out of the
  cell that owns the test function, sigma = ip * gamma * (1/h_in + 1/h_out) / 2;
- Dirichlet boundary faces  int sigma u v - d_n u v - u d_n v, sigma = 2 * ip * gamma / h;
- gamma = k(k+1) (apps/common_integrator.h:30-37), and the face length h of each side is
  1 / |n . grad xi_normal| at the face's FIRST quadrature point, as the reference computes
  it from `normal * inverse_jacobian(0)` (laplace_integrator.h:649-652, 690-691).

Vertex coordinates are given lexicographically (x fastest) as [(n_0+1)...(n_{d-1}+1), d].
The DoFs of a cell are consecutive (FE_DGQ, Lagrange on Gauss-Lobatto nodes, direction 0
fastest) and cells are numbered lexicographically, as in the Cartesian oracle.
"""
from __future__ import annotations

import itertools

import numpy as np
from numpy.polynomial import legendre as npleg

try:
    from .np_crosscheck import gll_nodes, lagrange
    from . import oracle as _oracle
except ImportError:  # imported from inside the oracle folder
    from np_crosscheck import gll_nodes, lagrange
    import oracle as _oracle


def _vertex(X, dim, nc, v):
    nv = [n + 1 for n in nc]
    idx = v[0] + nv[0] * (v[1] + (nv[1] * v[2] if dim > 2 else 0)) if dim > 1 else v[0]
    return X[idx]


def cell_vertices(X, dim, nc, c):
    """The 2^dim vertices of cell c, ordered with bit d = upper in direction d."""
    out = np.zeros((2 ** dim, dim))
    for b in range(2 ** dim):
        v = [c[d] + ((b >> d) & 1) for d in range(dim)]
        out[b] = _vertex(X, dim, nc, v)
    return out


def jacobian(V, xi):
    """Jacobian J[i, j] = d x_i / d xi_j of the multilinear map with vertices V at xi."""
    dim = V.shape[1]
    J = np.zeros((dim, dim))
    for b in range(2 ** dim):
        for j in range(dim):
            t = 1.0
            for e in range(dim):
                up = (b >> e) & 1
                if e == j:
                    t *= 1.0 if up else -1.0
                else:
                    t *= xi[e] if up else 1.0 - xi[e]
            J[:, j] += t * V[b]
    return J


class _Basis:
    def __init__(self, dim, k):
        self.dim, self.k, self.npt = dim, k, k + 1
        nodes = gll_nodes(k)
        qx, qw = npleg.leggauss(k + 1)
        self.qx, self.qw = 0.5 * (qx + 1.0), 0.5 * qw
        self.V, self.D = lagrange(nodes, self.qx)  # [i, q]
        self.F, self.FD = lagrange(nodes, np.array([0.0, 1.0]))  # [i, side]
        self.nd = self.npt ** dim
        # multi-index of every cell DoF, direction 0 fastest
        self.I = np.array([[(a // self.npt ** d) % self.npt for d in range(dim)] for a in range(self.nd)])

    def ref_grad(self, pts):
        """values [nd] and reference gradients [nd, dim] at a point given per direction as
        ('q', index) for a Gauss point or ('f', side) for a face coordinate."""
        dim = self.dim
        val1, der1 = [], []
        for d in range(dim):
            kind, i = pts[d]
            if kind == "q":
                val1.append(self.V[:, i])
                der1.append(self.D[:, i])
            else:
                val1.append(self.F[:, i])
                der1.append(self.FD[:, i])
        val = np.ones(self.nd)
        for d in range(dim):
            val = val * val1[d][self.I[:, d]]
        grad = np.ones((self.nd, dim))
        for g in range(dim):
            for d in range(dim):
                grad[:, g] *= (der1[d] if d == g else val1[d])[self.I[:, d]]
        return val, grad

    def xi(self, pts):
        return np.array([self.qx[i] if kind == "q" else float(i) for kind, i in pts])


def _cell_index(dim, nc, c):
    lex = c[0]
    if dim > 1:
        lex += nc[0] * c[1]
    if dim > 2:
        lex += nc[0] * nc[1] * c[2]
    return lex


def sipg_matrix_mapped(dim, k, nc, X, ip=1.0):
    """Dense global SIPG matrix on the multilinear mesh with vertex coordinates X."""
    nc = list(nc)
    B = _Basis(dim, k)
    nd = B.nd
    gamma = 1.0 if k == 0 else k * (k + 1.0)
    ncell = int(np.prod(nc))
    A = np.zeros((ncell * nd, ncell * nd))

    def dofs(c):
        lex = _cell_index(dim, nc, c)
        return np.arange(lex * nd, (lex + 1) * nd)

    def face_points(d, side):
        tdirs = [e for e in range(dim) if e != d]
        for tq in itertools.product(range(B.npt), repeat=dim - 1):
            tq = tq[::-1]  # first tangential direction fastest
            pts = [None] * dim
            pts[d] = ("f", side)
            w = 1.0
            for j, e in enumerate(tdirs):
                pts[e] = ("q", tq[j])
                w *= B.qw[tq[j]]
            yield pts, w

    for c in itertools.product(*[range(n) for n in nc[::-1]]):
        c = list(c[::-1])
        Vc = cell_vertices(X, dim, nc, c)
        dc = dofs(c)
        # cell term
        K = np.zeros((nd, nd))
        for q in itertools.product(range(B.npt), repeat=dim):
            pts = [("q", i) for i in q]
            w = np.prod([B.qw[i] for i in q])
            J = jacobian(Vc, B.xi(pts))
            Ji = np.linalg.inv(J)
            _, g = B.ref_grad(pts)
            pg = g @ Ji  # physical gradients: grad phi = J^-T ghat -> row form ghat^T J^-1
            K += w * abs(np.linalg.det(J)) * pg @ pg.T
        A[np.ix_(dc, dc)] += K
        # faces, seen from this cell (outward normal)
        for d in range(dim):
            for side in (0, 1):
                nb = list(c)
                nb[d] += 1 if side else -1
                boundary = nb[d] < 0 or nb[d] >= nc[d]
                sgn = 1.0 if side else -1.0
                vals, dns, wts = [], [], []
                nbvals, nbdns = [], []
                h_c = h_nb = None
                if not boundary:
                    Vn = cell_vertices(X, dim, nc, nb)
                for qi, (pts, w) in enumerate(face_points(d, side)):
                    J = jacobian(Vc, B.xi(pts))
                    Ji = np.linalg.inv(J)
                    gxi = Ji[d, :]  # grad of xi_d
                    ng = np.linalg.norm(gxi)
                    n = sgn * gxi / ng
                    v, g = B.ref_grad(pts)
                    vals.append(v)
                    dns.append(g @ (Ji @ n))
                    wts.append(w * abs(np.linalg.det(J)) * ng)
                    if qi == 0:
                        h_c = 1.0 / abs(n @ gxi)
                    if not boundary:
                        pn = list(pts)
                        pn[d] = ("f", 1 - side)
                        Jn = jacobian(Vn, B.xi(pn))
                        Jni = np.linalg.inv(Jn)
                        vn, gn = B.ref_grad(pn)
                        nbvals.append(vn)
                        nbdns.append(gn @ (Jni @ n))
                        if qi == 0:
                            h_nb = 1.0 / abs(n @ Jni[d, :])
                vals, dns, wts = np.array(vals).T, np.array(dns).T, np.array(wts)
                if boundary:
                    sig = ip * 2.0 * gamma / h_c
                    A[np.ix_(dc, dc)] += (sig * vals * wts) @ vals.T - (vals * wts) @ dns.T - (dns * wts) @ vals.T
                else:
                    sig = ip * gamma * (1.0 / h_c + 1.0 / h_nb) / 2.0
                    nbvals, nbdns = np.array(nbvals).T, np.array(nbdns).T
                    # test in this cell: [v] = v, {d_n v} = d_n v / 2
                    A[np.ix_(dc, dc)] += (sig * vals * wts) @ vals.T - 0.5 * (vals * wts) @ dns.T \
                        - 0.5 * (dns * wts) @ vals.T
                    dn_ = dofs(nb)
                    # trial in the neighbour: [u] = -u, {d_n u} = d_n u / 2
                    A[np.ix_(dc, dn_)] += -(sig * vals * wts) @ nbvals.T - 0.5 * (vals * wts) @ nbdns.T \
                        + 0.5 * (dns * wts) @ nbvals.T
    return A


def cartesian_coords(dim, nc):
    nv = [n + 1 for n in nc]
    grids = np.meshgrid(*[np.arange(n) / (n - 1) for n in reversed(nv)], indexing="ij")
    return np.ascontiguousarray(np.stack([grids[dim - 1 - d] for d in range(dim)], axis=-1).reshape(-1, dim))


def coarsen_coords(dim, nc, X):
    """Vertex coordinates of the next coarser level: every second vertex per direction."""
    nv = [n + 1 for n in nc]
    G = X.reshape(list(reversed(nv)) + [dim])
    sl = tuple(slice(None, None, 2) for _ in range(dim))
    return np.ascontiguousarray(G[sl].reshape(-1, dim))


def level_coords(dim, nc_fine, X, levels_down):
    """Vertices of the level `levels_down` coarsenings below the finest one."""
    nc = [nc_fine] * dim
    for _ in range(levels_down):
        X = coarsen_coords(dim, nc, X)
        nc = [n // 2 for n in nc]
    return X


def lcg_start(n):
    """The power iteration's start vector: 64-bit LCG (Knuth MMIX constants), seed 0x5eed,
    top 53 bits as a uniform in [0,1), minus 0.5."""
    out = np.zeros(n)
    st = 0x5EED
    M = (1 << 64) - 1
    for i in range(n):
        st = (st * 6364136223846793005 + 1442695040888963407) & M
        out[i] = (st >> 11) * (1.0 / 9007199254740992.0) - 0.5
    return out


def scaled_relaxation(A, smooth1, omega, dim, steps=30):
    """omega * 2^dim / (1.05 lambda) if smaller than omega, lambda = Rayleigh-quotient power
    estimate of lambda_max(P A) (P = undamped smoother)."""
    x = lcg_start(A.shape[0])
    lam = 0.0
    for _ in range(steps):
        t = A @ x
        r = smooth1(t)
        xt, tr, rr = x @ t, t @ r, r @ r
        if not (xt > 0 and rr > 0):
            break
        lam = tr / xt
        x = r / np.sqrt(rr)
    w = min(omega, omega * 2 ** dim / (1.05 * lam)) if lam > 0 else omega
    return w, lam


def mg_cg_solve_mapped(dim, k, n_rep, nc_fine, X, f, omega, rel_tol=1e-8, abs_tol=1e-14,
                       max_iter=100, ip=1.0, local="surrogate", auto_relaxation=False):
    """CG preconditioned by one V-cycle on a distorted hierarchy: dense mapped SIPG level
    matrices, DG embedding transfer, additive vertex-patch Schwarz smoother with surrogate-patch
    FD local solvers (one pre-, one post-step), dense exact coarse solve. Same V-cycle and
    ReductionControl semantics as the Cartesian oracle (apps/multigrid.h, poisson_problem.h:
    726-755). Returns (iterations, residual history, solution)."""
    o = _oracle
    nl = 0
    n = n_rep
    while n <= nc_fine:
        nl += 1
        n *= 2
    ncs = [n_rep << l for l in range(nl)]
    Xs = [level_coords(dim, nc_fine, X, nl - 1 - l) for l in range(nl)]
    A = [sipg_matrix_mapped(dim, k, [ncs[l]] * dim, Xs[l], ip) for l in range(nl)]
    hp = [None] + [o.surrogate_h(dim, [ncs[l]] * dim, Xs[l]) for l in range(1, nl)]
    Ainv0 = np.linalg.inv(A[0])

    inv = [None] * nl
    if local != "surrogate":
        try:
            from .np_crosscheck import patch_dofs
        except ImportError:
            from np_crosscheck import patch_dofs
        for l in range(1, nl):
            inv[l] = []
            for lo, MA, _, _ in patch_problems(dim, k, [ncs[l]] * dim, Xs[l], ip):
                idx = patch_dofs(dim, k, [ncs[l]] * dim, lo, 2)
                K = A[l][np.ix_(idx, idx)]
                if local == "exact":
                    inv[l].append((idx, np.linalg.inv(K)))
                else:
                    Ms = [m for m, _ in MA]
                    Af = keep_definite(Ms, ksum_fit_closed(K, Ms), [a for _, a in MA])
                    inv[l].append((idx, fd_inverse(Ms, Af)))

    omegas = [omega] * nl

    def smooth(l, r, w=None):
        w = omegas[l] if w is None else w
        if local == "surrogate":
            return o.schwarz_vmult_surrogate(dim, k, [ncs[l]] * dim, hp[l], r, omega=w, ip=ip)
        out = np.zeros_like(r)
        for idx, Pinv in inv[l]:
            out[idx] += w * (Pinv @ r[idx])
        return out

    if auto_relaxation:
        for l in range(1, nl):
            omegas[l], _ = scaled_relaxation(A[l], lambda v, l=l: smooth(l, v, 1.0), omega, dim)
    mg_cg_solve_mapped.last_omegas = list(omegas)

    def vcycle(l, b):
        if l == 0:
            return Ainv0 @ b
        x = smooth(l, b)
        t = b - A[l] @ x
        bc = o.restrict_add(dim, k, [ncs[l - 1]] * dim, np.zeros(A[l - 1].shape[0]), t)
        xc = vcycle(l - 1, bc)
        x = o.prolongate_add(dim, k, [ncs[l - 1]] * dim, xc, x)
        t = b - A[l] @ x
        return x + smooth(l, t)

    top = A[-1]
    u = np.zeros_like(f)
    r = f.copy()
    res = np.linalg.norm(r)
    hist = [res]
    tol = max(abs_tol, rel_tol * res)
    if res <= tol:
        return 0, np.array(hist), u
    z = vcycle(nl - 1, r)
    p = z.copy()
    rz = r @ z
    for it in range(1, max_iter + 1):
        Ap = top @ p
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


# --------------------------------------------------------------------------------------
# Separable approximations of exact patch matrices and the learned-solver data
# --------------------------------------------------------------------------------------
def kron_dirs(mats):
    """Kronecker product with mats[0] as the rightmost factor (direction 0 fastest)."""
    K = mats[-1]
    for m in reversed(mats[:-1]):
        K = np.kron(K, m)
    return K


def ksum_fit_lstsq(K, Ms):
    """Least-squares Kronecker sum sum_d (M x .. x A_d x .. x M) ~ K for fixed masses, by
    numpy lstsq on the explicit basis (minimum-norm solution), returned as the sum's
    1-D matrices after the even split of the mass shifts."""
    dim, n = len(Ms), Ms[0].shape[0]
    cols = []
    for d in range(dim):
        for i in range(n):
            for j in range(n):
                E = np.zeros((n, n))
                E[i, j] = 1.0
                cols.append(kron_dirs([Ms[e] if e != d else E for e in range(dim)]).reshape(-1))
    x = np.linalg.lstsq(np.array(cols).T, K.reshape(-1), rcond=None)[0]
    A = [x[d * n * n:(d + 1) * n * n].reshape(n, n) for d in range(dim)]
    # normalise the free shifts A_d + a_d M_d (sum a_d = 0): make <A_d, M_d> c_d equal for all d
    mu = [np.sum(M * M) for M in Ms]
    P = np.prod(mu)
    t = [np.sum(A[d] * Ms[d]) * P / mu[d] for d in range(dim)]  # c_d <A_d, M_d>
    S = sum(t)
    for d in range(dim):
        A[d] = A[d] + (S / dim - t[d]) / P * Ms[d]
    return [(a + a.T) / 2 for a in A]


def surrogate_problem(k, hp_pd, lo, hi, ip=1.0):
    M, A = _oracle.patch_matrices_1d(k, hp_pd, lo, hi, ip)
    return M, A


def patch_problems(dim, k, nc, X, ip=1.0):
    """Per interior-vertex patch: lower cell, surrogate (M_d, A_d) and boundary flags."""
    lower, _, _ = _oracle.patches(dim, list(nc), 1)
    hp = _oracle.surrogate_h(dim, list(nc), X)
    out = []
    for p, lo in enumerate(lower):
        MA, flags = [], []
        for d in range(dim):
            blo, bhi = lo[d] == 0, lo[d] + 2 == nc[d]
            MA.append(surrogate_problem(k, hp[p, d], blo, bhi, ip))
            flags += [float(blo), float(bhi)]
        out.append((lo[:dim].copy(), MA, flags, hp[p]))
    return out


def fd_inverse(Ms, As):
    """Dense S Lambda^-1 S^T of the Kronecker sum of (M_d, A_d)."""
    import scipy.linalg as sl
    dim, n = len(Ms), Ms[0].shape[0]
    S, lam = [], np.zeros([n] * dim)
    for d in range(dim):
        l, s = sl.eigh(As[d], Ms[d])
        S.append(s)
        sh = [1] * dim
        sh[dim - 1 - d] = n
        lam = lam + l.reshape(sh)
    Sk = kron_dirs(S)
    return Sk @ np.diag(1.0 / lam.reshape(-1)) @ Sk.T


def learned_features(dim, nc, X, problems):
    """Network inputs: vertex displacements from the lattice around the centre vertex,
    coordinate d in units of the patch's mean surrogate width in direction d, then the
    boundary flags."""
    nv = [n + 1 for n in nc] + [1] * (3 - dim)
    out = []
    for lo, _, flags, hp in problems:
        hbar = 0.5 * (hp[:, 0] + hp[:, 1])
        c = [lo[d] + 1 for d in range(dim)] + [0] * (3 - dim)
        vid = lambda v: v[0] + nv[0] * (v[1] + nv[1] * v[2])
        xc = X[vid(c)]
        f = []
        for v in range(3 ** dim):
            off = [(v // 3 ** d) % 3 - 1 for d in range(dim)] + [0] * (3 - dim)
            xv = X[vid([c[d] + off[d] for d in range(3)])]
            f += list((xv - xc) / hbar - np.array(off[:dim]))
        out.append(f + flags)
    return np.array(out)


def learned_targets(dim, k, nc, A_level, problems):
    """Upper triangles of D^-1/2 (A_fit - A_sur) D^-1/2, D = diag(A_sur), per direction."""
    try:
        from .np_crosscheck import patch_dofs
    except ImportError:
        from np_crosscheck import patch_dofs
    rows = []
    for lo, MA, _, _ in problems:
        idx = patch_dofs(dim, k, list(nc), lo, 2)
        K = A_level[np.ix_(idx, idx)]
        Ms = [m for m, _ in MA]
        Af = ksum_fit_lstsq(K, Ms)
        t = []
        for d in range(dim):
            A = MA[d][1]
            dg = np.sqrt(np.diag(A))
            H = (Af[d] - A) / np.outer(dg, dg)
            t += list(H[np.triu_indices(A.shape[0])])
        rows.append(t)
    return np.array(rows)


def ksum_fit_closed(K, Ms):
    """The same fit in closed form: R_d = contraction of K with every mass but M_d,
    A_d = R_d / c_d - (D-1)/D <K, M x..x M> / prod mu * M_d (c_d = prod_{e != d} mu_e)."""
    dim, n = len(Ms), Ms[0].shape[0]
    T = K.reshape([n] * (2 * dim))  # axes: rows (dir D-1 ... 0), cols (dir D-1 ... 0)
    mu = [np.sum(M * M) for M in Ms]
    P = np.prod(mu)
    letters_r = "abc"[:dim]
    letters_c = "xyz"[:dim]
    A = []
    full = np.einsum(f"{letters_r}{letters_c}," + ",".join(
        f"{letters_r[dim - 1 - e]}{letters_c[dim - 1 - e]}" for e in range(dim)) + "->",
        T, *Ms)
    for d in range(dim):
        others = [e for e in range(dim) if e != d]
        spec = f"{letters_r}{letters_c}," + ",".join(
            f"{letters_r[dim - 1 - e]}{letters_c[dim - 1 - e]}" for e in others)
        out = f"->{letters_r[dim - 1 - d]}{letters_c[dim - 1 - d]}"
        R = np.einsum(spec + out, T, *[Ms[e] for e in others])
        cd = P / mu[d]
        Ad = R / cd - (dim - 1) / dim * full / P * Ms[d]
        A.append((Ad + Ad.T) / 2)
    return A


def keep_definite(Ms, A_new, A_sur):
    """The fitted 1-D problems if the smallest eigenvalue of their Kronecker sum is at least
    half of the surrogate's, else the surrogate problems (the product's fallback rule)."""
    import scipy.linalg as sl
    snew = sum(sl.eigh(A_new[d], Ms[d], eigvals_only=True).min() for d in range(len(Ms)))
    ssur = sum(sl.eigh(A_sur[d], Ms[d], eigvals_only=True).min() for d in range(len(Ms)))
    return A_new if (np.isfinite(snew) and snew >= 0.5 * ssur) else A_sur
