"""Independent numpy restatement used to validate the C oracle (TEST INFRASTRUCTURE ONLY).

It assembles the DG SIPG level matrix of a small structured mesh by plain d-dimensional
quadrature -- cell and face loops, no Kronecker structure -- following the reference's
matrix-free operator (apps/laplace_integrator.h:613-743: cell gradient term, interior faces
with sigma = ip * gamma * (1/h_in + 1/h_out) / 2, Dirichlet boundary faces with
sigma = 2 * ip * gamma / h, gamma = k(k+1), apps/common_integrator.h:30-37), with FE_DGQ(k)
shape functions (Lagrange on Gauss-Lobatto nodes, lexicographic, direction 0 fastest).
Patch solves are then dense solves on submatrices, i.e. the Schwarz preconditioner in its
definition sum_j omega R_j^T (R_j A R_j^T)^-1 R_j (schwarz_preconditioner.h:194-225).
"""
from __future__ import annotations

import itertools

import numpy as np
from numpy.polynomial import legendre as npleg


def gll_nodes(k):
    if k == 0:
        return np.array([0.5])
    interior = npleg.Legendre.basis(k).deriv().roots()
    z = np.concatenate([[-1.0], np.sort(np.real(interior)), [1.0]])
    return 0.5 * (z + 1.0)


def lagrange(nodes, x):
    """values [i, len(x)] and derivatives of the Lagrange basis on `nodes` at points x."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    n = len(nodes)
    val = np.ones((n, len(x)))
    der = np.zeros((n, len(x)))
    for i in range(n):
        for j in range(n):
            if j != i:
                val[i] *= (x - nodes[j]) / (nodes[i] - nodes[j])
        for l in range(n):
            if l == i:
                continue
            t = np.full(len(x), 1.0 / (nodes[i] - nodes[l]))
            for j in range(n):
                if j != i and j != l:
                    t *= (x - nodes[j]) / (nodes[i] - nodes[j])
            der[i] += t
    return val, der


def _cell_dofs(dim, k, nc, c):
    nd = (k + 1) ** dim
    lex = c[0] + nc[0] * ((c[1] if dim > 1 else 0) + (nc[1] if dim > 1 else 1) * (c[2] if dim > 2 else 0))
    return np.arange(lex * nd, (lex + 1) * nd)


def sipg_matrix(dim, k, nc, ip=1.0, h=None, penalty="reference"):
    """Dense global SIPG matrix on [0,1]^dim with nc cells per direction (DoFs cell-wise).

    penalty "reference": sigma = ip k(k+1) (1/h_l + 1/h_r)/2 inside, 2 ip k(k+1)/h on the
    boundary; "kp1sq": sigma = ip 2(k+1)^2 (1/h_l + 1/h_r)/2 inside, ip 2(k+1)^2/h on the
    boundary (2(k+1)^2/h on every face of a uniform mesh)."""
    nc = list(nc)
    if h is None:
        h = [np.full(nc[d], 1.0 / nc[d]) for d in range(dim)]
    npt = k + 1
    nodes = gll_nodes(k)
    qx, qw = npleg.leggauss(npt)
    qx, qw = 0.5 * (qx + 1.0), 0.5 * qw
    V, D = lagrange(nodes, qx)  # [i, q]
    F, FD = lagrange(nodes, np.array([0.0, 1.0]))  # [i, face]
    gamma = 1.0 if k == 0 else k * (k + 1.0)
    if penalty == "reference":
        def sig_bd(hb):
            return ip * 2.0 * gamma / hb

        def sig_in(hl, hr):
            return ip * gamma * (1.0 / hl + 1.0 / hr) / 2.0
    elif penalty == "kp1sq":
        def sig_bd(hb):
            return ip * 2.0 * (k + 1.0) ** 2 / hb

        def sig_in(hl, hr):
            return ip * 2.0 * (k + 1.0) ** 2 * (1.0 / hl + 1.0 / hr) / 2.0
    else:
        raise ValueError(penalty)
    ncell = int(np.prod(nc))
    N = ncell * npt ** dim
    A = np.zeros((N, N))
    multi = list(itertools.product(range(npt), repeat=dim))  # tuples (i_{d-1},...,i_0)
    # lexicographic: index = sum_d i_d npt^d, with i_0 fastest -> reverse tuples
    idx_tuples = [tuple(reversed(t)) for t in multi]
    order = np.argsort([sum(t[d] * npt ** d for d in range(dim)) for t in idx_tuples])
    idx_tuples = [idx_tuples[o] for o in order]
    qtuples = [tuple(reversed(t)) for t in itertools.product(range(npt), repeat=dim)]

    def cell_matrix(hc):
        nd = npt ** dim
        K = np.zeros((nd, nd))
        for q in qtuples:
            w = np.prod([qw[q[d]] * hc[d] for d in range(dim)])
            g = np.zeros((nd, dim))
            for a, I in enumerate(idx_tuples):
                for d in range(dim):
                    val = D[I[d], q[d]] / hc[d]
                    for e in range(dim):
                        if e != d:
                            val *= V[I[e], q[e]]
                    g[a, d] = val
            K += w * g @ g.T
        return K

    def face_vals(hc, d, side):
        """values and normal(+x_d) derivatives of all cell basis functions at the face
        quadrature points of face `side` (0 lower, 1 upper) in direction d."""
        nd = npt ** dim
        tq = [t for t in itertools.product(range(npt), repeat=dim - 1)]
        vals = np.zeros((nd, len(tq)))
        ders = np.zeros((nd, len(tq)))
        wts = np.zeros(len(tq))
        tdirs = [e for e in range(dim) if e != d]
        for p, tt in enumerate(tq):
            wts[p] = np.prod([qw[tt[j]] * hc[tdirs[j]] for j in range(dim - 1)]) if dim > 1 else 1.0
            for a, I in enumerate(idx_tuples):
                tv = np.prod([V[I[tdirs[j]], tt[j]] for j in range(dim - 1)]) if dim > 1 else 1.0
                vals[a, p] = F[I[d], side] * tv
                ders[a, p] = FD[I[d], side] / hc[d] * tv
        return vals, ders, wts

    for c in itertools.product(*[range(nc[d]) for d in range(dim)]):
        hc = [h[d][c[d]] for d in range(dim)]
        dofs = _cell_dofs(dim, k, nc + [1] * (3 - dim), list(c) + [0] * (3 - dim))
        A[np.ix_(dofs, dofs)] += cell_matrix(hc)
        for d in range(dim):
            # lower boundary face
            if c[d] == 0:
                v, dn, w = face_vals(hc, d, 0)
                dn = -dn  # outward normal -x_d
                sig = sig_bd(hc[d])
                A[np.ix_(dofs, dofs)] += (sig * v * w) @ v.T - (v * w) @ dn.T - (dn * w) @ v.T
            if c[d] == nc[d] - 1:
                v, dn, w = face_vals(hc, d, 1)
                sig = sig_bd(hc[d])
                A[np.ix_(dofs, dofs)] += (sig * v * w) @ v.T - (v * w) @ dn.T - (dn * w) @ v.T
            if c[d] + 1 < nc[d]:
                cr = list(c)
                cr[d] += 1
                hr = [h[e][cr[e]] for e in range(dim)]
                dofs_r = _cell_dofs(dim, k, nc + [1] * (3 - dim), cr + [0] * (3 - dim))
                vl, dl, w = face_vals(hc, d, 1)
                vr, dr, _ = face_vals(hr, d, 0)
                sig = sig_in(hc[d], hr[d])
                # jump [w] = w_l - w_r ; average {dn w} = (dl + dr)/2, normal +x_d
                J = np.vstack([vl, -vr])
                Av = 0.5 * np.vstack([dl, dr])
                blk = (sig * J * w) @ J.T - (J * w) @ Av.T - (Av * w) @ J.T
                both = np.concatenate([dofs, dofs_r])
                A[np.ix_(both, both)] += blk
    return A


def patch_dofs(dim, k, nc, lower, ncp):
    """Global DoF indices of a patch in patch-local lexicographic order (DG)."""
    npt = k + 1
    n = ncp * npt
    nloc = n ** dim
    out = np.zeros(nloc, dtype=np.int64)
    nc3 = list(nc) + [1] * (3 - dim)
    for loc in range(nloc):
        rem = loc
        cell = [0, 0, 0]
        e_multi = []
        for d in range(dim):
            pd = rem % n
            rem //= n
            cell[d] = lower[d] + pd // npt
            e_multi.append(pd % npt)
        e = sum(e_multi[d] * npt ** d for d in range(dim))
        out[loc] = _cell_dofs(dim, k, nc3, cell)[e]
    return out


def schwarz_vmult_dense(A, dim, k, nc, lowers, ncp, omega, src):
    dst = np.zeros_like(src)
    for lo in lowers:
        idx = patch_dofs(dim, k, nc, lo, ncp)
        Kj = A[np.ix_(idx, idx)]
        dst[idx] += omega * np.linalg.solve(Kj, src[idx])
    return dst


# --------------------------------------------------------------------------------------
# Smooth load vector of the reference's Poisson test problem: u = sum of three Gaussian
# bells (apps/equation_data.h:45-190, width 1/3), f = -Laplace(u), Nitsche boundary data
# g = u (apps/poisson_problem.h:442-520).  Used by the iteration-bound tests.
# --------------------------------------------------------------------------------------
_CENTERS = {2: np.array([[0.0, 0.0], [0.25, 0.85], [0.6, 0.4]]),
            3: np.array([[0.0, 0.0, 0.0], [0.25, 0.85, 0.85], [0.6, 0.4, 0.4]])}
_WIDTH = 1.0 / 3.0


def bells_value(X):
    dim = X.shape[-1]
    u0 = 1.0 / (np.sqrt(2 * np.pi) * _WIDTH) ** dim
    v0 = -1.0 / _WIDTH ** 2
    val = np.zeros(X.shape[:-1])
    for c in _CENTERS[dim]:
        val += u0 * np.exp(v0 * np.sum((X - c) ** 2, axis=-1))
    return val


def bells_rhs(X):
    dim = X.shape[-1]
    u0 = 1.0 / (np.sqrt(2 * np.pi) * _WIDTH) ** dim
    v0 = -1.0 / _WIDTH ** 2
    lap = np.zeros(X.shape[:-1])
    for c in _CENTERS[dim]:
        r2 = np.sum((X - c) ** 2, axis=-1)
        lap += u0 * 2.0 * v0 * np.exp(v0 * r2) * (dim + 2.0 * v0 * r2)
    return -lap


def bells_load_vector(dim, k, nc_per_dir, ip=1.0):
    """Load vector (cell-wise lexicographic DoFs) of the Gaussian-bell problem on a uniform
    mesh with nc_per_dir cells per direction."""
    n = nc_per_dir
    h = 1.0 / n
    npt = k + 1
    nodes = gll_nodes(k)
    qx, qw = npleg.leggauss(npt)
    qx, qw = 0.5 * (qx + 1.0), 0.5 * qw
    V, _ = lagrange(nodes, qx)                  # [i, q]
    F, FD = lagrange(nodes, np.array([0.0, 1.0]))
    gamma = 1.0 if k == 0 else k * (k + 1.0)
    x1 = (np.arange(n)[:, None] + qx[None, :]) * h   # [c, q]
    W = V * qw[None, :] * h                          # [i, q] weighted
    # axis order of grids: (c_{d-1}, q_{d-1}, ..., c_0, q_0)
    mesh = np.meshgrid(*([x1.reshape(-1)] * dim), indexing="ij")  # axis j <-> direction dim-1-j
    X = np.stack([mesh[dim - 1 - d] for d in range(dim)], axis=-1)
    f = bells_rhs(X).reshape([n, npt] * dim)
    if dim == 2:
        b = np.einsum("aqbr,iq,jr->abij", f, W, W)
    else:
        b = np.einsum("aqbrcs,iq,jr,ks->abcijk", f, W, W, W)
    # Nitsche boundary terms
    sigma = ip * 2.0 * gamma / h
    for d in range(dim):
        for side in (0, 1):
            coord = float(side)
            nrm = -1.0 if side == 0 else 1.0
            cb = 0 if side == 0 else n - 1
            tdirs = [e for e in range(dim) if e != d]
            # points on the face: tangential grids
            tm = np.meshgrid(*([x1.reshape(-1)] * (dim - 1)), indexing="ij")
            Xf = np.zeros(tm[0].shape + (dim,))
            for j, e in enumerate(reversed(tdirs)):
                Xf[..., e] = tm[j]
            Xf[..., d] = coord
            g = bells_value(Xf).reshape([n, npt] * (dim - 1))
            # normal-direction test factors: value and normal derivative
            vn = F[:, side]
            dn = nrm * FD[:, side] / h
            fac = sigma * vn - dn                    # [i_d]
            if dim == 2:
                e = tdirs[0]
                contrib = np.einsum("aq,iq,m->aim", g, W, fac)   # [c_e, i_e, i_d]
                for ce in range(n):
                    for ie in range(npt):
                        for idd in range(npt):
                            c = [0, 0]; i = [0, 0]
                            c[e] = ce; i[e] = ie; c[d] = cb; i[d] = idd
                            b[c[1], c[0], i[1], i[0]] += contrib[ce, ie, idd]
            else:
                e1, e0 = tdirs[1], tdirs[0]   # grid axis order (e1 slow, e0 fast)
                contrib = np.einsum("aqbr,iq,jr,m->abijm", g, W, W, fac)
                cidx = np.indices((n, n, npt, npt, npt)).reshape(5, -1)
                c = np.zeros((3, cidx.shape[1]), dtype=int)
                i = np.zeros((3, cidx.shape[1]), dtype=int)
                c[e1], c[e0], i[e1], i[e0], i[d] = cidx
                c[d] = cb
                np.add.at(b, (c[2], c[1], c[0], i[2], i[1], i[0]), contrib.reshape(-1))
    return b.reshape(-1)
