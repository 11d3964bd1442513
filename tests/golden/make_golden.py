"""Regenerates the golden fixtures in tests/golden from the CPU oracle.

    python tests/golden/make_golden.py            # small fixtures (seconds)
    python tests/golden/make_golden.py --large    # benchmark-size CG+MG histories (minutes)

The reference (jwitte08/TPSS) cannot be built here (it needs deal.II) and its tests draw
unseeded rand() values, so it ships no numeric vectors for this path.  These fixtures are
produced by the oracle after it has passed the reference's own relations (tests/test_oracle.py)
and are cross-checked here against the independent numpy/scipy restatement
(oracle/np_crosscheck.py, scipy.linalg.eigh) before they are written.  Inputs use numpy's
Philox bit generator with the seed stored next to them.
"""
import json
import os
import sys

import numpy as np
import scipy.linalg as sl

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import np_crosscheck as X  # noqa: E402
from oracle import oracle as O  # noqa: E402


def rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def fd1d():
    out = {}
    for k in range(1, 8):
        for ncp in (1, 2):
            for lo, hi in ((0, 0), (1, 0), (0, 1), (1, 1)):
                h = [0.125] * ncp
                M, A = O.patch_matrices_1d(k, h, lo, hi, ip=1.0)
                S, lam = O.gen_eig(A, M)
                ref = sl.eigh(A, M, eigvals_only=True)
                assert np.allclose(lam, ref, rtol=1e-12, atol=0), (k, ncp, lo, hi)
                key = f"k{k}_ncp{ncp}_lo{lo}_hi{hi}"
                out[key + "_M"] = M
                out[key + "_A"] = A
                out[key + "_lam"] = lam
    np.savez_compressed(os.path.join(HERE, "fd1d.npz"), **out)


VMULT_CASES = [
    # dim, k, n_cells, patch_variant, smoother_variant, omega, ip, seed
    (2, 3, (6, 6), 1, 0, 0.5, 1.0, 11),
    (2, 2, (5, 3), 0, 0, 0.7, 1.0, 12),
    (3, 2, (4, 3, 3), 1, 0, 0.15, 1.0, 13),
    (3, 4, (3, 3, 3), 1, 0, 0.15, 1.0, 14),
    (2, 4, (4, 4), 1, 1, 1.0, 1.0, 15),
    (3, 1, (3, 3, 2), 0, 1, 1.0, 2.5, 16),
]


def vmult():
    out = {}
    meta = []
    for i, (dim, k, nc, pv, sv, om, ip, seed) in enumerate(VMULT_CASES):
        N = int(np.prod(nc)) * (k + 1) ** dim
        src = rng(seed).uniform(-1.0, 1.0, N)
        dst = O.schwarz_vmult(dim, k, nc, src, patch_variant=pv, smoother_variant=sv, omega=om, ip=ip)
        if sv == 0 and N <= 3000:
            A = X.sipg_matrix(dim, k, list(nc), ip=ip)
            lowers, _, _ = O.patches(dim, nc, pv, sv)
            ref = X.schwarz_vmult_dense(A, dim, k, list(nc), lowers, 2 if pv else 1, om, src)
            assert np.abs(ref - dst).max() <= 1e-11 * np.abs(ref).max(), i
        out[f"c{i}_src"] = src
        out[f"c{i}_dst"] = dst
        meta.append(dict(dim=dim, k=k, n_cells=list(nc), patch_variant=pv, smoother_variant=sv,
                         omega=om, ip=ip, seed=seed))
    np.savez_compressed(os.path.join(HERE, "vmult.npz"), **out)
    with open(os.path.join(HERE, "vmult_cases.json"), "w") as f:
        json.dump(meta, f, indent=1)


MG_CASES = [
    # dim, k, n_rep, n_cells_fine, patch_variant, smoother_variant, rhs
    (2, 3, 1, 16, 1, 0, "random"),
    (2, 4, 2, 16, 1, 0, "bells"),
    (2, 2, 2, 16, 0, 0, "bells"),
    (3, 2, 2, 8, 1, 0, "bells"),
    (3, 3, 1, 8, 1, 0, "random"),
    (2, 3, 2, 8, 1, 1, "bells"),
]


def mg():
    res = []
    for dim, k, nrep, ncf, pv, sv, rhs in MG_CASES:
        N = ncf ** dim * (k + 1) ** dim
        f = rng(7).uniform(-1, 1, N) if rhs == "random" else X.bells_load_vector(dim, k, ncf)
        it, u, hist = O.mg_cg_solve(dim, k, nrep, ncf, f, patch_variant=pv, smoother_variant=sv,
                                    rel_tol=1e-8)
        res.append(dict(dim=dim, k=k, n_rep=nrep, n_cells_fine=ncf, patch_variant=pv,
                        smoother_variant=sv, rhs=rhs, rhs_seed=7, rel_tol=1e-8, iterations=it,
                        final_residual=float(hist[-1]), initial_residual=float(hist[0])))
    with open(os.path.join(HERE, "mg_iterations.json"), "w") as f:
        json.dump(res, f, indent=1)


def mg_large():
    """CG + V-cycle iteration counts and residual histories of the two benchmark problems,
    FP64, coarse CG to 1e-12 (the reference's coarse solver), right-hand side f ~ U[-1,1] per
    DoF from numpy's Philox generator with seed 0:
      3D SIPG DGQ4 on 64^3 cells (one root cell, 7 levels), damping 0.15 (TPSS.h:121-163);
      2D SIPG DGQ3 on 64^2 cells (2 root cells, 6 levels), damping 0.25, both penalty modes.
    The 3D case takes minutes on a few CPU cores: it is not run by pytest."""
    res = []
    for dim, k, nrep, ncf, om, pen in ((2, 3, 2, 64, 0.25, "reference"), (2, 3, 2, 64, 0.25, "kp1sq"),
                                       (3, 4, 1, 64, 0.15, "reference")):
        N = ncf ** dim * (k + 1) ** dim
        f = rng(0).uniform(-1.0, 1.0, N)
        it, u, hist = O.mg_cg_solve(dim, k, nrep, ncf, f, omega=om, rel_tol=1e-8, penalty=pen)
        assert it > 0, (dim, k, ncf, pen)
        res.append(dict(dim=dim, k=k, n_rep=nrep, n_cells_fine=ncf, patch_variant=1,
                        smoother_variant=0, omega=om, penalty=pen, rhs="random", rhs_seed=0,
                        rel_tol=1e-8, iterations=it, residual_history=[float(r) for r in hist]))
        print(dim, k, ncf, pen, it, flush=True)
    with open(os.path.join(HERE, "mg_large.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    O.build()
    if "--large" in sys.argv:
        mg_large()
    else:
        fd1d()
        vmult()
        mg()
    print("golden fixtures written to", HERE)
