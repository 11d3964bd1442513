"""GPU parity of the Schwarz smoother path against the CPU oracle (through the C ABI).

Tolerances:
  FP64 smoother, operator, transfer: relative max-norm error <= 1e-12
  FP32 smoother (FP32 gather / FD / scatter into FP64 vectors): relative error <= 2e-5
  FP32 level operator (single-precision V-cycle): relative error <= 1e-5
  CG+MG: identical iteration counts to the oracle (the exceptions are stated at the test).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def philox(seed, n):
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, n)


def gpu_vmult(tpss, cuda, dim, k, nc, src, pv=1, sv=0, omega=1.0, ip=1.0, precision=0, h=None,
              cell_start=None, ras=False, reverse=False, symmetrized=False, coloring=None):
    import torch
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=pv,
                                              smoother_variant=sv, cell_h=h,
                                              cell_dof_start=cell_start, coloring=coloring)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh, ip) if sv == 1 else None
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(
        relaxation=omega, precision=precision, ip_factor=ip, use_ras_weights=ras is True,
        use_ras_boolean_weights=ras == "boolean", reverse=reverse, symmetrized=symmetrized))
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    d = torch.full_like(s, 123.0)  # vmult must overwrite dst
    p.vmult(d, s)
    torch.cuda.synchronize()
    return d.cpu().numpy(), p


CASES = [
    # dim, k, n_cells, patch_variant
    (2, 1, (4, 4), 1), (2, 3, (6, 5), 1), (2, 5, (3, 4), 1), (2, 7, (3, 3), 1),
    (3, 1, (3, 3, 3), 1), (3, 2, (4, 3, 5), 1), (3, 4, (4, 4, 4), 1), (3, 7, (2, 3, 2), 1),
    (2, 2, (5, 3), 0), (2, 6, (3, 3), 0), (3, 3, (3, 2, 4), 0), (3, 5, (2, 2, 3), 0),
]


@pytest.mark.parametrize("dim,k,nc,pv", CASES)
def test_additive_fp64_parity(tpss, oracle, cuda, dim, k, nc, pv):
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = philox(100 + k, N)
    om = 0.37
    got, _ = gpu_vmult(tpss, cuda, dim, k, nc, src, pv=pv, omega=om)
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=pv, omega=om)
    assert rel_err(got, ref) <= 1e-12


@pytest.mark.parametrize("dim,k,nc,pv", CASES)
def test_additive_fp32_parity(tpss, oracle, cuda, dim, k, nc, pv):
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = philox(200 + k, N)
    got, _ = gpu_vmult(tpss, cuda, dim, k, nc, src, pv=pv, omega=0.5, precision=1)
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=pv, omega=0.5)
    assert rel_err(got, ref) <= 2e-5


def test_golden_vmult_fixtures(tpss, cuda):
    g = np.load(os.path.join(GOLDEN, "vmult.npz"))
    cases = json.load(open(os.path.join(GOLDEN, "vmult_cases.json")))
    for i, c in enumerate(cases):
        got, _ = gpu_vmult(tpss, cuda, c["dim"], c["k"], c["n_cells"], g[f"c{i}_src"],
                           pv=c["patch_variant"], sv=c["smoother_variant"], omega=c["omega"],
                           ip=c["ip"])
        assert rel_err(got, g[f"c{i}_dst"]) <= 1e-12, i


def test_nonuniform_h_permuted_cells_ras(tpss, oracle, cuda):
    dim, k, nc = 3, 2, (4, 3, 3)
    g = np.random.default_rng(1)
    h = [g.uniform(0.5, 1.5, n) for n in nc]
    h = [x / x.sum() for x in h]
    ncell = int(np.prod(nc))
    nd = (k + 1) ** dim
    cell_start = g.permutation(ncell) * nd
    src = philox(7, ncell * nd)
    for ras in (False, True, "boolean"):
        got, _ = gpu_vmult(tpss, cuda, dim, k, nc, src, pv=1, omega=0.8, h=h, cell_start=cell_start,
                           ras=ras)
        ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.8, h=h,
                                   cell_start=cell_start, use_ras=ras)
        assert rel_err(got, ref) <= 1e-12, ras


@pytest.mark.parametrize("dim,k,nc", [(2, 1, (4, 4)), (2, 3, (6, 5)), (2, 5, (2, 3)), (3, 1, (3, 3, 3)),
                                      (3, 2, (4, 3, 5)), (3, 4, (4, 4, 4)), (3, 6, (2, 3, 2))])
def test_ras_boolean_weights_parity(tpss, oracle, cuda, dim, k, nc):
    """Restricted prolongation (rscatter_add): FP64 <= 1e-12, FP32 <= 2e-5 against the oracle;
    the streamed kernel is not used for it (the per-color kernel skips the restricted DoFs)."""
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = philox(300 + k, N)
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.45, use_ras="boolean")
    plain = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.45)
    assert rel_err(plain, ref) > 1e-3  # the restriction changes the result
    for precision, tol in ((0, 1e-12), (1, 2e-5)):
        got, _ = gpu_vmult(tpss, cuda, dim, k, nc, src, pv=1, omega=0.45, precision=precision, ras="boolean")
        assert rel_err(got, ref) <= tol, precision


@pytest.mark.parametrize("dim,k,nc,pv,rev,sym", [(2, 3, (5, 4), 1, False, False),
                                                 (2, 2, (4, 4), 0, False, False),
                                                 (3, 2, (3, 3, 3), 1, True, False),
                                                 (3, 1, (3, 4, 3), 0, False, True),
                                                 (2, 4, (4, 3), 1, False, True)])
def test_multiplicative_parity(tpss, oracle, cuda, dim, k, nc, pv, rev, sym):
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = philox(31, N)
    got, _ = gpu_vmult(tpss, cuda, dim, k, nc, src, pv=pv, sv=1, omega=1.0, reverse=rev,
                       symmetrized=sym)
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=pv, smoother_variant=1, omega=1.0,
                               reverse=rev, symmetrized=sym)
    assert rel_err(got, ref) <= 1e-11


def test_user_coloring_same_additive_result(tpss, oracle, cuda):
    dim, k, nc = 2, 2, (5, 5)
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1)
    P = tpss.SubdomainHandler(ad).n_subdomains()
    src = philox(3, 25 * 9)
    got, _ = gpu_vmult(tpss, cuda, dim, k, nc, src, pv=1, omega=1.0, coloring=list(range(P)))
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=1.0)
    assert rel_err(got, ref) <= 1e-12


def test_edge_cases(tpss, oracle, cuda):
    import torch
    # a single vertex patch (2^dim cells) and no vertex patch at all (1 cell per direction)
    for dim in (2, 3):
        N = 2 ** dim * 27 if dim == 3 else 4 * 9
        src = philox(1, N)
        got, _ = gpu_vmult(tpss, cuda, dim, 2, (2,) * dim, src, pv=1)
        assert rel_err(got, oracle.schwarz_vmult(dim, 2, (2,) * dim, src, patch_variant=1)) <= 1e-12
        src1 = philox(2, 3 ** dim)
        got1, p = gpu_vmult(tpss, cuda, dim, 2, (1,) * dim, src1, pv=1)
        assert np.all(got1 == 0.0) and p.subdomain_handler.n_subdomains() == 0
    # elongated meshes
    src = philox(4, 9 * 2 * 4)
    got, _ = gpu_vmult(tpss, cuda, 2, 1, (9, 2), src, pv=1)
    assert rel_err(got, oracle.schwarz_vmult(2, 1, (9, 2), src, patch_variant=1)) <= 1e-12
    # Tvmult is not implemented in the reference either
    ad = tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(3, 3), patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData())
    x = torch.zeros(sh.n_dofs(), dtype=torch.float64, device=cuda)
    with pytest.raises(tpss.TPSSNotImplemented):
        p.Tvmult(x, x.clone())
    with pytest.raises(ValueError):
        p.vmult(x[:-1], x[:-1].clone())
    with pytest.raises(tpss.TPSSInvalidArgument):
        p.vmult(x, x)  # aliasing dst and src is rejected


def test_vmult_add_and_time_data(tpss, oracle, cuda):
    import torch
    dim, k, nc = 2, 3, (4, 4)
    N = 16 * 16
    src = philox(5, N)
    base = philox(6, N)
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.25))
    d = torch.tensor(base, dtype=torch.float64, device=cuda)
    p.vmult_add(d, torch.tensor(src, dtype=torch.float64, device=cuda))
    ref = base + oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.25)
    assert rel_err(d.cpu().numpy(), ref) <= 1e-12
    td = p.get_time_data()
    assert len(td) == 5 and td[4].description.startswith("[SchwarzPrecond] Step")
    assert td[4].n_calls >= 1 and td[1].time > 0.0 and td[2].n_calls == 1
    # shallow copy shares the local solvers
    q = tpss.SchwarzPreconditioner()
    q.initialize(p, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.5))
    d2 = torch.zeros(N, dtype=torch.float64, device=cuda)
    q.vmult(d2, torch.tensor(src, dtype=torch.float64, device=cuda))
    ref2 = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.5)
    assert rel_err(d2.cpu().numpy(), ref2) <= 1e-12


@pytest.mark.parametrize("dim,k,nc,ip", [(2, 3, (5, 4), 1.0), (3, 2, (3, 4, 2), 2.5), (3, 4, (4, 4, 4), 1.0),
                                         (2, 7, (3, 3), 1.0)])
def test_operator_parity(tpss, oracle, cuda, dim, k, nc, ip):
    import torch
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh, ip)
    src = philox(9, sh.n_dofs())
    d = torch.zeros(sh.n_dofs(), dtype=torch.float64, device=cuda)
    op.vmult(d, torch.tensor(src, dtype=torch.float64, device=cuda))
    ref = oracle.sipg_vmult(dim, k, nc, src, ip=ip)
    assert rel_err(d.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("dim,k,nc,ip", [(2, 3, (5, 4), 1.0), (3, 2, (3, 4, 2), 2.5), (3, 4, (6, 5, 4), 1.0),
                                         (2, 7, (3, 3), 1.0), (3, 1, (7, 3, 5), 1.0)])
def test_operator_fp32_parity(tpss, oracle, cuda, dim, k, nc, ip):
    """The single-precision level operator (FP32 arithmetic, FP64 vectors) against the FP64
    oracle: relative error of FP32 rounding (tolerance 1e-5 in the 2-norm)."""
    import torch
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh, ip)
    src = philox(19, sh.n_dofs())
    d = torch.full((sh.n_dofs(),), float("nan"), dtype=torch.float64, device=cuda)
    op.vmult_fp32(d, torch.tensor(src, dtype=torch.float64, device=cuda))
    ref = oracle.sipg_vmult(dim, k, nc, src, ip=ip)
    err = rel_err(d.cpu().numpy(), ref)
    assert 0.0 < err <= 1e-5, err


def test_mg_fp32_vcycle_operator(tpss, oracle, xcheck, cuda):
    """CG with a V-cycle whose smoothing residuals use the FP32 level operator (FP32 smoothers):
    converges to the tolerance in at most two more iterations than the FP64 V-cycle operator."""
    import torch
    for c in json.load(open(os.path.join(GOLDEN, "mg_iterations.json"))):
        if c["smoother_variant"] != 0:
            continue
        N = c["n_cells_fine"] ** c["dim"] * (c["k"] + 1) ** c["dim"]
        if c["rhs"] == "random":
            f = np.random.Generator(np.random.Philox(c["rhs_seed"])).uniform(-1, 1, N)
        else:
            f = xcheck.bells_load_vector(c["dim"], c["k"], c["n_cells_fine"])
        its = {}
        for opp in (0, 1):
            mg = tpss.MultigridSolver(c["dim"], c["k"], c["n_rep"], c["n_cells_fine"],
                                      patch_variant=c["patch_variant"], smoother_variant=0,
                                      precision=1, coarse_solver=1, vcycle_precision=opp)
            u = torch.zeros(N, dtype=torch.float64, device=cuda)
            ft = torch.tensor(f, dtype=torch.float64, device=cuda)
            it, hist = mg.solve(u, ft, rel_tol=c["rel_tol"])
            assert hist[-1] <= c["rel_tol"] * hist[0] * (1 + 1e-12), (c, opp)
            # true residual of the returned solution with the FP64 operator
            sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
                dim=c["dim"], degree=c["k"], n_cells=(c["n_cells_fine"],) * c["dim"], patch_variant=1))
            A = tpss.LaplaceOperator(sh, 1.0)
            r = torch.empty_like(u)
            A.vmult(r, u)
            true_rel = float(torch.linalg.norm(ft - r) / torch.linalg.norm(ft))
            assert true_rel <= 2 * c["rel_tol"], (c, opp, true_rel)
            its[opp] = it
        assert its[1] <= its[0] + 2, (c, its)


@pytest.mark.parametrize("dim,k,ncc", [(2, 3, (3, 2)), (3, 2, (2, 3, 2)), (3, 5, (2, 2, 2))])
def test_transfer_parity(tpss, oracle, cuda, dim, k, ncc):
    import torch
    nf = [2 * n for n in ncc]
    nd = (k + 1) ** dim
    uc = philox(1, int(np.prod(ncc)) * nd)
    uf = philox(2, int(np.prod(nf)) * nd)
    f = torch.tensor(uf, dtype=torch.float64, device=cuda)
    c = torch.tensor(uc, dtype=torch.float64, device=cuda)
    tpss.prolongate_add(dim, k, ncc, f, c)
    ref = oracle.prolongate_add(dim, k, ncc, uc, uf)
    assert rel_err(f.cpu().numpy(), ref) <= 1e-13
    c2 = torch.tensor(uc, dtype=torch.float64, device=cuda)
    tpss.restrict_add(dim, k, ncc, c2, torch.tensor(uf, dtype=torch.float64, device=cuda))
    ref2 = oracle.restrict_add(dim, k, ncc, uc, uf)
    assert rel_err(c2.cpu().numpy(), ref2) <= 1e-13


def test_smoother_step(tpss, oracle, cuda):
    import torch
    dim, k, nc = 2, 3, (6, 6)
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh, 1.0)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.25))
    sm = tpss.SchwarzSmoother()
    sm.initialize(op, p, tpss.SchwarzSmoother.AdditionalData(number_of_smoothing_steps=2))
    b = philox(3, sh.n_dofs())
    x0 = philox(4, sh.n_dofs())
    x = torch.tensor(x0, dtype=torch.float64, device=cuda)
    sm.step(x, torch.tensor(b, dtype=torch.float64, device=cuda))
    ref = x0.copy()
    for _ in range(2):
        r = b - oracle.sipg_vmult(dim, k, nc, ref)
        ref = ref + oracle.schwarz_vmult(dim, k, nc, r, patch_variant=1, omega=0.25)
    assert rel_err(x.cpu().numpy(), ref) <= 1e-12
    y = torch.tensor(x0, dtype=torch.float64, device=cuda)
    sm.vmult(y, torch.tensor(b, dtype=torch.float64, device=cuda))
    ref = np.zeros_like(b)
    for _ in range(2):
        r = b - oracle.sipg_vmult(dim, k, nc, ref)
        ref = ref + oracle.schwarz_vmult(dim, k, nc, r, patch_variant=1, omega=0.25)
    assert rel_err(y.cpu().numpy(), ref) <= 1e-12


def test_mg_cg_iterations_match_oracle(tpss, oracle, xcheck, cuda):
    import torch
    for c in json.load(open(os.path.join(GOLDEN, "mg_iterations.json"))):
        N = c["n_cells_fine"] ** c["dim"] * (c["k"] + 1) ** c["dim"]
        if c["rhs"] == "random":
            f = np.random.Generator(np.random.Philox(c["rhs_seed"])).uniform(-1, 1, N)
        else:
            f = xcheck.bells_load_vector(c["dim"], c["k"], c["n_cells_fine"])
        for coarse_solver in (0, 1):
            for graph in (False, True):
                mg = tpss.MultigridSolver(c["dim"], c["k"], c["n_rep"], c["n_cells_fine"],
                                          patch_variant=c["patch_variant"],
                                          smoother_variant=c["smoother_variant"],
                                          coarse_solver=coarse_solver, use_graph=graph)
                u = torch.zeros(N, dtype=torch.float64, device=cuda)
                it, hist = mg.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda),
                                    rel_tol=c["rel_tol"])
                if coarse_solver == 0:
                    # the reference's coarse solver (CG to 1e-12): identical iteration counts,
                    # except where the oracle's own residual sits at the tolerance: the coarse CG
                    # stops at an absolute 1e-12, so late in the outer solve the V-cycle is a
                    # slightly variable preconditioner and rounding moves the last iteration
                    if it != c["iterations"]:
                        _, _, h_ref = oracle.mg_cg_solve(c["dim"], c["k"], c["n_rep"], c["n_cells_fine"], f,
                                                         patch_variant=c["patch_variant"],
                                                         smoother_variant=c["smoother_variant"],
                                                         rel_tol=c["rel_tol"])
                        edge = h_ref[min(it, c["iterations"])] / h_ref[0] / c["rel_tol"]
                        assert abs(it - c["iterations"]) == 1 and abs(edge - 1.0) < 0.25, (c, graph, it, edge)
                        assert hist[-1] <= c["rel_tol"] * hist[0]
                    else:
                        assert abs(hist[-1] - c["final_residual"]) <= 1e-6 * c["initial_residual"]
                else:
                    # the exact (dense) coarse solve differs from CG-to-1e-12 below 1e-12;
                    # the count may move by one when a residual lands next to the tolerance
                    assert abs(it - c["iterations"]) <= 1, (c, graph, it)
        # the FP32 smoother converges within two iterations of the FP64 count: its rounding
        # (about 1e-7 relative per application) delays CG's superlinear phase, by two iterations
        # on 3D DGQ4 64^3, and the exact count moves with the rounding of the other kernels
        mg32 = tpss.MultigridSolver(c["dim"], c["k"], c["n_rep"], c["n_cells_fine"],
                                    patch_variant=c["patch_variant"],
                                    smoother_variant=c["smoother_variant"], precision=1,
                                    coarse_solver=1)
        u = torch.zeros(N, dtype=torch.float64, device=cuda)
        it32, _ = mg32.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda), rel_tol=c["rel_tol"])
        assert it32 <= c["iterations"] + 2, (c, it32)


@pytest.mark.parametrize("dim,k,n,prec", [(2, 3, 16, 0), (3, 2, 8, 1)])
def test_device_cg_loop_equals_host_loop(tpss, cuda, dim, k, n, prec):
    """The device-side CG loop (one graph, a conditional WHILE node around one iteration) runs
    the host loop's kernels in the same order: same iteration count, residual history and
    solution; both stop at max_iter with TPSSNotConverged."""
    import torch
    res = []
    for use_graph in (True, False):
        mg = tpss.MultigridSolver(dim, k, 1, n, precision=prec, coarse_solver=1, use_graph=use_graph)
        f = torch.tensor(philox(91, mg.n_dofs()), dtype=torch.float64, device=cuda)
        u = torch.zeros_like(f)
        it, hist = mg.solve(u, f)
        res.append((it, hist, u.cpu().numpy()))
        with pytest.raises(tpss.TPSSNotConverged):
            mg.solve(torch.zeros_like(f), f, max_iter=3)
    assert res[0][0] == res[1][0] > 3
    assert np.array_equal(res[0][1], res[1][1])
    assert np.array_equal(res[0][2], res[1][2])


def test_mg_solution_matches_oracle(tpss, oracle, xcheck, cuda):
    import torch
    dim, k, nrep, ncf = 2, 4, 2, 16
    f = xcheck.bells_load_vector(dim, k, ncf)
    it_ref, u_ref, _ = oracle.mg_cg_solve(dim, k, nrep, ncf, f, rel_tol=1e-10)
    mg = tpss.MultigridSolver(dim, k, nrep, ncf)
    u = torch.zeros(f.size, dtype=torch.float64, device=cuda)
    it, _ = mg.solve(u, torch.tensor(f, dtype=torch.float64, device=cuda), rel_tol=1e-10)
    assert it == it_ref
    assert rel_err(u.cpu().numpy(), u_ref) <= 1e-9


def test_full_size_config2_fp32_vs_oracle(tpss, oracle, cuda):
    """3D DGQ4 on 64^3 cells (32.8M DoFs): the FP32 smoother against the FP64 oracle at full
    size, plus linearity and symmetry of the GPU operator."""
    import torch
    dim, k, n = 3, 4, 64
    N = n ** 3 * 125
    src = philox(2024, N)
    got, p = gpu_vmult(tpss, cuda, dim, k, (n, n, n), src, pv=1, omega=0.15, precision=1)
    ref = oracle.schwarz_vmult(dim, k, (n, n, n), src, patch_variant=1, omega=0.15)
    assert rel_err(got, ref) <= 2e-5
    # linearity P(a x + b y) = a P x + b P y and symmetry y.Px = x.Py (FP64 smoother)
    p64 = tpss.SchwarzPreconditioner()
    p64.initialize(p.subdomain_handler, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.15))
    x = torch.tensor(src, dtype=torch.float64, device=cuda)
    y = torch.tensor(philox(2025, N), dtype=torch.float64, device=cuda)
    Px, Py, Pz = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    p64.vmult(Px, x)
    p64.vmult(Py, y)
    p64.vmult(Pz, 2.0 * x - 3.0 * y)
    lin = (Pz - (2.0 * Px - 3.0 * Py)).abs().max().item() / Pz.abs().max().item()
    assert lin <= 1e-12
    sym = abs((y * Px).sum().item() - (x * Py).sum().item()) / abs((y * Px).sum().item())
    assert sym <= 1e-10
    assert rel_err(Px.cpu().numpy(), ref) <= 1e-12


STREAM_CASES = [
    # k, n_cells: partial columns, several z segments, minimal meshes
    (1, (9, 5, 17)), (2, (6, 6, 6)), (3, (5, 7, 11)), (4, (2, 2, 2)), (4, (13, 3, 10)),
    (4, (9, 9, 18)), (3, (17, 4, 2)),
]


@pytest.mark.parametrize("k,nc", STREAM_CASES)
@pytest.mark.parametrize("variant", [1, 2])
def test_fp32_streamed_and_color_kernels(tpss, oracle, cuda, k, nc, variant):
    """FP32 additive vertex patches in 3D: the column-streamed kernel (variant 2) and the
    per-color kernel (variant 1) against the FP64 oracle."""
    import torch
    N = int(np.prod(nc)) * (k + 1) ** 3
    src = philox(300 + k, N)
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
        relaxation=0.15, precision=1, kernel_variant=variant))
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    d = torch.full_like(s, float("nan"))  # every entry must be written
    p.vmult(d, s)
    torch.cuda.synchronize()
    ref = oracle.schwarz_vmult(3, k, nc, src, patch_variant=1, omega=0.15)
    assert rel_err(d.cpu().numpy(), ref) <= 2e-5


@pytest.mark.parametrize("k,nc,variant", [(3, (6, 5, 10), 0), (4, (8, 11, 9), 4), (4, (8, 11, 9), 6),
                                         (4, (7, 5, 12), 7), (5, (6, 7, 9), 4), (5, (5, 6, 7), 1)])
def test_streamed_kernel_general_layouts(tpss, oracle, cuda, k, nc, variant):
    """Permuted cell numbering, non-uniform tensor-product h (1-D problems without mirror
    symmetry everywhere, so the plane passes run their full-matrix path) and RAS weights, for
    pencil and plane decompositions. Tolerance 2e-5, at degree 5 3e-4: FP32 fast
    diagonalization of the degree-5 1-D problems on these graded cells (widths up to 3x apart)
    ends 1.4e-4 from the FP64 oracle in the per-color kernel as well (FP64 kernels: 3e-11), so
    at degree 5 the streamed result must also be as close as the per-color kernel's."""
    import torch
    tol = 2e-5 if k <= 4 else 3e-4
    g = np.random.default_rng(11)
    h = [g.uniform(0.5, 1.5, n) for n in nc]
    h = [x / x.sum() for x in h]
    ncell, nd = int(np.prod(nc)), (k + 1) ** 3
    cell_start = g.permutation(ncell) * nd
    src = philox(12, ncell * nd)
    for ras in (False, True):
        ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1,
                                                  cell_h=h, cell_dof_start=cell_start)
        sh = tpss.SubdomainHandler(ad)
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=0.7, precision=1, kernel_variant=2, stream_variant=variant, use_ras_weights=ras))
        s = torch.tensor(src, dtype=torch.float64, device=cuda)
        d = torch.empty_like(s)
        p.vmult(d, s)
        ref = oracle.schwarz_vmult(3, k, nc, src, patch_variant=1, omega=0.7, h=h,
                                   cell_start=cell_start, use_ras=ras)
        err = rel_err(d.cpu().numpy(), ref)
        assert err <= tol, ras
        if k == 5:
            pc = tpss.SchwarzPreconditioner()
            pc.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
                relaxation=0.7, precision=1, kernel_variant=1, use_ras_weights=ras))
            dc = torch.empty_like(s)
            pc.vmult(dc, s)
            assert err <= 1.1 * rel_err(dc.cpu().numpy(), ref), ras


@pytest.mark.parametrize("variant", [0, 6])
def test_streamed_kernel_is_deterministic(tpss, cuda, variant):
    import torch
    k, nc = 4, (20, 12, 17)
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.15, precision=1,
                                                                     kernel_variant=2, stream_variant=variant))
    s = torch.tensor(philox(5, sh.n_dofs()), dtype=torch.float64, device=cuda)
    a, b = torch.empty_like(s), torch.empty_like(s)
    p.vmult(a, s)
    p.vmult(b, s)
    assert torch.equal(a, b)


def test_streamed_kernel_rejects_unsupported(tpss, cuda):
    ad = tpss.SubdomainHandler.AdditionalData(dim=2, degree=3, n_cells=(4, 4), patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(precision=1, kernel_variant=2))
    import torch
    x = torch.zeros(sh.n_dofs(), dtype=torch.float64, device=cuda)
    with pytest.raises(tpss.TPSSInvalidArgument):
        p.vmult(x, x.clone())


@pytest.mark.parametrize("dim,k,nc,precision", [(2, 3, (6, 5), 0), (3, 2, (4, 3, 5), 0), (3, 3, (5, 4, 4), 1),
                                                 (2, 5, (4, 4), 1)])
def test_surrogate_patches_on_distorted_mesh(tpss, oracle, cuda, dim, k, nc, precision):
    """Vertex patches on a distorted mesh with surrogate Cartesian widths (average arc lengths)."""
    import torch
    X = oracle.distorted_coords(dim, nc, 42)
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = philox(77, N)
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=1,
                                              vertex_coords=X)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.4, precision=precision))
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    d = torch.empty_like(s)
    p.vmult(d, s)
    ref = oracle.schwarz_vmult_surrogate(dim, k, nc, oracle.surrogate_h(dim, nc, X), src, omega=0.4)
    assert rel_err(d.cpu().numpy(), ref) <= (1e-12 if precision == 0 else 2e-5)


@pytest.mark.parametrize("k,nc", [(3, (7, 5, 13)), (2, (6, 9, 17)), (1, (5, 6, 11))])
def test_streamed_kernel_per_patch_tables(tpss, oracle, cuda, k, nc):
    """Distorted 3D level: the streamed kernel on per-patch 1-D problems (surrogate widths, and
    Kronecker sums fitted per patch) gives the oracle's / the per-color kernel's result in every
    work decomposition, ragged item tiles included."""
    import torch
    X = oracle.distorted_coords(3, list(nc), 31, 0.2)
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1,
                                              vertex_coords=X)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh, 1.0)
    src = philox(78, sh.n_dofs())
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    ref = oracle.schwarz_vmult_surrogate(3, k, nc, oracle.surrogate_h(3, nc, X), src, omega=0.6)

    def run(local_solver, kv, sv=0):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=0.6, precision=1, kernel_variant=kv, stream_variant=sv, local_solver=local_solver))
        d = torch.full_like(s, 3.0)
        p.vmult(d, s)
        torch.cuda.synchronize()
        return d.cpu().numpy()

    ksum_color = run(tpss.LocalSolver.ksum, 1)
    for v in range(6):
        assert rel_err(run(tpss.LocalSolver.fd, 2, v), ref) <= 2e-5, v
        assert rel_err(run(tpss.LocalSolver.ksum, 2, v), ksum_color) <= 2e-5, v
    # host buffers: the pipelined entry point runs the 4-layer-deep twin (5 for variant 4)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(
        relaxation=0.6, precision=1, kernel_variant=2, stream_variant=4, local_solver=tpss.LocalSolver.ksum))
    h_src = torch.tensor(src, dtype=torch.float64).pin_memory()
    h_dst = torch.full((sh.n_dofs(),), float("nan"), dtype=torch.float64).pin_memory()
    p.vmult_host(h_dst, h_src)
    torch.cuda.synchronize()
    assert np.array_equal(h_dst.numpy(), run(tpss.LocalSolver.ksum, 2, 5))


@pytest.mark.parametrize("k,nc", [(5, (6, 5, 11)), (4, (9, 6, 19)), (3, (7, 5, 13)), (2, (6, 6, 17)),
                                  (1, (5, 9, 18))])
def test_streamed_variants_and_autotune(tpss, oracle, cuda, k, nc):
    """Every work decomposition of the streamed kernel gives the oracle's result; the autotuner
    keeps one of them and leaves dst = P src."""
    import torch
    N = int(np.prod(nc)) * (k + 1) ** 3
    src = philox(400 + k, N)
    ref = oracle.schwarz_vmult(3, k, nc, src, patch_variant=1, omega=0.15)
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    nv = 8 if k == 4 else 6  # degree 4 adds the two plane-pass decompositions
    for v in range(nv):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=0.15, precision=1, kernel_variant=2, stream_variant=v))
        d = torch.full_like(s, float("nan"))
        p.vmult(d, s)
        assert rel_err(d.cpu().numpy(), ref) <= 2e-5, v
    d = torch.full_like(s, float("nan"))
    chosen, ms = p.autotune(d, s, reps=2)
    assert 0 <= chosen < nv and len(ms) == nv and all(t > 0 for t in ms)
    assert rel_err(d.cpu().numpy(), ref) <= 2e-5
    d2 = torch.empty_like(s)
    p.vmult(d2, s)
    assert rel_err(d2.cpu().numpy(), ref) <= 2e-5


@pytest.mark.parametrize("dim,k,nc,pv,sv,precision", [
    (2, 3, (9, 7), 1, 0, 0), (2, 1, (8, 9), 1, 0, 1), (2, 6, (4, 5), 0, 0, 0), (3, 4, (5, 4, 6), 1, 0, 0),
    (3, 2, (5, 5, 4), 0, 0, 1), (3, 6, (3, 3, 2), 1, 0, 1), (2, 4, (5, 4), 1, 1, 0), (3, 1, (3, 4, 3), 0, 1, 0)])
def test_color_kernel_variants_and_autotune(tpss, oracle, cuda, dim, k, nc, pv, sv, precision):
    """Every patches-per-CTA decomposition of the per-color kernel (2D, cell patches, FP64,
    k > 4, multiplicative) gives the oracle's result (FP64 1e-12, FP32 2e-5); the autotuner times
    them, keeps one and leaves dst = P src."""
    import torch
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = philox(500 + k, N)
    om = 0.3 if sv == 0 else 1.0
    ref = oracle.schwarz_vmult(dim, k, nc, src, patch_variant=pv, smoother_variant=sv, omega=om)
    tol = 1e-12 if precision == 0 else 2e-5
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=nc, patch_variant=pv,
                                              smoother_variant=sv)
    sh = tpss.SubdomainHandler(ad)
    op = tpss.LaplaceOperator(sh) if sv == 1 else None
    s = torch.tensor(src, dtype=torch.float64, device=cuda)
    for v in range(3):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=om, precision=precision, kernel_variant=1, stream_variant=v))
        d = torch.full_like(s, float("nan"))
        p.vmult(d, s)
        assert rel_err(d.cpu().numpy(), ref) <= tol, v
    d = torch.full_like(s, float("nan"))
    chosen, ms = p.autotune(d, s, reps=2)
    assert 1 <= len(ms) <= 3 and 0 <= chosen < len(ms)
    if len(ms) > 1:
        assert all(t > 0 for t in ms)
    assert rel_err(d.cpu().numpy(), ref) <= tol
    if dim == 2 or k <= 4:
        assert len(ms) >= 2, "small patches offer at least two decompositions"


@pytest.mark.parametrize("k,nc,variant", [(4, (9, 6, 19), 0), (3, (7, 5, 33), 2), (2, (6, 6, 17), 3), (1, (5, 9, 40), 1),
                                         (4, (10, 7, 21), 4), (3, (6, 9, 18), 5), (4, (8, 11, 23), 6),
                                         (4, (7, 5, 12), 7), (5, (6, 5, 13), 0), (5, (5, 6, 11), 4)])
def test_vmult_host_buffers_pipelined(tpss, oracle, cuda, k, nc, variant):
    """The host-buffer entry point (copies pipelined with the streamed kernel along z) gives
    the oracle's result and the bits of the device path with the decomposition the pipeline
    runs (the 4-layer-deep twin of the chosen one: 5 for the warp-per-patch variants 4 and 5,
    7 for the plane-pass variants 6 and 7, 2 otherwise); also for the per-color path."""
    import torch
    N = int(np.prod(nc)) * (k + 1) ** 3
    src = philox(500 + k, N)
    ref = oracle.schwarz_vmult(3, k, nc, src, patch_variant=1, omega=0.15)
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    host_variant = 5 if variant in (4, 5) else 7 if variant in (6, 7) else 2
    for kv in (2, 1):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=0.15, precision=1, kernel_variant=kv, stream_variant=variant))
        h_src = torch.tensor(src, dtype=torch.float64).pin_memory()
        h_dst = torch.full((N,), float("nan"), dtype=torch.float64).pin_memory()
        p.vmult_host(h_dst, h_src)
        torch.cuda.synchronize()
        pd = tpss.SchwarzPreconditioner()
        pd.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
            relaxation=0.15, precision=1, kernel_variant=kv, stream_variant=host_variant))
        d = torch.empty(N, dtype=torch.float64, device=cuda)
        pd.vmult(d, h_src.to(cuda))
        torch.cuda.synchronize()
        assert rel_err(h_dst.numpy(), ref) <= 2e-5
        assert np.array_equal(h_dst.numpy(), d.cpu().numpy())
