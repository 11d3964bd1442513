"""Batched solves: each problem gets its own CG + GMG result (same kernels, same order),
and a seeded sample of the benchmark family matches the CPU oracle's iteration counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def philox(seed, n):
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, n)


def test_batch_equals_individual_solves(tpss, cuda):
    import torch
    problems = [dict(dim=2, degree=2, n_rep=1, n_cells_fine=16), dict(dim=3, degree=3, n_rep=1, n_cells_fine=8),
                dict(dim=2, degree=5, n_rep=1, n_cells_fine=8), dict(dim=3, degree=2, n_rep=1, n_cells_fine=16),
                dict(dim=2, degree=7, n_rep=1, n_cells_fine=4), dict(dim=3, degree=4, n_rep=1, n_cells_fine=4)]
    for pr in problems:
        pr["precision"] = tpss.Precision.fp32
    b = tpss.BatchSolver(problems, n_streams=3)
    fs = [torch.tensor(philox(i, n), dtype=torch.float64, device=cuda) for i, n in enumerate(b.n_dofs)]
    us = [torch.empty_like(f) for f in fs]
    its = b.solve(us, fs)
    for pr, f, u, it in zip(problems, fs, us, its):
        # the batch autotunes its levels; the same shapes reuse the same choices here
        mg = tpss.MultigridSolver(pr["dim"], pr["degree"], 1, pr["n_cells_fine"], precision=pr["precision"],
                                  coarse_solver=1, autotune=True)
        v = torch.zeros_like(f)
        it1, _ = mg.solve(v, f)
        assert it == it1
        assert torch.equal(u, v)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_sample_matches_oracle_iterations(tpss, oracle, cuda, precision):
    """A seeded sample of the batched problem family (drawn by tpss.draw_batch_problems, the
    rule of the 512-problem benchmark, with caps the CPU oracle finishes in seconds), solved in
    a batch with autotuned kernels and the dense coarse solve the batch needs: FP64 smoothers
    give the oracle's CG + GMG iteration count within one (the oracle's coarse solver is CG to an
    absolute 1e-12, a slightly different preconditioner late in the solve than the exact dense
    coarse solve: on this sample 3D DGQ3 8^3 and 3D DGQ2 8^3 end one iteration apart, at 1.3 and
    1.9 times the tolerance; GPU solves with the coarse CG match the oracle's counts,
    tests/test_gpu_parity.py); FP32 smoothers take between one fewer and two more (the
    FP32 preconditioner's rounding delays CG's superlinear phase by up to two iterations, as 41
    against 39 on 3D DGQ4 64^3)."""
    import torch
    problems, _ = tpss.draw_batch_problems(10, 2024, 600_000, 80_000)
    for pr in problems:
        pr["precision"] = precision
        pr["autotune"] = 1
    b = tpss.BatchSolver(problems, n_streams=4)
    fs_h = [philox(100 + i, n) for i, n in enumerate(b.n_dofs)]
    fs = [torch.tensor(f, dtype=torch.float64, device=cuda) for f in fs_h]
    us = [torch.empty_like(f) for f in fs]
    its = b.solve(us, fs)
    for pr, f, it in zip(problems, fs_h, its):
        it_ref, _, hist = oracle.mg_cg_solve(pr["dim"], pr["degree"], 1, pr["n_cells_fine"], f, rel_tol=1e-8)
        assert it_ref > 0
        if precision == 0:
            assert abs(it - it_ref) <= 1, (pr, it, it_ref)
            if it != it_ref:
                assert hist[min(it, it_ref)] / hist[0] <= 2.5e-8, (pr, it, it_ref)
        else:
            assert -1 <= it - it_ref <= 2, (pr, it, it_ref)


def test_batch_rejects_coarse_cg(tpss, cuda):
    with pytest.raises(tpss.TPSSInvalidArgument, match="dense coarse"):
        tpss.BatchSolver([dict(dim=2, degree=2, n_rep=1, n_cells_fine=8, coarse_solver=0)])
