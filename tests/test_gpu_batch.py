"""Batched lockstep solves give each problem's own CG + GMG result (same kernels, same order)."""
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
        mg = tpss.MultigridSolver(pr["dim"], pr["degree"], 1, pr["n_cells_fine"], precision=pr["precision"],
                                  coarse_solver=1)
        v = torch.zeros_like(f)
        it1, _ = mg.solve(v, f)
        assert it == it1
        assert torch.equal(u, v)
