"""Small standalone workloads of the library's secondary kernels, for profiling them one at a
time (`python -m tpss_gb300.workloads <name>`):

  bsr    mapped SIPG operator (block-sparse FP64 product) on a distorted 3D DGQ3 24^3 level
  c0ip   C0IP biharmonic FE_Q(3) 512^2 level: operator and Bilaplacian-FD FP32 smoother
  mlp    one training epoch of the learned local solver's network (87 -> 3 x 64 -> 108) on
         119,164 samples
  host   the streamed FP32 smoother between pinned host buffers on 3D DGQ4 64^3
"""
from __future__ import annotations

import sys


def run(name: str) -> None:
    import torch

    import tpss_gb300 as tpss
    from tpss_gb300.mesh import distorted_cube

    if name == "bsr":
        n, k = 24, 3
        X = distorted_cube(3, [n] * 3, 7, 0.15)
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
            dim=3, degree=k, n_cells=(n,) * 3, vertex_coords=X))
        op = tpss.LaplaceOperator(sh)
        x = torch.rand(sh.n_dofs(), dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(3):
            op.vmult(y, x)
    elif name == "c0ip":
        P = tpss.C0IPBiharmonic(3, 2, 512, local_solver=tpss.LocalSolver.fd, precision=tpss.Precision.fp32)
        x = torch.rand(P.n_dofs(), dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(3):
            P.vmult(y, x)
            P.smooth(y, x)
    elif name == "mlp":
        m = tpss.MLP(87, 108, 64, 3, seed=1)
        x = torch.rand(119164, 87, device="cuda")
        t = torch.rand(119164, 108, device="cuda")
        m.train(x, t, epochs=1, batch=256)
    elif name == "host":
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=3, degree=4, n_cells=(64,) * 3))
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.15, precision=tpss.Precision.fp32))
        N = sh.n_dofs()
        h_src = torch.rand(N, dtype=torch.float64).pin_memory()
        h_dst = torch.empty(N, dtype=torch.float64).pin_memory()
        for _ in range(3):
            p.vmult_host(h_dst, h_src)
    else:
        raise SystemExit(f"unknown workload {name!r}")
    torch.cuda.synchronize()
    print("done", name)


if __name__ == "__main__":
    run(sys.argv[1] if len(sys.argv) > 1 else "bsr")
