"""Allocation-free smoother entry point (tpss_precond_vmult_static_scratch).

Some callers cannot allocate device memory once their solve is running -- an application that
owns all GPU memory through its own pool, or one that cannot risk cudaFree's implicit device
synchronization or an out-of-memory error mid-iteration.  For them the library offers a vmult
whose scratch space is a fixed 32 MiB device array instead of a lazily allocated buffer.  This
file checks, through the C ABI, that it gives the same result as the regular vmult on two calls
in a row (the second call must not see the first call's leftovers) and that levels whose
scratch need exceeds the array are rejected.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(tpss, cuda, k, nc, omega=0.15):
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=omega, precision=1))
    return sh, p


def test_static_scratch_matches_regular_vmult(tpss, cuda):
    import torch
    lib = tpss.load()
    sh, p = _setup(tpss, cuda, 4, (20, 17, 24))
    n = sh.n_dofs()
    g = np.random.Generator(np.random.Philox(9))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        src = torch.tensor(g.uniform(-1.0, 1.0, n), dtype=torch.float64, device=cuda)
        ref = torch.empty_like(src)
        rc = lib.tpss_precond_vmult(p.handle, C.c_void_p(ref.data_ptr()), C.c_void_p(src.data_ptr()), stream)
        assert rc == 0, lib.tpss_last_error()
        out = torch.full_like(src, float("nan"))
        rc = lib.tpss_precond_vmult_static_scratch(p.handle, C.c_void_p(out.data_ptr()),
                                                   C.c_void_p(src.data_ptr()), stream)
        assert rc == 0, lib.tpss_last_error()
        torch.cuda.synchronize()
        err = (out - ref).abs().max().item() / ref.abs().max().item()
        assert err <= 2e-5, (call, err)  # the FP32 smoother tolerance of the parity tests


def test_static_scratch_rejects_too_large_levels(tpss, cuda):
    import torch
    lib = tpss.load()
    sh, p = _setup(tpss, cuda, 4, (48, 48, 48))  # needs ~97 MB of halo scratch
    x = torch.zeros(sh.n_dofs(), dtype=torch.float64, device=cuda)
    y = torch.zeros_like(x)
    rc = lib.tpss_precond_vmult_static_scratch(p.handle, C.c_void_p(y.data_ptr()), C.c_void_p(x.data_ptr()),
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 1
    assert b"32 MiB" in lib.tpss_last_error()
