"""Allocation-free smoother entry point (tpss_precond_vmult_static_scratch).

Some callers cannot allocate device memory once their solve is running -- an application that
owns all GPU memory through its own pool, or one that cannot risk cudaFree's implicit device
synchronization or an out-of-memory error mid-iteration.  For them the library offers a vmult
whose scratch space is a fixed 32 MiB device array instead of a lazily allocated buffer.  This
file checks, through the C ABI, that

  - on a freshly created preconditioner the call leaves the device's free memory unchanged
    (the regular vmult, which grows its scratch buffer with cudaMalloc, runs only afterwards);
  - it gives the same result as the regular vmult on two calls in a row (the second call must
    not see the first call's leftovers), within the FP32 smoother tolerance 2e-5 of the
    parity tests;
  - levels whose scratch need exceeds the array, and options it does not honour
    (check_finite, the per-color kernel), are rejected.

It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(tpss, cuda, k, nc, omega=0.15, **kw):
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=k, n_cells=nc, patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=omega, precision=1, **kw))
    return sh, p


def _call(lib, fn, p, out, src, stream):
    rc = fn(p.handle, C.c_void_p(out.data_ptr()), C.c_void_p(src.data_ptr()), stream)
    assert rc == 0, lib.tpss_last_error()


def test_static_scratch_allocates_nothing_and_matches_regular_vmult(tpss, cuda):
    import torch
    lib = tpss.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = np.random.Generator(np.random.Philox(9))
    # warm-up on a separate preconditioner: loads the kernels' code and looks up the static
    # array's device address, both of which are one-time, per-process costs
    shw, pw = _setup(tpss, cuda, 4, (9, 8, 10))
    xw = torch.zeros(shw.n_dofs(), dtype=torch.float64, device=cuda)
    yw = torch.empty_like(xw)
    _call(lib, lib.tpss_precond_vmult_static_scratch, pw, yw, xw, stream)
    torch.cuda.synchronize()

    sh, p = _setup(tpss, cuda, 4, (20, 17, 24))
    n = sh.n_dofs()
    srcs = [torch.tensor(g.uniform(-1.0, 1.0, n), dtype=torch.float64, device=cuda) for _ in range(2)]
    outs = [torch.full_like(srcs[0], float("nan")) for _ in range(2)]
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for call in range(2):
        _call(lib, lib.tpss_precond_vmult_static_scratch, p, outs[call], srcs[call], stream)
        torch.cuda.synchronize()
        free_after, _ = torch.cuda.mem_get_info()
        assert free_after == free_before, (call, free_before - free_after)
    for call in range(2):
        ref = torch.empty_like(srcs[call])
        _call(lib, lib.tpss_precond_vmult, p, ref, srcs[call], stream)
        torch.cuda.synchronize()
        err = (outs[call] - ref).abs().max().item() / ref.abs().max().item()
        assert err <= 2e-5, (call, err)


def test_static_scratch_rejects_too_large_levels_and_unhonoured_options(tpss, cuda):
    import torch
    lib = tpss.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    sh, p = _setup(tpss, cuda, 4, (48, 48, 48))  # needs ~97 MB of halo scratch
    x = torch.zeros(sh.n_dofs(), dtype=torch.float64, device=cuda)
    y = torch.zeros_like(x)
    rc = lib.tpss_precond_vmult_static_scratch(p.handle, C.c_void_p(y.data_ptr()), C.c_void_p(x.data_ptr()),
                                               stream)
    assert rc == 1
    assert b"32 MiB" in lib.tpss_last_error()
    for kw, word in ((dict(check_finite=True), b"check_finite"), (dict(kernel_variant=1), b"per-color")):
        sh, p = _setup(tpss, cuda, 2, (6, 6, 6), **kw)
        x = torch.zeros(sh.n_dofs(), dtype=torch.float64, device=cuda)
        y = torch.zeros_like(x)
        rc = lib.tpss_precond_vmult_static_scratch(p.handle, C.c_void_p(y.data_ptr()),
                                                   C.c_void_p(x.data_ptr()), stream)
        assert rc == 1 and word in lib.tpss_last_error(), kw
