"""C-ABI library checks that need no GPU: it loads, exports every symbol that
include/tpss_gpu.h declares, builds patch layouts identical to the oracle's, and rejects
invalid input with the documented status codes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "tpss_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tpss_[a-zA-Z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(tpss):
    lib = tpss.load()
    syms = header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s
    from tpss_gb300 import _lib
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)
    assert b"sm_103a" in lib.tpss_version()


@pytest.mark.parametrize("dim,nc,pv,sv", [(2, (5, 4), 1, 0), (3, (3, 4, 5), 1, 0), (2, (3, 3), 0, 0),
                                          (3, (3, 2, 2), 0, 1), (2, (6, 5), 0, 1), (2, (2, 2), 1, 0),
                                          (3, (2, 2, 2), 1, 1), (2, (64, 64), 1, 0)])
def test_layout_matches_oracle(tpss, oracle, dim, nc, pv, sv):
    ad = tpss.SubdomainHandler.AdditionalData(dim=dim, degree=2, n_cells=nc, patch_variant=pv,
                                              smoother_variant=sv)
    sh = tpss.SubdomainHandler(ad)
    lo, col = sh.patches()
    lo2, col2, nco = oracle.patches(dim, nc, pv, sv)
    assert sh.n_colors() == nco
    np.testing.assert_array_equal(lo, lo2)
    np.testing.assert_array_equal(col, col2)
    assert sh.n_dofs() == int(np.prod(nc)) * 3 ** dim


def test_layout_colors_are_conflict_free(tpss):
    ad = tpss.SubdomainHandler.AdditionalData(dim=3, degree=1, n_cells=(6, 5, 4), patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    lo, col = sh.patches()
    for c in range(sh.n_colors()):
        cells = set()
        for l in lo[col == c]:
            for b in range(8):
                cell = (l[0] + (b & 1), l[1] + ((b >> 1) & 1), l[2] + ((b >> 2) & 1))
                assert cell not in cells
                cells.add(cell)
    # interior patches before boundary patches within each color
    nc = np.array([6, 5, 4])
    for c in range(sh.n_colors()):
        bd = [bool(np.any(l == 0) or np.any(l + 1 == nc - 1)) for l in lo[col == c]]
        assert bd == sorted(bd)


def test_user_coloring_conflict_is_rejected(tpss):
    ad = tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(4, 4), patch_variant=1)
    P = tpss.SubdomainHandler(ad).n_subdomains()
    ad.coloring = [0] * P  # all overlapping vertex patches in one color
    with pytest.raises(tpss.TPSSInvalidArgument, match="conflict"):
        tpss.SubdomainHandler(ad)
    ad.coloring = list(range(P))  # one patch per color is always race-free
    sh = tpss.SubdomainHandler(ad)
    assert sh.n_colors() == P


@pytest.mark.parametrize("bad", [dict(dim=4), dict(degree=0), dict(degree=8),
                                 dict(n_cells=(0, 3)), dict(patch_variant=7)])
def test_invalid_layouts(tpss, bad):
    args = dict(dim=2, degree=2, n_cells=(3, 3), patch_variant=1)
    args.update(bad)
    with pytest.raises(tpss.TPSSInvalidArgument):
        tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(**args))


def test_cell_dof_start_must_be_a_permutation(tpss):
    ad = tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(2, 2), patch_variant=1,
                                              cell_dof_start=[0, 4, 4, 12])
    with pytest.raises(tpss.TPSSInvalidArgument):
        tpss.SubdomainHandler(ad)


def test_precond_option_errors_before_gpu_work(tpss):
    """Both RAS options together are rejected as in schwarz_preconditioner.templates.h:599-600,
    RAS boolean weights on cell patches ("TODO") and on a multiplicative smoother ("Additive
    scheme is only supported.") as in dof_info.templates.h:208-212 -- before any device memory
    is touched."""
    ad = tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(3, 3), patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    with pytest.raises(tpss.TPSSInvalidArgument, match="more than one RAS"):
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
            use_ras_weights=True, use_ras_boolean_weights=True))
    shc = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(3, 3),
                                                                      patch_variant=0))
    with pytest.raises(tpss.TPSSNotImplemented):
        p.initialize(shc, None, tpss.SchwarzPreconditioner.AdditionalData(use_ras_boolean_weights=True))
    shm = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(3, 3),
                                                                      patch_variant=1, smoother_variant=1))
    with pytest.raises(tpss.TPSSInvalidArgument, match="Additive"):
        p.initialize(shm, None, tpss.SchwarzPreconditioner.AdditionalData(use_ras_boolean_weights=True))
    with pytest.raises(tpss.TPSSInvalidArgument, match="relaxation"):
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.0))


def test_damping_lookup(tpss, oracle):
    for pv in (0, 1):
        for sv in (0, 1):
            for dim in (2, 3):
                assert tpss.lookup_damping_factor(pv, sv, dim) == oracle.lookup_damping_factor(pv, sv, dim)


def test_null_arguments_return_status(tpss):
    lib = tpss.load()
    assert lib.tpss_layout_create(None, None) == 1
    assert b"null" in lib.tpss_last_error()
    assert lib.tpss_precond_vmult(None, None, None, None) == 1
    n = C.c_int(0)
    assert lib.tpss_mg_n_levels(None, C.byref(n)) == 1


def test_new_entry_points_reject_invalid_input_before_gpu_work(tpss):
    """C0IP, network, batch and local-solver options are validated on the host first."""
    with pytest.raises(tpss.TPSSInvalidArgument, match="degree"):
        tpss.C0IPBiharmonic(1, 2, 8)
    with pytest.raises(tpss.TPSSInvalidArgument, match="n_rep"):
        tpss.C0IPBiharmonic(3, 1, 8)
    with pytest.raises(tpss.TPSSInvalidArgument, match="n_rep"):
        tpss.C0IPBiharmonic(3, 2, 12)
    with pytest.raises(tpss.TPSSInvalidArgument, match="local_solver"):
        tpss.C0IPBiharmonic(3, 2, 8, local_solver=2)
    with pytest.raises(tpss.TPSSInvalidArgument, match="sizes"):
        tpss.MLP(0, 4)
    ad = tpss.SubdomainHandler.AdditionalData(dim=2, degree=1, n_cells=(3, 3), patch_variant=1)
    sh = tpss.SubdomainHandler(ad)
    p = tpss.SchwarzPreconditioner()
    with pytest.raises(tpss.TPSSInvalidArgument, match="trained model"):
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(local_solver=3))
    with pytest.raises(tpss.TPSSInvalidArgument, match="local solver"):
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(local_solver=7))
    with pytest.raises(tpss.TPSSNotImplemented, match="RAS"):
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(local_solver=1, use_ras_weights=True))
    lib = tpss.load()
    h = C.c_void_p()
    assert lib.tpss_batch_create(None, 0, 1, C.byref(h)) == 1
    assert lib.tpss_precond_vmult_host(None, None, None, None) == 1
    assert lib.tpss_c0ip_cg_solve(None, None, None, 1e-8, 1e-14, 10, None, None, None) == 1
    assert lib.tpss_operator_vmult_fp32(None, None, None, None) == 1
    with pytest.raises(tpss.TPSSInvalidArgument, match="vcycle_precision"):
        tpss.MultigridSolver(2, 2, 2, 8, vcycle_precision=5)


def test_ctypes_descriptors_match_the_c_structs(tpss):
    """Field lists of the Python descriptors equal the C struct members (names, in order)."""
    src = open(os.path.join(ROOT, "include", "tpss_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    from tpss_gb300 import _lib
    for cname, pyname in (("tpss_layout_desc", "LayoutDesc"), ("tpss_precond_desc", "PrecondDesc"),
                          ("tpss_mg_desc", "MgDesc"), ("tpss_c0ip_desc", "C0ipDesc"),
                          ("tpss_mlp_desc", "MlpDesc")):
        body = re.search(r"typedef struct %s\s*\{(.*?)\}\s*%s;" % (cname, cname), src, flags=re.S).group(1)
        names = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            for part in decl.split(","):
                m = re.search(r"(\w+)\s*(\[\d+\])?\s*$", part.strip())
                names.append(m.group(1))
        assert [f[0] for f in getattr(_lib, pyname)._fields_] == names, cname


def test_build_compiles_every_cuda_source():
    """Every translation unit under tpss_gb300/csrc is in the build's unit list (a kernel file
    left out would leave its entry points unresolved in the library)."""
    from tpss_gb300 import build
    csrc = os.path.join(ROOT, "tpss_gb300", "csrc")
    sources = sorted(f for f in os.listdir(csrc) if f.endswith(".cu"))
    units = sorted({u[0] for u in build.UNITS})
    assert units == sources


def test_batch_draw_is_seeded_and_respects_the_caps(tpss):
    """The 512-problem family's draw: deterministic per seed, every problem within the
    per-problem cap, the sum within the total budget, degrees and sizes from the stated sets."""
    a, ra = tpss.draw_batch_problems(512, 4, 96_000_000, 8_000_000)
    b, rb = tpss.draw_batch_problems(512, 4, 96_000_000, 8_000_000)
    assert a == b and ra == rb and len(a) == 512
    sizes = [(p["n_cells_fine"] * (p["degree"] + 1)) ** p["dim"] for p in a]
    assert max(sizes) <= 8_000_000 and sum(sizes) <= 96_000_000
    assert all(p["dim"] in (2, 3) and 2 <= p["degree"] <= 7 and p["n_cells_fine"] in (8, 16, 32, 64) for p in a)
    c, _ = tpss.draw_batch_problems(512, 5, 96_000_000, 8_000_000)
    assert c != a
    with pytest.raises(ValueError):
        tpss.draw_batch_problems(512, 4, 1000, 8_000_000)
