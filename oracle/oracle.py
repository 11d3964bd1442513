"""ctypes front end of the CPU oracle (oracle/tpss_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py``, always as the checker or the timed CPU baseline.  The
product (``tpss_gb300``) never imports it.

The C file restates the reference's Schwarz-smoother path in FP64; see its header for the
reference files each part follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)


_SIMD_PATH = os.path.join(_HERE, "_build", "liboracle_simd.so")


def build(force: bool = False) -> str:
    """Compile the oracle and the SIMD CPU baseline with their Makefile (gcc) and return the
    oracle library path."""
    srcs = [os.path.join(_HERE, f) for f in ("tpss_oracle.c", "simd_baseline.c")]
    newest = max(os.path.getmtime(s) for s in srcs)
    stale = any(not os.path.exists(p) or os.path.getmtime(p) < newest for p in (_LIB_PATH, _SIMD_PATH))
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            L.or_gauss.argtypes = [C.c_int, _dp, _dp]
            L.or_gauss_lobatto.argtypes = [C.c_int, _dp]
            L.or_shape_data.argtypes = [C.c_int] + [_dp] * 7
            L.or_patch_matrices_1d.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.c_int,
                                               C.c_double, _dp, _dp]
            L.or_gen_eig.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
            L.or_fd_apply_packed.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp]
            L.or_patches.argtypes = [C.c_int, _ip, C.c_int, C.c_int, _i32p, _i32p, _ip]
            L.or_patches.restype = C.c_int64
            L.or_schwarz_vmult.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _dp, C.c_double,
                                           _i64p, C.c_int, C.c_int, C.c_double, C.c_int,
                                           C.c_int, C.c_int, _dp, _dp]
            L.or_sipg_vmult.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _dp, C.c_double,
                                        _i64p, _dp, _dp]
            L.or_prolongate_add.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp]
            L.or_restrict_add.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp]
            L.or_mg_cg_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                         C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_int, _dp, _dp, _dp]
            L.or_schwarz_create.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _dp, C.c_double,
                                            _i64p, C.c_int, C.c_int, C.c_double]
            L.or_schwarz_create.restype = C.c_void_p
            L.or_schwarz_apply.argtypes = [C.c_void_p, _dp, _dp]
            L.or_schwarz_apply_range.argtypes = [C.c_void_p, C.c_int64, C.c_int64, _dp, _dp]
            L.or_schwarz_n_patches.argtypes = [C.c_void_p]
            L.or_schwarz_n_patches.restype = C.c_int64
            L.or_schwarz_destroy.argtypes = [C.c_void_p]
            L.or_num_threads.restype = C.c_int
            L.or_set_num_threads.argtypes = [C.c_int]
            L.or_set_penalty_mode.argtypes = [C.c_int]
            _lib = L
    return _lib


PENALTY_MODES = {"reference": 0, "kp1sq": 1}


class _penalty:
    """Holds the oracle's SIPG penalty mode for one call: "reference" (ip k(k+1)(1/h_l+1/h_r)/2
    inside, 2 ip k(k+1)/h on the boundary, apps/common_integrator.h:30-37) or "kp1sq"
    (ip 2(k+1)^2 (1/h_l+1/h_r)/2 inside, ip 2(k+1)^2/h on the boundary)."""

    _mutex = threading.RLock()

    def __init__(self, mode):
        if mode not in PENALTY_MODES:
            raise ValueError(f"unknown penalty mode {mode!r}")
        self.mode = PENALTY_MODES[mode]

    def __enter__(self):
        self._mutex.acquire()
        lib().or_set_penalty_mode(self.mode)

    def __exit__(self, *exc):
        lib().or_set_penalty_mode(0)
        self._mutex.release()


def _d(a):
    return a.ctypes.data_as(_dp)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def gauss(n):
    x, w = np.zeros(n), np.zeros(n)
    assert lib().or_gauss(n, _d(x), _d(w)) == 0
    return x, w


def gauss_lobatto(n):
    x = np.zeros(n)
    assert lib().or_gauss_lobatto(n, _d(x)) == 0
    return x


def shape_data(k):
    np1 = k + 1
    out = [np.zeros(np1), np.zeros(np1), np.zeros(np1), np.zeros(np1 * np1),
           np.zeros(np1 * np1), np.zeros(2 * np1), np.zeros(2 * np1)]
    assert lib().or_shape_data(k, *[_d(a) for a in out]) == 0
    qx, qw, nodes, val, grad, fval, fgrad = out
    return dict(qx=qx, qw=qw, nodes=nodes, val=val.reshape(np1, np1), grad=grad.reshape(np1, np1),
                fval=fval.reshape(2, np1), fgrad=fgrad.reshape(2, np1))


def patch_matrices_1d(k, h, bdry_lo, bdry_hi, ip=1.0, penalty="reference"):
    """1-D mass M and SIPG Laplace A of a DG patch of len(h) (1 or 2) cells."""
    h = _c64(h)
    n = len(h) * (k + 1)
    M, A = np.zeros((n, n)), np.zeros((n, n))
    with _penalty(penalty):
        rc = lib().or_patch_matrices_1d(k, len(h), _d(h), int(bdry_lo), int(bdry_hi), float(ip),
                                        _d(M), _d(A))
    assert rc == 0
    return M, A


def gen_eig(A, M):
    A, M = _c64(A), _c64(M)
    n = A.shape[0]
    S, lam = np.zeros((n, n)), np.zeros(n)
    assert lib().or_gen_eig(n, _d(A), _d(M), _d(S), _d(lam)) == 0
    return S, lam


def fd_apply(S_list, lam_list, r):
    dim = len(S_list)
    n = S_list[0].shape[0]
    Sp = _c64(np.concatenate([s.reshape(-1) for s in S_list]))
    Lp = _c64(np.concatenate(lam_list))
    r = _c64(r)
    u = np.zeros_like(r)
    assert lib().or_fd_apply_packed(dim, n, _d(Sp), _d(Lp), _d(r), _d(u)) == 0
    return u


def _nc3(dim, nc):
    a = np.ones(3, dtype=np.int32)
    a[:dim] = nc
    return a


def patches(dim, nc, patch_variant, smoother_variant=0):
    """(lower cell coords [P,3], colors [P], n_colors) in the oracle's patch order."""
    nc3 = _nc3(dim, nc)
    ncol = C.c_int(0)
    P = lib().or_patches(dim, nc3.ctypes.data_as(_ip), patch_variant, smoother_variant,
                         None, None, C.byref(ncol))
    lower = np.zeros((max(P, 1), 3), dtype=np.int32)
    color = np.zeros(max(P, 1), dtype=np.int32)
    P = lib().or_patches(dim, nc3.ctypes.data_as(_ip), patch_variant, smoother_variant,
                         lower.ctypes.data_as(_i32p), color.ctypes.data_as(_i32p), C.byref(ncol))
    return lower[:P], color[:P], ncol.value


def _h_arrays(dim, nc, h):
    """Per-direction cell widths; h None -> uniform 1/nc."""
    hs = []
    for d in range(3):
        if d < dim:
            if h is None or h[d] is None:
                hs.append(np.full(nc[d], 1.0 / nc[d]))
            else:
                hs.append(_c64(h[d]))
        else:
            hs.append(np.ones(1))
    return hs


def schwarz_vmult(dim, k, nc, src, patch_variant=1, smoother_variant=0, omega=1.0, ip=1.0,
                  h=None, cell_start=None, reverse=False, symmetrized=False, use_ras=False,
                  penalty="reference"):
    nc3 = _nc3(dim, nc)
    hs = _h_arrays(dim, nc, h)
    src = _c64(src)
    dst = np.zeros_like(src)
    cs = None
    if cell_start is not None:
        cs = np.ascontiguousarray(cell_start, dtype=np.int64)
    with _penalty(penalty):
        rc = lib().or_schwarz_vmult(dim, k, nc3.ctypes.data_as(_ip), _d(hs[0]), _d(hs[1]),
                                    _d(hs[2]), float(ip),
                                    cs.ctypes.data_as(_i64p) if cs is not None else None,
                                    patch_variant, smoother_variant, float(omega), int(reverse),
                                    int(symmetrized), 2 if use_ras == "boolean" else int(bool(use_ras)),
                                    _d(src), _d(dst))
    assert rc == 0
    return dst


def sipg_vmult(dim, k, nc, src, ip=1.0, h=None, cell_start=None, penalty="reference"):
    nc3 = _nc3(dim, nc)
    hs = _h_arrays(dim, nc, h)
    src = _c64(src)
    dst = np.zeros_like(src)
    cs = None if cell_start is None else np.ascontiguousarray(cell_start, dtype=np.int64)
    with _penalty(penalty):
        rc = lib().or_sipg_vmult(dim, k, nc3.ctypes.data_as(_ip), _d(hs[0]), _d(hs[1]), _d(hs[2]),
                                 float(ip), cs.ctypes.data_as(_i64p) if cs is not None else None,
                                 _d(src), _d(dst))
    assert rc == 0
    return dst


def prolongate_add(dim, k, nc_coarse, coarse, fine):
    nc3 = _nc3(dim, nc_coarse)
    coarse, fine = _c64(coarse), _c64(fine).copy()
    assert lib().or_prolongate_add(dim, k, nc3.ctypes.data_as(_ip), _d(coarse), _d(fine)) == 0
    return fine


def restrict_add(dim, k, nc_coarse, coarse, fine):
    nc3 = _nc3(dim, nc_coarse)
    coarse, fine = _c64(coarse).copy(), _c64(fine)
    assert lib().or_restrict_add(dim, k, nc3.ctypes.data_as(_ip), _d(coarse), _d(fine)) == 0
    return coarse


def mg_cg_solve(dim, k, n_rep, nc_fine, f, ip=1.0, patch_variant=1, smoother_variant=0,
                omega=None, rel_tol=1e-8, abs_tol=1e-14, max_iter=100, penalty="reference"):
    """CG + one V-cycle per iteration; returns (iterations, u, residual history)."""
    if omega is None:
        omega = lookup_damping_factor(patch_variant, smoother_variant, dim)
    f = _c64(f)
    u = np.zeros_like(f)
    hist = np.zeros(max_iter + 1)
    with _penalty(penalty):
        it = lib().or_mg_cg_solve(dim, k, n_rep, nc_fine, float(ip), patch_variant,
                                  smoother_variant, float(omega), float(rel_tol), float(abs_tol),
                                  max_iter, _d(f), _d(u), _d(hist))
    n = it if it >= 0 else max_iter
    return it, u, hist[: n + 1]


def lookup_damping_factor(patch_variant, smoother_variant, dim):
    """TPSS::lookup_damping_factor (include/solvers_and_preconditioners/TPSS/TPSS.h:121-163)."""
    if smoother_variant == 1:
        return 1.0
    if patch_variant == 0:
        return 0.7
    return 0.25 if dim == 2 else 0.15


def fractional_steps(hist, rel_tol):
    """compute_fractional_steps (apps/postprocess.h:41-60)."""
    n = len(hist) - 1
    rho = (hist[-1] / hist[0]) ** (1.0 / n)
    return float(np.log(rel_tol) / np.log(rho)), float(rho)


class SchwarzHandle:
    """Prebuilt oracle smoother for repeated timing (CPU baseline)."""

    def __init__(self, dim, k, nc, patch_variant=1, smoother_variant=0, omega=1.0, ip=1.0):
        self.nc3 = _nc3(dim, nc)
        self.hs = _h_arrays(dim, nc, None)
        self.h = lib().or_schwarz_create(dim, k, self.nc3.ctypes.data_as(_ip), _d(self.hs[0]),
                                         _d(self.hs[1]), _d(self.hs[2]), float(ip), None,
                                         patch_variant, smoother_variant, float(omega))
        assert self.h, "oracle smoother setup failed"

    @property
    def n_patches(self):
        return lib().or_schwarz_n_patches(self.h)

    def apply(self, dst, src):
        lib().or_schwarz_apply(self.h, _d(dst), _d(src))

    def apply_range(self, p0, p1, dst, src):
        lib().or_schwarz_apply_range(self.h, int(p0), int(p1), _d(dst), _d(src))

    def close(self):
        if self.h:
            lib().or_schwarz_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_simd = None


def simd_lib():
    """The timed CPU baseline (oracle/simd_baseline.c: SIMD macro patches of 8 FP64 lanes)."""
    global _simd
    with _lock:
        if _simd is None:
            build()
            L = C.CDLL(_SIMD_PATH)
            L.or_simd_create.argtypes = [C.c_int, C.c_int, _ip, C.c_int, C.c_double]
            L.or_simd_create.restype = C.c_void_p
            L.or_simd_apply.argtypes = [C.c_void_p, _dp, _dp]
            L.or_simd_apply_range.argtypes = [C.c_void_p, C.c_int64, C.c_int64, _dp, _dp]
            L.or_simd_n_patches.argtypes = [C.c_void_p]
            L.or_simd_n_patches.restype = C.c_int64
            L.or_simd_destroy.argtypes = [C.c_void_p]
            L.or_num_threads.restype = C.c_int
            L.or_set_num_threads.argtypes = [C.c_int]
            _simd = L
    return _simd


class SimdSchwarzHandle:
    """Additive Schwarz smoother of the reference's CPU path with SIMD macro patches (8 FP64
    lanes, FMA), the timed CPU baseline; same interface as SchwarzHandle."""

    def __init__(self, dim, k, nc, patch_variant=1, omega=1.0):
        self.nc3 = _nc3(dim, nc)
        self.h = simd_lib().or_simd_create(dim, k, self.nc3.ctypes.data_as(_ip), patch_variant, float(omega))
        assert self.h, "SIMD baseline setup failed"

    @property
    def n_patches(self):
        return simd_lib().or_simd_n_patches(self.h)

    def apply(self, dst, src):
        simd_lib().or_simd_apply(self.h, _d(dst), _d(src))

    def apply_range(self, p0, p1, dst, src):
        simd_lib().or_simd_apply_range(self.h, int(p0), int(p1), _d(dst), _d(src))

    def close(self):
        if self.h:
            simd_lib().or_simd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simd_set_num_threads(n):
    simd_lib().or_set_num_threads(int(n))


def simd_num_threads():
    return simd_lib().or_num_threads()


def num_threads():
    return lib().or_num_threads()


def set_num_threads(n):
    lib().or_set_num_threads(int(n))


def _lib_ext():
    L = lib()
    if not getattr(L, "_ext_ready", False):
        L.or_ksvd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp]
        L.or_ksvd_diag.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _dp, _dp]
        L.or_surrogate_h.argtypes = [C.c_int, _ip, _dp, C.c_int, _dp]
        L.or_schwarz_vmult_surrogate.argtypes = [C.c_int, C.c_int, _ip, _dp, C.c_double, C.c_double,
                                                 _dp, _dp]
        L._ext_ready = True
    return L


def ksvd(M, big_shape, small_shape, rank):
    """Best Kronecker rank-r approximation M ~ sum_r B_r (x) A_r (compute_ksvd)."""
    M = _c64(M)
    bm, bn = big_shape
    sm, sn = small_shape
    B = np.zeros((rank, bm, bn))
    A = np.zeros((rank, sm, sn))
    assert _lib_ext().or_ksvd(bm, bn, sm, sn, _d(M), rank, _d(B), _d(A)) == 0
    return B, A


def ksvd_diag(d, big, small, rank):
    """Diagonal variant: diagonals of B_r (big) and A_r (small)."""
    d = _c64(d)
    B = np.zeros((rank, big))
    A = np.zeros((rank, small))
    assert _lib_ext().or_ksvd_diag(big, small, _d(d), rank, _d(B), _d(A)) == 0
    return B, A


def distorted_coords(dim, nc, seed, amplitude=0.25, mode="cube"):
    """Vertex coordinates of the unit cube with nc cells per direction, every interior vertex
    displaced (numpy Philox, seed).
    mode "cube": by U[-amplitude h_d, amplitude h_d] in every coordinate d;
    mode "edge": as the reference's mesh generator does it (GridTools::distort_random called
    from apps/mesh.h:160-190): in a uniformly random direction, by amplitude times the
    shortest edge at the vertex. Per-coordinate shifts of 0.25 h can invert cells (a 32^3
    mesh with seed 7 has 8 cells with a negative corner Jacobian); shifts of at most 0.25 of
    the shortest edge cannot."""
    if mode == "edge":
        nv = [n + 1 for n in nc]
        grids = np.meshgrid(*[np.arange(n) / (n - 1) for n in reversed(nv)], indexing="ij")
        X = np.stack([grids[dim - 1 - d] for d in range(dim)], axis=-1).reshape(-1, dim)
        g = np.random.Generator(np.random.Philox(seed))
        v = g.normal(size=X.shape)
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        hmin = 1.0 / max(nc[:dim])
        idx = np.indices(list(reversed(nv))).reshape(dim, -1)[::-1].T
        interior = np.all((idx > 0) & (idx < np.array(nc)[None, :]), axis=1)
        X[interior] += amplitude * hmin * v[interior]
        return np.ascontiguousarray(X)
    nv = [n + 1 for n in nc]
    grids = np.meshgrid(*[np.arange(n) / (n - 1) for n in reversed(nv)], indexing="ij")
    X = np.stack([grids[dim - 1 - d] for d in range(dim)], axis=-1).reshape(-1, dim)
    g = np.random.Generator(np.random.Philox(seed))
    disp = g.uniform(-amplitude, amplitude, X.shape) / np.array(nc)[None, :]
    idx = np.indices(list(reversed(nv))).reshape(dim, -1)[::-1].T  # (x, y[, z]) per vertex
    interior = np.all((idx > 0) & (idx < np.array(nc)[None, :]), axis=1)
    X[interior] += disp[interior]
    return np.ascontiguousarray(X)


def surrogate_h(dim, nc, coords, nq=5):
    """Per vertex patch, direction and 1-D cell: surrogate width [P, dim, 2]."""
    nc3 = _nc3(dim, nc)
    lower, _, _ = patches(dim, nc, 1, 0)
    out = np.zeros((len(lower), dim, 2))
    assert _lib_ext().or_surrogate_h(dim, nc3.ctypes.data_as(_ip), _d(_c64(coords)), nq, _d(out)) == 0
    return out


def schwarz_vmult_surrogate(dim, k, nc, hp, src, omega=1.0, ip=1.0):
    nc3 = _nc3(dim, nc)
    src = _c64(src)
    dst = np.zeros_like(src)
    assert _lib_ext().or_schwarz_vmult_surrogate(dim, k, nc3.ctypes.data_as(_ip), _d(_c64(hp)), float(ip),
                                                 float(omega), _d(src), _d(dst)) == 0
    return dst
