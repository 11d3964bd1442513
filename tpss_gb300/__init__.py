"""tpss_gb300 -- GB300 (sm_103a) Schwarz smoother of TPSS behind its operator interface.

Python mirror of the reference's smoother-path API (jwitte08/TPSS):

  SubdomainHandler      SubdomainHandler<dim,Number>::reinit / AdditionalData
                        (include/solvers_and_preconditioners/TPSS/subdomain_handler.h:33-262)
  LaplaceOperator       MF::Operator (apps/laplace_integrator.h:396-786), matrix-free SIPG
  SchwarzPreconditioner SchwarzPreconditioner<dim,OperatorType,VectorType,MatrixType>
                        (preconditioner/schwarz_preconditioner.h:88-588)
  SchwarzSmoother       SchwarzSmoother / SmootherRichardson
                        (smoother/schwarz_smoother.h, smoother/smoother_richardson.h)
  MultigridSolver       GMG V-cycle + CG of apps/poisson_problem.h:642-755

Every call goes through the C ABI of include/tpss_gpu.h (libtpss_gpu.so, built in-tree);
vectors are torch CUDA float64 tensors (or raw device pointers) and work is ordered on
torch's current CUDA stream.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (TPSS_ADDITIVE, TPSS_FP32, TPSS_FP64, TPSS_MULTIPLICATIVE, TPSS_PATCH_CELL,
                   TPSS_PATCH_VERTEX, TPSSError, TPSSInvalidArgument, TPSSNotConverged,
                   TPSSNotImplemented, check, load)

__all__ = ["SubdomainHandler", "LaplaceOperator", "SchwarzPreconditioner", "SchwarzSmoother",
           "MultigridSolver", "PatchVariant", "SmootherVariant", "Precision", "Penalty", "TimeInfo",
           "lookup_damping_factor", "prolongate_add", "restrict_add", "TPSSError",
           "TPSSNotImplemented", "TPSSInvalidArgument", "TPSSNotConverged", "load"]


class PatchVariant:
    """TPSS::PatchVariant"""
    cell = TPSS_PATCH_CELL
    vertex = TPSS_PATCH_VERTEX


class SmootherVariant:
    """TPSS::SmootherVariant"""
    additive = TPSS_ADDITIVE
    multiplicative = TPSS_MULTIPLICATIVE


class Precision:
    fp64 = TPSS_FP64
    fp32 = TPSS_FP32


class Penalty:
    """SIPG penalty of the operator and the local solvers (tpss_*_desc.penalty_mode)."""
    reference = _lib.TPSS_PENALTY_REFERENCE  # ip k(k+1) (1/h_l+1/h_r)/2 inside, 2 ip k(k+1)/h on the boundary
    kp1sq = _lib.TPSS_PENALTY_2KP1SQ          # ip 2(k+1)^2 (1/h_l+1/h_r)/2 inside, ip 2(k+1)^2/h on the boundary


def lookup_damping_factor(patch_variant: int, smoother_variant: int, dim: int) -> float:
    """TPSS::lookup_damping_factor (include/solvers_and_preconditioners/TPSS/TPSS.h:121-163)."""
    if smoother_variant == SmootherVariant.multiplicative:
        return 1.0
    if patch_variant == PatchVariant.cell:
        return 0.7
    if dim == 2:
        return 0.25
    if dim == 3:
        return 0.15
    raise ValueError("This case is not listed!")


def _stream(stream):
    if stream is not None:
        return C.c_void_p(int(stream))
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(x, n: Optional[int] = None, writable: bool = False):
    """Device pointer of a torch CUDA float64 contiguous tensor (or an int address)."""
    if isinstance(x, int):
        return C.c_void_p(x)
    import torch
    if not isinstance(x, torch.Tensor):
        raise TypeError("vectors must be torch CUDA tensors or device addresses")
    if not x.is_cuda or x.dtype != torch.float64 or not x.is_contiguous():
        raise TypeError("vectors must be contiguous float64 CUDA tensors")
    if n is not None and x.numel() != n:
        raise ValueError(f"vector has {x.numel()} entries, expected {n}")
    return C.c_void_p(x.data_ptr())


@dataclass
class TimeInfo:
    """TPSS::TimeInfo (include/solvers_and_preconditioners/TPSS/time_info.h:23-64)."""
    time: float
    description: str
    unit: str = "[s]"
    n_calls: int = 0


class SubdomainHandler:
    """Patch layout of one structured level (SubdomainHandler::reinit).

    Vertex patches are gathered around interior vertices with their cells in lexicographic
    order; colors follow the tiled coloring (vertex patches), one color (additive cell
    patches) or red-black (multiplicative cell patches), or a user coloring.
    """

    @dataclass
    class AdditionalData:
        dim: int = 2
        degree: int = 1
        n_cells: Sequence[int] = (2, 2)
        patch_variant: int = PatchVariant.vertex
        smoother_variant: int = SmootherVariant.additive
        level: int = 0
        cell_h: Optional[Sequence[Sequence[float]]] = None
        cell_dof_start: Optional[Sequence[int]] = None
        coloring: Optional[Sequence[int]] = None  # user coloring in default patch order
        vertex_coords: Optional[Sequence[float]] = None  # distorted mesh: [(n+1)^dim, dim]
        surrogate_n_q: int = 5

    def __init__(self, additional_data: Optional["SubdomainHandler.AdditionalData"] = None):
        self._h = None
        self.additional_data = None
        if additional_data is not None:
            self.reinit(additional_data)

    def reinit(self, ad: "SubdomainHandler.AdditionalData"):
        L = load()
        self.clear()
        d = _lib.LayoutDesc()
        d.dim, d.degree, d.dof_layout = ad.dim, ad.degree, _lib.TPSS_DOF_DGQ
        d.patch_variant, d.smoother_variant = ad.patch_variant, ad.smoother_variant
        nc = list(ad.n_cells) + [1] * (3 - len(ad.n_cells))
        for i in range(3):
            d.n_cells[i] = int(nc[i])
        keep = []
        if ad.cell_h is not None:
            for i, h in enumerate(ad.cell_h):
                arr = np.ascontiguousarray(h, dtype=np.float64)
                keep.append(arr)
                d.cell_h[i] = arr.ctypes.data_as(C.POINTER(C.c_double))
        if ad.cell_dof_start is not None:
            cs = np.ascontiguousarray(ad.cell_dof_start, dtype=np.int64)
            keep.append(cs)
            d.cell_dof_start = cs.ctypes.data_as(C.POINTER(C.c_int64))
        if ad.coloring is not None:
            col = np.ascontiguousarray(ad.coloring, dtype=np.int32)
            keep.append(col)
            d.patch_color = col.ctypes.data_as(C.POINTER(C.c_int32))
        if ad.vertex_coords is not None:
            vc = np.ascontiguousarray(ad.vertex_coords, dtype=np.float64)
            keep.append(vc)
            d.vertex_coords = vc.ctypes.data_as(C.POINTER(C.c_double))
        d.surrogate_n_q = int(ad.surrogate_n_q)
        h = C.c_void_p()
        check(L.tpss_layout_create(C.byref(d), C.byref(h)))
        self._h = h
        self.additional_data = ad
        n_dofs, n_patches, n_colors = C.c_int64(), C.c_int64(), C.c_int()
        check(L.tpss_layout_info(h, C.byref(n_dofs), C.byref(n_patches), C.byref(n_colors)))
        self._n_dofs, self._n_patches, self._n_colors = n_dofs.value, n_patches.value, n_colors.value

    def clear(self):
        if self._h:
            load().tpss_layout_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def n_dofs(self) -> int:
        return self._n_dofs

    def n_subdomains(self) -> int:
        return self._n_patches

    def n_dofs_per_patch(self) -> int:
        ad = self.additional_data
        ncp = 2 if ad.patch_variant == PatchVariant.vertex else 1
        return (ncp * (ad.degree + 1)) ** ad.dim

    def n_colors(self) -> int:
        return self._n_colors

    def get_additional_data(self):
        return self.additional_data

    def patches(self):
        """(lower cell coordinates [P,3], colors [P]) in storage order."""
        P = self._n_patches
        lower = np.zeros((max(P, 1), 3), dtype=np.int32)
        col = np.zeros(max(P, 1), dtype=np.int32)
        check(load().tpss_layout_patches(self._h, lower.ctypes.data_as(C.POINTER(C.c_int32)),
                                         col.ctypes.data_as(C.POINTER(C.c_int32))))
        return lower[:P], col[:P]


class LaplaceOperator:
    """Matrix-free SIPG operator of one level (MF::Operator, FP64)."""

    def __init__(self, subdomain_handler: SubdomainHandler, ip_factor: float = 1.0,
                 penalty_mode: int = Penalty.reference):
        self.subdomain_handler = subdomain_handler
        h = C.c_void_p()
        check(load().tpss_operator_create_penalty(subdomain_handler.handle, float(ip_factor),
                                                  int(penalty_mode), C.byref(h)))
        self._h = h
        self.ip_factor = ip_factor
        self.penalty_mode = penalty_mode

    def m(self):
        return self.subdomain_handler.n_dofs()

    n = m

    def vmult(self, dst, src, stream=None):
        n = self.m()
        check(load().tpss_operator_vmult(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def vmult_fp32(self, dst, src, stream=None):
        """The same product in FP32 arithmetic (FP64 vectors): the level operator of a
        single-precision V-cycle."""
        n = self.m()
        check(load().tpss_operator_vmult_fp32(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def Tvmult(self, dst, src, stream=None):
        self.vmult(dst, src, stream)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        try:
            if self._h:
                load().tpss_operator_destroy(self._h)
                self._h = None
        except Exception:
            pass


class SchwarzPreconditioner:
    """SchwarzPreconditioner: vmult(dst, src) sets dst = sum_j omega R_j^T A_j^-1 R_j src."""

    @dataclass
    class AdditionalData:
        relaxation: float = 1.0
        reverse: bool = False
        symmetrized: bool = False
        use_ras_weights: bool = False
        use_ras_boolean_weights: bool = False
        precision: int = Precision.fp64
        ip_factor: float = 1.0
        check_finite: bool = False
        kernel_variant: int = 0  # 0 auto, 1 one launch per color, 2 column-streamed (3D, FP32)
        stream_variant: int = 0  # work decomposition of the column-streamed kernel (0..7 at degree 4, else 0..5)
        local_solver: int = 0    # LocalSolver.fd / exact / ksum / learned
        model: "MLP" = None      # trained network for LocalSolver.learned
        penalty_mode: int = Penalty.reference  # must match the level operator's

    def __init__(self):
        self._h = None
        self.subdomain_handler = None
        self.linear_operator = None
        self.additional_data = None

    @staticmethod
    def _desc(ad):
        d = _lib.PrecondDesc()
        d.relaxation = float(ad.relaxation)
        d.reverse, d.symmetrized = int(ad.reverse), int(ad.symmetrized)
        d.use_ras_weights = int(ad.use_ras_weights)
        d.use_ras_boolean_weights = int(ad.use_ras_boolean_weights)
        d.precision, d.ip_factor = int(ad.precision), float(ad.ip_factor)
        d.check_finite = int(ad.check_finite)
        d.kernel_variant = int(ad.kernel_variant)
        d.stream_variant = int(ad.stream_variant)
        d.local_solver = int(ad.local_solver)
        d.model = ad.model.handle if ad.model is not None else None
        d.penalty_mode = int(ad.penalty_mode)
        return d

    def initialize(self, subdomain_handler, linear_operator=None, additional_data=None):
        """initialize(subdomain_handler, operator, additional_data), or the shallow copy
        initialize(other_preconditioner, additional_data)."""
        if isinstance(subdomain_handler, SchwarzPreconditioner):
            other, ad = subdomain_handler, linear_operator
            self.clear()
            h = C.c_void_p()
            check(load().tpss_precond_create_shallow(other._h, C.byref(self._desc(ad)), C.byref(h)))
            self._h = h
            self.subdomain_handler = other.subdomain_handler
            self.linear_operator = other.linear_operator
            self.additional_data = ad
            return
        ad = additional_data or SchwarzPreconditioner.AdditionalData()
        self.clear()
        h = C.c_void_p()
        op = linear_operator.handle if linear_operator is not None else None
        check(load().tpss_precond_create(subdomain_handler.handle, op, C.byref(self._desc(ad)),
                                         C.byref(h)))
        self._h = h
        self.subdomain_handler = subdomain_handler
        self.linear_operator = linear_operator
        self.additional_data = ad

    def clear(self):
        if self._h:
            load().tpss_precond_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    def get_additional_data(self):
        return self.additional_data

    def get_subdomain_handler(self):
        return self.subdomain_handler

    def m(self):
        return self.subdomain_handler.n_dofs()

    n = m

    def vmult(self, dst, src, stream=None):
        n = self.m()
        check(load().tpss_precond_vmult(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def vmult_add(self, dst, src, stream=None):
        n = self.m()
        check(load().tpss_precond_vmult_add(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def Tvmult(self, dst, src, stream=None):
        n = self.m()
        check(load().tpss_precond_Tvmult(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def vmult_host(self, dst, src, stream=None):
        """vmult with dst and src in host memory (pinned CPU float64 tensors or numpy arrays);
        the copies overlap the streamed kernel. Stream-ordered."""
        n = self.m()

        def hptr(a):
            if isinstance(a, np.ndarray):
                assert a.dtype == np.float64 and a.size == n and a.flags.c_contiguous
                return C.c_void_p(a.ctypes.data)
            assert (not a.is_cuda) and a.dtype.is_floating_point and a.element_size() == 8 and a.numel() == n
            return C.c_void_p(a.data_ptr())

        check(load().tpss_precond_vmult_host(self._h, hptr(dst), hptr(src), _stream(stream)))

    def autotune(self, dst, src, reps=5, stream=None):
        """Time the kernel variants for this level on (src -> dst) and keep the fastest.
        Returns (chosen variant, milliseconds per variant)."""
        n = self.m()
        chosen, nv = C.c_int(0), C.c_int(0)
        ms = np.zeros(8)
        check(load().tpss_precond_autotune(self._h, _ptr(dst, n), _ptr(src, n), int(reps),
                                           C.byref(chosen), ms.ctypes.data_as(C.POINTER(C.c_double)),
                                           C.byref(nv), _stream(stream)))
        return chosen.value, ms[: nv.value].tolist()

    def get_time_data(self):
        L = load()
        n = C.c_int(0)
        check(L.tpss_precond_time_info(self._h, None, C.byref(n)))
        arr = (_lib.TimeInfo * n.value)()
        check(L.tpss_precond_time_info(self._h, arr, C.byref(n)))
        return [TimeInfo(a.time, a.description.decode(), "[s]", a.n_calls) for a in arr]

    @property
    def handle(self):
        return self._h


class SchwarzSmoother:
    """SchwarzSmoother / SmootherRichardson: step(x, b) does x += damping P (b - A x)."""

    @dataclass
    class AdditionalData:
        number_of_smoothing_steps: int = 1
        damping_factor: float = 1.0

    def __init__(self):
        self._h = None

    def initialize(self, linear_operator: LaplaceOperator, preconditioner: SchwarzPreconditioner,
                   additional_data=None):
        ad = additional_data or SchwarzSmoother.AdditionalData()
        self.clear()
        h = C.c_void_p()
        check(load().tpss_smoother_create(linear_operator.handle, preconditioner.handle,
                                          int(ad.number_of_smoothing_steps),
                                          float(ad.damping_factor), C.byref(h)))
        self._h = h
        self.linear_operator = linear_operator
        self.preconditioner = preconditioner
        self.additional_data = ad

    def step(self, dst, src, stream=None):
        n = self.preconditioner.m()
        check(load().tpss_smoother_step(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def vmult(self, dst, src, stream=None):
        n = self.preconditioner.m()
        check(load().tpss_smoother_vmult(self._h, _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def clear(self):
        if self._h:
            load().tpss_smoother_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass


class C0IPBiharmonic:
    """Clamped C0IP biharmonic problem on the unit square (FE_Q(k), Gauss-Lobatto nodes):
    level operators, the additive vertex-patch smoother and CG + V-cycle. Vectors: interior
    nodes, x fastest, float64 CUDA tensors. With problem = Q_POISSON the same node grid carries
    the Poisson problem with continuous FE_Q(k) (Laplacian M x L + L x M, Q vertex patches)."""

    BIHARMONIC = 0  # tpss_c0ip_desc.problem: TPSS_C0IP_BIHARMONIC
    Q_POISSON = 1   # TPSS_Q_POISSON: Laplacian with continuous FE_Q(k), the Q vertex-patch layout

    def __init__(self, degree, n_rep, n_cells_fine, ip_factor=1.0, local_solver=1, precision=0,
                 relaxation=0.25, problem=0):
        d = _lib.C0ipDesc()
        d.degree, d.n_rep, d.n_cells_fine = degree, n_rep, n_cells_fine
        d.ip_factor, d.local_solver, d.precision, d.relaxation = float(ip_factor), int(local_solver), int(precision), float(relaxation)
        d.problem = int(problem)
        h = C.c_void_p()
        check(load().tpss_c0ip_create(C.byref(d), C.byref(h)))
        self._h = h
        nl = C.c_int()
        check(load().tpss_c0ip_info(h, -1, None, C.byref(nl)))
        self.n_levels = nl.value

    def n_dofs(self, level=-1):
        n = C.c_int64()
        check(load().tpss_c0ip_info(self._h, int(level), C.byref(n), None))
        return n.value

    def vmult(self, dst, src, level=-1, stream=None):
        n = self.n_dofs(level)
        check(load().tpss_c0ip_operator_vmult(self._h, int(level), _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def smooth(self, dst, src, level=-1, stream=None):
        n = self.n_dofs(level)
        check(load().tpss_c0ip_smoother_vmult(self._h, int(level), _ptr(dst, n), _ptr(src, n), _stream(stream)))

    def solve(self, u, f, rel_tol=1e-8, abs_tol=1e-14, max_iter=200, stream=None):
        n = self.n_dofs()
        hist = np.zeros(max_iter + 1)
        it = C.c_int(0)
        check(load().tpss_c0ip_cg_solve(self._h, _ptr(u, n), _ptr(f, n), float(rel_tol), float(abs_tol),
                                        int(max_iter), C.byref(it), hist.ctypes.data_as(C.POINTER(C.c_double)),
                                        _stream(stream)))
        return it.value, hist[: it.value + 1]

    def __del__(self):
        try:
            if self._h:
                load().tpss_c0ip_destroy(self._h)
                self._h = None
        except Exception:
            pass


class BatchSolver:
    """Many independent CG + GMG problems (unit-cube SIPG levels) solved concurrently: every
    problem's device-side CG loop (one CUDA graph) launched once on one of n_streams streams,
    one host synchronization for the whole batch."""

    def __init__(self, problems, n_streams=64):
        """problems: list of dicts with MultigridSolver keyword arguments (dim, degree, n_rep,
        n_cells_fine, relaxation, precision, coarse_solver, use_graph, ...)."""
        arr = (_lib.MgDesc * len(problems))()
        for d, pr in zip(arr, problems):
            dim = pr["dim"]
            pv = pr.get("patch_variant", PatchVariant.vertex)
            sv = pr.get("smoother_variant", SmootherVariant.additive)
            d.dim, d.degree, d.n_rep, d.n_cells_fine = dim, pr["degree"], pr["n_rep"], pr["n_cells_fine"]
            d.ip_factor, d.patch_variant, d.smoother_variant = float(pr.get("ip_factor", 1.0)), pv, sv
            rel = pr.get("relaxation")
            d.relaxation = float(rel if rel is not None else lookup_damping_factor(pv, sv, dim))
            d.precision = int(pr.get("precision", Precision.fp32))
            d.coarse_tol = float(pr.get("coarse_tol", 1e-12))
            d.coarse_solver = int(pr.get("coarse_solver", 1))
            d.use_graph = int(pr.get("use_graph", 1))
            d.autotune = int(pr.get("autotune", 1))  # kernel decompositions chosen per level shape
            d.penalty_mode = int(pr.get("penalty_mode", Penalty.reference))
        h = C.c_void_p()
        check(load().tpss_batch_create(arr, len(problems), int(n_streams), C.byref(h)))
        self._h = h
        self.problems = list(problems)
        self.n_dofs = [pr["n_cells_fine"] ** pr["dim"] * (pr["degree"] + 1) ** pr["dim"] for pr in problems]

    def solve(self, us, fs, rel_tol=1e-8, abs_tol=1e-14, max_iter=200, stream=None):
        """us, fs: lists of float64 CUDA tensors; returns the CG iteration counts."""
        n = len(self.problems)
        assert len(us) == n and len(fs) == n
        U = (C.c_void_p * n)(*[_ptr(u, m).value for u, m in zip(us, self.n_dofs)])
        F = (C.c_void_p * n)(*[_ptr(f, m).value for f, m in zip(fs, self.n_dofs)])
        its = (C.c_int * n)()
        check(load().tpss_batch_solve(self._h, U, F, float(rel_tol), float(abs_tol), int(max_iter), its,
                                      _stream(stream)))
        return list(its)

    def __del__(self):
        try:
            if self._h:
                load().tpss_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass


def draw_batch_problems(count, seed, max_dofs_total, max_dofs_problem, dims=(2, 3), degrees=(2, 7),
                        cells=(8, 16, 32, 64)):
    """Seeded draw of independent Poisson problems for BatchSolver: dimension, degree k in
    [degrees[0], degrees[1]] and cells per direction uniformly from `cells` (one root cell).
    A draw is rejected and drawn again when its DoFs exceed max_dofs_problem, or when it would
    leave less of the budget max_dofs_total than the smallest problem needs for every problem
    still to be drawn. Returns (problems, rejected draws)."""
    rng = np.random.Generator(np.random.Philox(seed))
    n_min = min((n * (k + 1)) ** d for d in dims for k in range(degrees[0], degrees[1] + 1) for n in cells)
    if count * n_min > max_dofs_total:
        raise ValueError("max_dofs_total is below count times the smallest problem")
    problems, rejected, total = [], 0, 0
    while len(problems) < count:
        dim = int(rng.choice(dims))
        k = int(rng.integers(degrees[0], degrees[1] + 1))
        n = int(rng.choice(cells))
        N = (n * (k + 1)) ** dim
        if N > max_dofs_problem or total + N + (count - len(problems) - 1) * n_min > max_dofs_total:
            rejected += 1
            continue
        total += N
        problems.append(dict(dim=dim, degree=k, n_rep=1, n_cells_fine=n))
    return problems, rejected


class LocalSolver:
    """How the patch inverses are formed (tpss_precond_desc.local_solver)."""
    fd = 0       # fast diagonalization of the layout's (Cartesian or surrogate) 1-D problems
    exact = 1    # dense inverse of the exact patch matrix (basic state + InverseTable)
    ksum = 2     # FD of the Kronecker sum fitted to the exact patch matrix
    learned = 3  # surrogate 1-D problems corrected by a trained MLP
    ksvd = 4     # rank-2 Kronecker approximation of the exact patch matrix (CP/ALS), simultaneously diagonalized


class MLP:
    """Fully connected tanh network trained on the GPU by the library's own kernels."""

    def __init__(self, n_in, n_out, n_hidden=64, n_hidden_layers=3, seed=0):
        d = _lib.MlpDesc()
        d.n_in, d.n_out, d.n_hidden, d.n_hidden_layers, d.seed = n_in, n_out, n_hidden, n_hidden_layers, seed
        h = C.c_void_p()
        check(load().tpss_mlp_create(C.byref(d), C.byref(h)))
        self._h = h
        self.n_in, self.n_out = n_in, n_out
        n = C.c_int64()
        check(load().tpss_mlp_n_params(h, C.byref(n)))
        self.n_params = n.value

    @property
    def handle(self):
        return self._h

    def get_params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        check(load().tpss_mlp_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        check(load().tpss_mlp_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def forward(self, x, stream=None):
        import torch
        assert x.dtype == torch.float32 and x.is_cuda and x.shape[1] == self.n_in
        y = torch.empty((x.shape[0], self.n_out), dtype=torch.float32, device=x.device)
        check(load().tpss_mlp_forward(self._h, C.c_void_p(x.data_ptr()), x.shape[0],
                                      C.c_void_p(y.data_ptr()), _stream(stream)))
        return y

    def loss_grad(self, x, target):
        loss = C.c_double()
        g = np.zeros(self.n_params, dtype=np.float32)
        check(load().tpss_mlp_loss_grad(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(target.data_ptr()),
                                        x.shape[0], C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    def loss(self, x, target):
        loss = C.c_double()
        check(load().tpss_mlp_eval_loss(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(target.data_ptr()),
                                        x.shape[0], C.byref(loss)))
        return loss.value

    def train(self, x, target, epochs, batch=256, lr=1e-3, seed=0, stream=None):
        """Adam on shuffled mini-batches; returns the full-set loss after every epoch."""
        hist = np.zeros(max(epochs, 1))
        check(load().tpss_mlp_train(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(target.data_ptr()),
                                    x.shape[0], int(epochs), int(batch), float(lr), int(seed),
                                    hist.ctypes.data_as(C.POINTER(C.c_double)), _stream(stream)))
        return hist[:epochs]

    def __del__(self):
        try:
            if self._h:
                load().tpss_mlp_destroy(self._h)
                self._h = None
        except Exception:
            pass


def learned_sizes(subdomain_handler):
    a, b = C.c_int(), C.c_int()
    check(load().tpss_learned_sizes(subdomain_handler.handle, C.byref(a), C.byref(b)))
    return a.value, b.value


def learned_features(subdomain_handler, device="cuda"):
    """Network inputs of every patch of a distorted layout, [P, n_in] float32 on the device."""
    import torch
    n_in, _ = learned_sizes(subdomain_handler)
    x = torch.empty((subdomain_handler.n_subdomains(), n_in), dtype=torch.float32, device=device)
    check(load().tpss_learned_features(subdomain_handler.handle, C.c_void_p(x.data_ptr())))
    return x


def learned_targets(subdomain_handler, operator, ip_factor=1.0, device="cuda"):
    """Training targets of every patch, [P, n_out] float32 on the device."""
    import torch
    _, n_out = learned_sizes(subdomain_handler)
    y = torch.empty((subdomain_handler.n_subdomains(), n_out), dtype=torch.float32, device=device)
    check(load().tpss_learned_targets(subdomain_handler.handle, operator.handle, float(ip_factor),
                                      C.c_void_p(y.data_ptr())))
    return y


def local_matrices(subdomain_handler, operator, first, count, device="cuda"):
    """Exact patch matrices [count, n_loc, n_loc] (FP64) of patches first..first+count-1."""
    import torch
    n_loc = subdomain_handler.n_dofs_per_patch()
    out = torch.empty((count, n_loc, n_loc), dtype=torch.float64, device=device)
    check(load().tpss_local_matrices(subdomain_handler.handle, operator.handle, int(first), int(count),
                                     C.c_void_p(out.data_ptr())))
    return out


def kronecker_approx(mats, m, n, init, iterations=14, stream=None):
    """Low Kronecker-rank approximation K_i ~ sum_r F_{dim-1,r} x .. x F_{0,r} of a batch of
    matrices by alternating least squares (compute_kcp / compute_ksvd), on the GPU.

    mats: [count, prod(m), prod(n)] float64 CUDA tensor (direction 0 fastest in rows and columns);
    m, n: factor shapes per direction; init: per matrix the initial factors, a list over
    directions of [rank, m_d, n_d] float64 CUDA tensors of shape [count, rank, m_d, n_d].
    Returns the fitted factors in the same layout."""
    import torch
    dim = len(m)
    count = mats.shape[0]
    rank = init[0].shape[1]
    flat = torch.cat([f.reshape(count, -1) for f in init], dim=1).contiguous()
    mm = (C.c_int * 3)(*(list(m) + [1] * (3 - dim)))
    nn = (C.c_int * 3)(*(list(n) + [1] * (3 - dim)))
    check(load().tpss_kronecker_approx(C.c_void_p(mats.contiguous().data_ptr()), count, dim, mm, nn, rank,
                                       int(iterations), C.c_void_p(flat.data_ptr()), _stream(stream)))
    out, o = [], 0
    for d in range(dim):
        sz = rank * m[d] * n[d]
        out.append(flat[:, o:o + sz].reshape(count, rank, m[d], n[d]))
        o += sz
    return out


def precond_local_inverse(preconditioner, first, count, device="cuda"):
    """Dense local inverses [count, n_loc, n_loc] (FP64) that the preconditioner applies to the
    patches first..first+count-1 (without the damping)."""
    import torch
    n_loc = preconditioner.subdomain_handler.n_dofs_per_patch()
    out = torch.empty((count, n_loc, n_loc), dtype=torch.float64, device=device)
    check(load().tpss_precond_local_inverse(preconditioner.handle, int(first), int(count),
                                            C.c_void_p(out.data_ptr())))
    return out


def local_inverse_error(preconditioner, operator, first, count):
    """||A_j^-1 - B_j||_F / ||A_j^-1||_F per patch j (numpy array): A_j the exact patch matrix of
    the mapped level operator, B_j the preconditioner's local inverse."""
    err = np.zeros(count)
    check(load().tpss_local_inverse_error(preconditioner.handle, operator.handle, int(first), int(count),
                                          err.ctypes.data_as(C.POINTER(C.c_double))))
    return err


class MultigridSolver:
    """CG preconditioned by one GMG V-cycle with Schwarz smoothers on the unit cube."""

    def __init__(self, dim, degree, n_rep, n_cells_fine, patch_variant=PatchVariant.vertex,
                 smoother_variant=SmootherVariant.additive, relaxation=None, ip_factor=1.0,
                 precision=Precision.fp64, coarse_tol=1e-12, coarse_solver=0, use_graph=True,
                 vertex_coords=None, surrogate_n_q=5, local_solver=0, model=None,
                 auto_relaxation=False, vcycle_precision=Precision.fp64,
                 penalty_mode=Penalty.reference, autotune=False, fp64_level_mask=0):
        if relaxation is None:
            relaxation = lookup_damping_factor(patch_variant, smoother_variant, dim)
        d = _lib.MgDesc()
        if vertex_coords is not None:
            self._coords = np.ascontiguousarray(vertex_coords, dtype=np.float64)
            assert self._coords.shape == ((n_cells_fine + 1) ** dim, dim), "vertex_coords shape"
            d.vertex_coords = self._coords.ctypes.data_as(C.POINTER(C.c_double))
            d.surrogate_n_q = int(surrogate_n_q)
        d.local_solver = int(local_solver)
        d.model = model.handle if model is not None else None
        d.auto_relaxation = int(auto_relaxation)
        d.vcycle_precision = int(vcycle_precision)
        d.penalty_mode = int(penalty_mode)
        d.autotune = int(autotune)
        d.fp64_level_mask = int(fp64_level_mask)
        self._model = model
        d.dim, d.degree, d.n_rep, d.n_cells_fine = dim, degree, n_rep, n_cells_fine
        d.ip_factor, d.patch_variant, d.smoother_variant = float(ip_factor), patch_variant, smoother_variant
        d.relaxation, d.precision, d.coarse_tol = float(relaxation), precision, float(coarse_tol)
        d.coarse_solver, d.use_graph = int(coarse_solver), int(use_graph)
        h = C.c_void_p()
        check(load().tpss_mg_create(C.byref(d), C.byref(h)))
        self._h = h
        n = C.c_int64()
        check(load().tpss_mg_n_dofs(h, C.byref(n)))
        self._n = n.value
        nl = C.c_int()
        check(load().tpss_mg_n_levels(h, C.byref(nl)))
        self.n_levels = nl.value

    def n_dofs(self):
        return self._n

    def relaxation(self, level):
        """(damping, lambda_max estimate) of the smoother on level 1..L."""
        w, lam = C.c_double(), C.c_double()
        check(load().tpss_mg_relaxation(self._h, int(level), C.byref(w), C.byref(lam)))
        return w.value, lam.value

    def vmult(self, dst, src, stream=None):
        check(load().tpss_mg_vmult(self._h, _ptr(dst, self._n), _ptr(src, self._n), _stream(stream)))

    def solve(self, u, f, rel_tol=1e-8, abs_tol=1e-14, max_iter=100, stream=None):
        """CG solve of A u = f; returns (iterations, residual history)."""
        hist = np.zeros(max_iter + 1)
        it = C.c_int(0)
        code = load().tpss_mg_cg_solve(self._h, _ptr(u, self._n), _ptr(f, self._n), float(rel_tol),
                                       float(abs_tol), int(max_iter), C.byref(it),
                                       hist.ctypes.data_as(C.POINTER(C.c_double)), _stream(stream))
        check(code)
        return it.value, hist[: it.value + 1]

    def __del__(self):
        try:
            if self._h:
                load().tpss_mg_destroy(self._h)
                self._h = None
        except Exception:
            pass


def prolongate_add(dim, degree, n_cells_coarse, fine, coarse, stream=None):
    nc = (C.c_int * 3)(*(list(n_cells_coarse) + [1] * (3 - len(n_cells_coarse))))
    check(load().tpss_transfer_prolongate_add(dim, degree, nc, _ptr(fine), _ptr(coarse), _stream(stream)))


def restrict_add(dim, degree, n_cells_coarse, coarse, fine, stream=None):
    nc = (C.c_int * 3)(*(list(n_cells_coarse) + [1] * (3 - len(n_cells_coarse))))
    check(load().tpss_transfer_restrict_add(dim, degree, nc, _ptr(coarse), _ptr(fine), _stream(stream)))
