/*
 * tpss_gpu.h -- C ABI of the GB300 (sm_103a) Schwarz-smoother library.
 *
 * This is the drop-in boundary for the TPSS Schwarz smoother path (jwitte08/TPSS):
 * SchwarzPreconditioner / SchwarzSmoother applied on one multigrid level, with the
 * SubdomainHandler's patch layout, coloring and damping semantics, plus the matrix-free SIPG
 * operator, DG level transfer and CG + V-cycle that the smoother runs inside.
 *
 * Conventions
 *  - Every entry point returns an int status (TPSS_OK == 0) and never aborts;
 *    tpss_last_error() gives a message for the calling thread's last failure.
 *  - Vectors passed to *_vmult / *_step / *_solve are DEVICE pointers to FP64 arrays in the
 *    layout's DoF numbering (cell-wise blocks of (k+1)^dim lexicographic DoFs, the deal.II
 *    FE_DGQ level numbering); the library owns all other device memory behind opaque handles.
 *  - Work is ordered on the caller's stream (a cudaStream_t passed as void*; NULL = legacy
 *    default stream).  Handles are not reentrant: one stream at a time per handle, as the
 *    reference's SchwarzPreconditioner::vmult is const but mutates timers and scratch
 *    (schwarz_preconditioner.h:184-236).
 *  - No torch or deal.II types appear here; plain pointers and sizes only.
 */
#ifndef TPSS_GPU_H
#define TPSS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define TPSS_OK 0
#define TPSS_ERR_INVALID_ARGUMENT 1
#define TPSS_ERR_NOT_IMPLEMENTED 2 /* reference throws ExcMessage("TODO ...") here too */
#define TPSS_ERR_CUDA 3
#define TPSS_ERR_OUT_OF_MEMORY 4
#define TPSS_ERR_NOT_FINITE 5 /* AssertIsFinite(dst.l2_norm()) of schwarz_preconditioner.templates.h:238 */
#define TPSS_ERR_NOT_CONVERGED 6
#define TPSS_ERR_STATE 7

/* TPSS::DoFLayout (TPSS/TPSS.h) */
#define TPSS_DOF_DGQ 0
/* TPSS::PatchVariant */
#define TPSS_PATCH_CELL 0
#define TPSS_PATCH_VERTEX 1
/* TPSS::SmootherVariant */
#define TPSS_ADDITIVE 0
#define TPSS_MULTIPLICATIVE 1
/* arithmetic of the smoother (gather, local solve, scatter); vectors stay FP64 */
/* local solvers (tpss_precond_desc.local_solver) */
#define TPSS_LOCAL_FD 0      /* fast diagonalization of the layout's 1-D patch problems
                                (Cartesian, or surrogate patches on a distorted level) */
#define TPSS_LOCAL_EXACT 1   /* dense inverse of the exact patch matrix (TensorProductMatrix
                                basic state + InverseTable); needs the mapped level operator,
                                at most 160 DoFs per patch */
#define TPSS_LOCAL_KSUM 2    /* fast diagonalization of the Kronecker sum closest to the
                                exact patch matrix with the surrogate masses fixed (low
                                Kronecker-rank approximation, kroneckersvd.h:207-402); needs
                                the mapped level operator */
#define TPSS_LOCAL_LEARNED 3 /* surrogate 1-D problems corrected by a trained network
                                (tpss_mlp) from the patch's vertex geometry */
#define TPSS_LOCAL_KSVD 4    /* rank-2 Kronecker approximation of the exact patch matrix
                                (CP/ALS, compute_kcp / compute_ksvd, kroneckersvd.h:306-585),
                                inverted by simultaneous diagonalization of its two terms
                                (fast diagonalization with eigenvalue combinations
                                1 + prod_d mu_d); patches whose fit is not safely positive
                                definite keep the surrogate; needs the mapped level operator */

#define TPSS_FP64 0
#define TPSS_FP32 1

/* SIPG penalty (tpss_precond_desc / tpss_mg_desc .penalty_mode, tpss_operator_create_penalty).
 * The operator and the local solvers of one level must use the same mode. */
#define TPSS_PENALTY_REFERENCE 0 /* the reference's: sigma = ip*gamma*(1/h_l+1/h_r)/2 on interior
                                    faces, 2*ip*gamma/h on Dirichlet faces, gamma = k(k+1)
                                    (apps/common_integrator.h:30-37,
                                    apps/laplace_integrator.h:134-148, 649-654, 691-693) */
#define TPSS_PENALTY_2KP1SQ 1    /* sigma = ip*2(k+1)^2*(1/h_l+1/h_r)/2 on interior faces and
                                    ip*2(k+1)^2/h on Dirichlet faces: "2(k+1)^2/h" on every face
                                    of a uniform mesh (no counterpart in the reference, whose
                                    formula cannot give this on both face kinds with one ip) */

typedef struct tpss_layout tpss_layout;
typedef struct tpss_operator tpss_operator;
typedef struct tpss_precond tpss_precond;
typedef struct tpss_smoother tpss_smoother;
typedef struct tpss_mg tpss_mg;
typedef struct tpss_mlp tpss_mlp;

/*
 * Patch layout of one level: replaces SubdomainHandler::reinit
 * (TPSS/subdomain_handler.templates.h:3-154) with PatchInfo vertex/cell patch gathering
 * (TPSS/patch_info.templates.h:59-409), the user coloring (apps/coloring.h:347-401 tiled
 * 2^dim colors for vertex patches; one color for additive cell patches; two red-black colors
 * for multiplicative cell patches), interior-before-boundary order within a color
 * (patch_info.templates.h:605-680) and DoFInfo's cell-wise DoF caching
 * (TPSS/dof_info.templates.h:44-182).
 */
typedef struct tpss_layout_desc
{
  int dim;              /* 2 or 3 */
  int degree;           /* k, 1..7 */
  int dof_layout;       /* TPSS_DOF_DGQ */
  int patch_variant;    /* TPSS_PATCH_VERTEX or TPSS_PATCH_CELL */
  int smoother_variant; /* TPSS_ADDITIVE or TPSS_MULTIPLICATIVE (selects the coloring) */
  int n_cells[3];       /* cells per direction of the structured (Cartesian) level */
  const double *cell_h[3];        /* host: n_cells[d] cell widths per direction; NULL = 1/n */
  const int64_t *cell_dof_start;  /* host: first DoF of each lexicographic cell (x fastest);
                                     NULL = cell index * (k+1)^dim */
  const int32_t *patch_color;     /* host: optional user coloring, one entry per patch in the
                                     default patch order (tpss_layout_patches); NULL = default */
  const double *vertex_coords;    /* host, optional: coordinates of the (n_cells[d]+1) vertices per
                                     direction (lexicographic, x fastest, dim values each) of a
                                     distorted mesh with trilinear cells.  Vertex patches then use
                                     surrogate Cartesian widths: the average arc length between
                                     opposite faces (MappingInfo, TPSS/mapping_info.templates.h:42-240,
                                     use_arc_length = true, no volume normalization) */
  int surrogate_n_q;              /* Gauss-Lobatto points per direction for the arc lengths; 0 = 5 */
} tpss_layout_desc;

/* Replaces SubdomainHandler<dim,Number>::reinit (TPSS/subdomain_handler.h:33-225). */
int tpss_layout_create(const tpss_layout_desc *desc, tpss_layout **out);
/* SchwarzPreconditioner::m() (schwarz_preconditioner.h:153-163) and PartitionData counts. */
int tpss_layout_info(const tpss_layout *layout, int64_t *n_dofs, int64_t *n_patches,
                     int *n_colors);
/* Host copy of the patch list: lower cell coordinate (3 ints, unused directions 0) and color
 * of each patch in storage order (colors ascending, interior patches first). */
int tpss_layout_patches(const tpss_layout *layout, int32_t *lower_cells, int32_t *colors);
void tpss_layout_destroy(tpss_layout *layout);

/*
 * Matrix-free SIPG Laplace operator of one level (apps/laplace_integrator.h:578-743):
 * dst = A src with interior penalty ip*gamma*(1/h_in+1/h_out)/2 and Dirichlet boundary
 * penalty 2*ip*gamma/h, gamma = k(k+1) (apps/common_integrator.h:30-37).
 */
int tpss_operator_create(const tpss_layout *layout, double ip_factor, tpss_operator **out);
/* The same with a TPSS_PENALTY_* mode (tpss_operator_create uses TPSS_PENALTY_REFERENCE). */
int tpss_operator_create_penalty(const tpss_layout *layout, double ip_factor, int penalty_mode,
                                 tpss_operator **out);
/* MF::Operator::vmult (apps/laplace_integrator.h:578-598), FP64. */
int tpss_operator_vmult(tpss_operator *op, double *dst, const double *src, void *stream);
/* The same product in FP32 arithmetic on FP64 vectors (src is converted once into a scratch
 * copy owned by the operator; dst is written in FP64): the level operator of a single-precision
 * V-cycle (no counterpart in the reference, which runs its multigrid in the vector precision).
 * On distorted (mapped) levels the block-sparse matrix gets an FP32 copy on first use. */
int tpss_operator_vmult_fp32(tpss_operator *op, double *dst, const double *src, void *stream);
void tpss_operator_destroy(tpss_operator *op);

/* SchwarzPreconditioner::AdditionalData (schwarz_preconditioner.h:495-515) plus the
 * local-solver and arithmetic choices. */
typedef struct tpss_precond_desc
{
  double relaxation;           /* local damping omega (> 0) */
  int reverse;                 /* reverse color sequence (multiplicative) */
  int symmetrized;             /* forward + backward color sweep (multiplicative) */
  int use_ras_weights;         /* divide local solutions by patch multiplicity (additive) */
  int use_ras_boolean_weights; /* restricted prolongation (rscatter_add): every DoF is added by
                                  one patch only, the one where it lies closest to the patch
                                  centre (dof_info.templates.h:194-313); additive vertex patches,
                                  FD local solvers (cell patches: TPSS_ERR_NOT_IMPLEMENTED) */
  int precision;               /* TPSS_FP64 or TPSS_FP32 smoother arithmetic */
  double ip_factor;            /* EquationData::ip_factor of the local SIPG matrices */
  int check_finite;            /* 1: vmult checks that dst is finite (one extra reduction) */
  int kernel_variant;          /* additive smoother kernel: TPSS_KERNEL_AUTO, TPSS_KERNEL_COLOR
                                  (one fused launch per color) or TPSS_KERNEL_STREAM (3D vertex
                                  patches, FP32, k <= 5 -- per-patch 1-D problems of distorted
                                  levels k <= 3: column-streamed, one pass) */
  int stream_variant;          /* initial work decomposition of the smoother kernel (see
                                  tpss_precond_autotune): 0..5 for the column-streamed kernel
                                  (6, 7: plane passes in registers, degree 4 only; other
                                  degrees use 0 instead),
                                  0..2 (patches per CTA x1, x2, x4) for the per-color kernel, which
                                  uses 0 where the level offers fewer; 0 by default */
  int local_solver;            /* TPSS_LOCAL_*: how the patch inverses are formed */
  const tpss_mlp *model;       /* trained network for TPSS_LOCAL_LEARNED, else NULL */
  int penalty_mode;            /* TPSS_PENALTY_* of the local SIPG matrices (0: the reference) */
} tpss_precond_desc;

#define TPSS_KERNEL_AUTO 0
#define TPSS_KERNEL_COLOR 1
#define TPSS_KERNEL_STREAM 2

/*
 * SchwarzPreconditioner::initialize(subdomain_handler, operator, additional_data)
 * (schwarz_preconditioner.templates.h:1-60): assembles the 1-D SIPG mass/Laplace matrices of
 * every patch and direction (FD::MatrixIntegrator::assemble_subspace_inverses,
 * apps/laplace_integrator.h:226-250) and solves their generalized eigenproblems in FP64 on
 * the GPU.  `op` is the level operator (required for TPSS_MULTIPLICATIVE, may be NULL for
 * additive); it is not owned and must outlive the preconditioner.
 */
int tpss_precond_create(const tpss_layout *layout, tpss_operator *op,
                        const tpss_precond_desc *desc, tpss_precond **out);
/* Shallow copy with different AdditionalData (schwarz_preconditioner.templates.h:63-86):
 * shares the layout and local solvers of `other`. */
int tpss_precond_create_shallow(const tpss_precond *other, const tpss_precond_desc *desc,
                                tpss_precond **out);
/* SchwarzPreconditioner::vmult (schwarz_preconditioner.templates.h:209-239): dst is set to
 * zero and receives sum over colors of omega R_j^T A_j^-1 R_j src. */
int tpss_precond_vmult(tpss_precond *p, double *dst, const double *src, void *stream);
/* vmult_add (schwarz_preconditioner.templates.h:185-194): dst += P src. */
int tpss_precond_vmult_add(tpss_precond *p, double *dst, const double *src, void *stream);
/* Tvmult: the reference throws "TODO transpose operation is not implemented"; so does this
 * (TPSS_ERR_NOT_IMPLEMENTED). */
int tpss_precond_Tvmult(tpss_precond *p, double *dst, const double *src, void *stream);

/*
 * Allocation-free vmult.  This entry point has no counterpart in the reference.
 *
 * Same result as tpss_precond_vmult for additive vertex patches in 3D with FP32 arithmetic,
 * degree <= 4, on a Cartesian level (the column-streamed smoother), but the call allocates
 * and frees no device memory.  It is meant for callers that may not allocate once their solve
 * has started: a host application that owns all device memory through its own pool and
 * forbids library-side cudaMalloc/cudaFree after setup, or one that cannot afford the device
 * synchronization of cudaFree or an out-of-memory failure in the middle of an iteration.
 * (tpss_precond_vmult grows its scratch buffer with cudaMalloc on first use.)
 *
 * The scratch for the partial sums of cells shared between work items is a fixed device array
 * of 32 MiB (8 Mi floats), held by every GPU that loads the library until the process exits.
 * A level whose scratch need exceeds it is rejected with TPSS_ERR_INVALID_ARGUMENT; 3D DGQ4
 * fits up to 33^3 cells.  Everything else the call uses (index tables, FD data) was
 * allocated when the preconditioner was created.
 *
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.  All calls share the
 * array and it keeps the last call's contents; every entry a call reads is written by the same
 * call first, so nothing needs clearing, but calls that overlap on the GPU (for example on two
 * streams at once) race on it.
 *
 * Differences from tpss_precond_vmult: the preconditioner must have been created with
 * check_finite = 0 (the check's flag would need a buffer) and a kernel_variant other than
 * TPSS_KERNEL_COLOR, else the call returns TPSS_ERR_INVALID_ARGUMENT; dense (TPSS_LOCAL_EXACT)
 * and per-patch (fitted, learned) local solvers are rejected the same way; the call is not
 * recorded in the preconditioner's timers (tpss_precond_time_info).
 */
int tpss_precond_vmult_static_scratch(tpss_precond *p, double *dst, const double *src, void *stream);

/* Autotuner (no counterpart in the reference): times every work decomposition of the smoother
 * kernel for this level (for the column-streamed kernel: pencils per thread, vertex layers per
 * work item and, for degree 4, pencil or plane passes; for the per-color kernel, which serves 2D, cell patches, FP64, k > 4 and the
 * multiplicative smoother: 1, 2 or 4 times its base number of patches per CTA, as far as 512
 * threads and 200 KB of shared memory allow) on the caller's vectors, `reps` applications each,
 * and keeps the fastest for later vmult calls.  On return dst = P src, *chosen is the selected variant, ms_per_variant (optional,
 * >= 8 entries) the measured milliseconds per application and *n_variants their count (1 when the
 * level has a single kernel). */
/* vmult with dst and src in HOST memory (the reference's vmult on host vectors; a device-vector
 * adapter would copy in, apply and copy out). For the streamed smoother the copies are pipelined
 * with the kernel along z (three internal streams), in chunks of one work item deep; the pipeline
 * runs the 4-layer-deep decomposition of the chosen kind (variant 5 when variant 4 or 5 is chosen,
 * 7 when 6 or 7 is chosen, else 2) for a short fill and drain, so its result carries that variant's FP32 rounding.
 * Otherwise copy-in, vmult, copy-out on `stream`. Stream-ordered: dst is complete when `stream`
 * reaches this point. Pin the host buffers (cudaHostRegister / cudaMallocHost) for the copies to
 * overlap. */
int tpss_precond_vmult_host(tpss_precond *p, double *dst, const double *src, void *stream);
int tpss_precond_autotune(tpss_precond *p, double *dst, const double *src, int reps, int *chosen,
                          double *ms_per_variant, int *n_variants, void *stream);

/* TimeInfo (TPSS/time_info.h:23-64): the five preconditioner timers of
 * schwarz_preconditioner.templates.h:22-26, in seconds, measured with CUDA events. */
typedef struct tpss_time_info
{
  double time;
  int64_t n_calls;
  char description[64];
} tpss_time_info;
int tpss_precond_time_info(tpss_precond *p, tpss_time_info *out, int *n_inout);
void tpss_precond_destroy(tpss_precond *p);

/*
 * SchwarzSmoother / SmootherRichardson (smoother/schwarz_smoother.h:16-52,
 * smoother/smoother_richardson.h:41-156): step computes x += damping * P (b - A x)
 * n_steps times; vmult sets x = 0 first.  Neither the operator nor the preconditioner is
 * owned.
 */
int tpss_smoother_create(tpss_operator *op, tpss_precond *p, int n_steps, double damping,
                         tpss_smoother **out);
int tpss_smoother_step(tpss_smoother *s, double *x, const double *b, void *stream);
int tpss_smoother_vmult(tpss_smoother *s, double *x, const double *b, void *stream);
void tpss_smoother_destroy(tpss_smoother *s);

/*
 * Geometric multigrid on the unit cube (apps/poisson_problem.h:642-755,
 * apps/multigrid.h:201-399): n_rep^dim root cells refined to n_cells_fine per direction,
 * SIPG level operators, DG embedding transfer, Schwarz pre/post smoothers on levels >= 1,
 * coarse CG to an absolute residual of coarse_tol on level 0, one V-cycle per application.
 */
typedef struct tpss_mg_desc
{
  int dim, degree;
  int n_rep;          /* root cells per direction */
  int n_cells_fine;   /* n_rep * 2^L */
  double ip_factor;
  int patch_variant, smoother_variant;
  double relaxation;  /* Schwarz local damping */
  int precision;      /* smoother arithmetic, TPSS_FP64 / TPSS_FP32 */
  double coarse_tol;  /* absolute; reference default 1e-12 (apps/multigrid.h:82-91) */
  int coarse_solver;  /* 0: CG to coarse_tol (CoarseGridParameter IterativeAcc, the reference
                         default); 1: dense inverse of the coarse matrix (the FullSVD variant of
                         apps/multigrid.h:176-182), which lets the whole V-cycle be one graph */
  int use_graph;      /* capture the V-cycle in CUDA graphs (one graph with the dense coarse
                         solver; down- and up-sweep graphs around the CG coarse solve) */
  const double *vertex_coords; /* NULL: Cartesian unit cube. Else the finest level's vertices,
                                  lexicographic (x fastest), dim coordinates each: every level
                                  is a distorted (multilinear) mesh whose vertices are every
                                  2^(L-l)-th finest vertex, with the mapped SIPG operator and
                                  surrogate-patch local solvers (create_distorted_cube,
                                  apps/mesh.h:160-200; mapping_info.templates.h:42-240) */
  int surrogate_n_q;           /* Gauss-Lobatto points of the surrogate arc lengths (0: 5) */
  int local_solver;            /* TPSS_LOCAL_* of the level smoothers (distorted levels) */
  const tpss_mlp *model;       /* trained network for TPSS_LOCAL_LEARNED */
  int auto_relaxation;         /* 0: every level uses `relaxation` (the reference). 1: a level
                                  whose smoother spectrum lambda_max(P A) exceeds the Cartesian
                                  2^dim is damped by relaxation * 2^dim / (1.05 lambda_max),
                                  lambda_max from 30 power steps at setup (no counterpart in
                                  the reference) */
  int vcycle_precision;        /* TPSS_FP64 (the reference) or TPSS_FP32: inside the V-cycle the
                                  level operators of the smoothing residuals and the transfers
                                  compute in FP32 (tpss_operator_vmult_fp32); the outer CG
                                  operator and the coarse solve stay FP64 (no counterpart in the
                                  reference, whose multigrid runs in the vector precision) */
  int penalty_mode;            /* TPSS_PENALTY_* of every level's operator and local solvers */
  int fp64_level_mask;         /* bit l set: the smoother of level l computes in FP64 whatever
                                  `precision` says (a mixed-precision hierarchy; 0 = none) */
  int autotune;                /* 1: every level's smoother kernel decomposition is chosen by the
                                  autotuner (tpss_precond_autotune) at setup; levels of a shape
                                  tuned before in this process (e.g. in another problem of a
                                  batch) reuse that choice (no counterpart in the reference) */
} tpss_mg_desc;

int tpss_mg_create(const tpss_mg_desc *desc, tpss_mg **out);
/* Finest-level vector size. */
int tpss_mg_n_dofs(const tpss_mg *mg, int64_t *n_dofs);
/* PreconditionMG::vmult: dst = V-cycle(src) on the finest level. */
int tpss_mg_vmult(tpss_mg *mg, double *dst, const double *src, void *stream);
/* SolverCG with ReductionControl (apps/poisson_problem.h:726-755, apps/rt_parameter.h:39-41):
 * solves A u = f (u := 0 first), stopping when ||r|| <= max(abs_tol, rel_tol ||r_0||).
 * On return *iterations holds the CG iteration count and res_history (host, length
 * max_iter+1, may be NULL) the residual norms. With use_graph and the dense coarse solve the
 * iteration loop runs on the device: one CUDA graph (a conditional WHILE node whose body is one
 * CG iteration and a one-thread kernel that tests the residual), captured at tpss_mg_create and
 * launched once per solve, so a solve synchronizes with the host once; otherwise the host
 * reads the residual norm every iteration. Both run the same kernels in the same order. */
int tpss_mg_cg_solve(tpss_mg *mg, double *u, const double *f, double rel_tol, double abs_tol,
                     int max_iter, int *iterations, double *res_history, void *stream);
/* Batched solves (no counterpart in the reference, which runs one problem per process): many
 * independent hierarchies (each described by a tpss_mg_desc with the dense coarse solve and
 * use_graph = 1) solved by CG concurrently -- every problem's device-side CG loop (see
 * tpss_mg_cg_solve) is launched once on one of n_streams streams, the problems dealt largest
 * first to the least-loaded stream, and one host synchronization at the end reads all
 * iteration counts. Each problem's result is the one its own tpss_mg_cg_solve gives.
 * iterations: n_problems entries (-1 if a problem did not converge within max_iter, which also
 * returns TPSS_ERR_NOT_CONVERGED). */
typedef struct tpss_batch tpss_batch;
int tpss_batch_create(const tpss_mg_desc *descs, int n_problems, int n_streams, tpss_batch **out);
int tpss_batch_problem(tpss_batch *b, int i, tpss_mg **mg);
int tpss_batch_solve(tpss_batch *b, double *const *u, const double *const *f, double rel_tol,
                     double abs_tol, int max_iter, int *iterations, void *stream);
void tpss_batch_destroy(tpss_batch *b);

/* Damping used by the smoother of level 1..L and, with auto_relaxation, the estimate of
 * lambda_max(P A) it was scaled by (0 otherwise). No counterpart in the reference. */
int tpss_mg_relaxation(const tpss_mg *mg, int level, double *relaxation, double *lambda_max);
/* Level objects for direct use (level 0 = coarsest). The hierarchy's CUDA graphs (V-cycle,
 * device CG loop) are captured at creation or first use with the levels' settings of that
 * time; later changes to a level object are not seen by them. */
int tpss_mg_level(tpss_mg *mg, int level, tpss_layout **layout, tpss_operator **op,
                  tpss_precond **precond);
int tpss_mg_n_levels(const tpss_mg *mg, int *n_levels);
void tpss_mg_destroy(tpss_mg *mg);

/* DG level transfer between lexicographic structured levels (MGTransferMatrixFree for DGQ):
 * fine += P coarse (prolongate_and_add), coarse += P^T fine (restrict_and_add). */
int tpss_transfer_prolongate_add(int dim, int degree, const int *n_cells_coarse,
                                 double *fine, const double *coarse, void *stream);
int tpss_transfer_restrict_add(int dim, int degree, const int *n_cells_coarse, double *coarse,
                               const double *fine, void *stream);

/* Measurement helper with no counterpart in the reference: FMA-pipe throughput of the
 * current GPU in FLOP/s for TPSS_FP32 or TPSS_FP64 (8 independent FMA chains per thread on
 * every SM, `iters` FMAs per chain, timed with CUDA events).  The roofline denominator of the
 * CUDA-core-bound fast-diagonalization kernels. */
/* ---------------------------------------------------------------------------------------
 * C0 interior-penalty biharmonic problem (apps/biharmonic_integrator.h, biharmonic_problem.h):
 * clamped, FE_Q(k) on Gauss-Lobatto nodes, 2D unit square with n_rep * 2^L cells per direction.
 * Vectors hold the interior nodes (n k - 1)^2, x fastest, FP64 on the device. Level -1 is the
 * finest. The additive vertex-patch smoother (2k-1)^2 nodes per patch, 4 colors) uses
 * TPSS_LOCAL_EXACT (dense inverse of the patch matrix, LocalSolverVariant::Exact) or
 * TPSS_LOCAL_FD (fast diagonalization of the patch matrix without the mixed-derivative
 * term, LocalSolverVariant::Bilaplacian).
 * ------------------------------------------------------------------------------------- */
typedef struct tpss_c0ip tpss_c0ip;
/* tpss_c0ip_desc.problem: the form on the FE_Q node grid */
#define TPSS_C0IP_BIHARMONIC 0 /* the clamped C0IP biharmonic form above */
#define TPSS_Q_POISSON 1       /* the Poisson problem with continuous FE_Q(k) (Dirichlet): the
                                  Laplacian A = M x L + L x M on the interior nodes, vertex patches
                                  of the (2k-1)^2 nodes inside their 2 x 2 cells (the Q layout of
                                  TPSS/dof_info.h:344-355, TPSS/patch_dof_worker.h:265-300;
                                  apps/laplace_integrator.h:800-1198 for the CFEM operator); the
                                  fast-diagonalization local solver is exact here */
typedef struct tpss_c0ip_desc
{
  int degree;          /* 2..7 */
  int n_rep;           /* coarse cells per direction (>= 2) */
  int n_cells_fine;    /* n_rep * 2^L */
  double ip_factor;    /* EquationData::ip_factor */
  int local_solver;    /* TPSS_LOCAL_EXACT or TPSS_LOCAL_FD */
  int precision;       /* smoother arithmetic, TPSS_FP64 / TPSS_FP32 */
  double relaxation;   /* Schwarz damping (vertex patches, 2D: 0.25 in TPSS.h:121-163) */
  int problem;         /* TPSS_C0IP_BIHARMONIC (0) or TPSS_Q_POISSON */
} tpss_c0ip_desc;

int tpss_c0ip_create(const tpss_c0ip_desc *desc, tpss_c0ip **out);
int tpss_c0ip_info(const tpss_c0ip *c, int level, int64_t *n_dofs, int *n_levels);
int tpss_c0ip_operator_vmult(tpss_c0ip *c, int level, double *dst, const double *src, void *stream);
/* dst = relaxation * sum_j R_j^T A_j^-1 R_j src on level 1..L (SchwarzPreconditioner::vmult) */
int tpss_c0ip_smoother_vmult(tpss_c0ip *c, int level, double *dst, const double *src, void *stream);
/* CG + one V-cycle per iteration (dense coarse solve), ReductionControl semantics */
int tpss_c0ip_cg_solve(tpss_c0ip *c, double *u, const double *f, double rel_tol, double abs_tol,
                       int max_iter, int *iterations, double *res_history, void *stream);
void tpss_c0ip_destroy(tpss_c0ip *c);

/* ---------------------------------------------------------------------------------------
 * Learned local solver (no counterpart in the reference: its distorted-mesh local solver is
 * the surrogate patch of mapping_info.templates.h:42-240). A small fully connected network
 * (tanh hidden layers, linear output, FP32) maps a vertex patch's geometry to corrections of
 * the surrogate 1-D problems; it is trained on the GPU against the Kronecker-sum fit of the
 * exact patch matrices and used through tpss_precond_desc.local_solver = TPSS_LOCAL_LEARNED.
 * All x / y / target arrays are device pointers, row-major [rows][width], FP32.
 * ------------------------------------------------------------------------------------- */
typedef struct tpss_mlp_desc
{
  int n_in, n_hidden, n_hidden_layers, n_out;
  uint64_t seed;               /* Glorot-uniform initialisation */
} tpss_mlp_desc;

int tpss_mlp_create(const tpss_mlp_desc *desc, tpss_mlp **out);
int tpss_mlp_sizes(const tpss_mlp *m, int *n_in, int *n_out);
/* parameters: per layer W [out][in] row-major then b [out] (host arrays of n_params floats) */
int tpss_mlp_n_params(const tpss_mlp *m, int64_t *n_params);
int tpss_mlp_get_params(const tpss_mlp *m, float *host);
int tpss_mlp_set_params(tpss_mlp *m, const float *host);
int tpss_mlp_forward(tpss_mlp *m, const float *x, int64_t rows, float *y, void *stream);
/* mean squared error over rows x n_out outputs and its gradient (host, n_params floats) */
int tpss_mlp_loss_grad(tpss_mlp *m, const float *x, const float *target, int64_t rows, double *loss,
                       float *grad_host);
int tpss_mlp_eval_loss(tpss_mlp *m, const float *x, const float *target, int64_t rows, double *loss);
/* Adam on mini-batches of a seeded permutation; loss_per_epoch (host, may be NULL) receives the
 * full-set loss after every epoch */
int tpss_mlp_train(tpss_mlp *m, const float *x, const float *target, int64_t rows, int epochs,
                   int batch, double lr, uint64_t seed, double *loss_per_epoch, void *stream);
void tpss_mlp_destroy(tpss_mlp *m);

/* network sizes for a layout's vertex patches: n_in = 3^d d + 2d, n_out = d n (n+1) / 2 */
int tpss_learned_sizes(const tpss_layout *layout, int *n_in, int *n_out);
/* features of every patch of a distorted layout (P x n_in, device) */
int tpss_learned_features(const tpss_layout *layout, float *x);
/* training targets of every patch (P x n_out, device): the surrogate-basis correction that the
 * Kronecker-sum fit of the exact patch matrix gives; needs the mapped level operator */
int tpss_learned_targets(const tpss_layout *layout, const tpss_operator *op, double ip_factor,
                         float *y);
/* exact patch matrices of patches [first, first + count) (count x n_loc x n_loc, row-major,
 * patch-local lexicographic DoFs, device FP64) from the mapped level operator */
int tpss_local_matrices(const tpss_layout *layout, const tpss_operator *op, int64_t first,
                        int64_t count, double *out);
/* Low Kronecker-rank approximation of a batch of matrices on the GPU (compute_kcp /
 * compute_ksvd, TPSS/kroneckersvd.h:306-402, 501-585): K_i ~ sum_r F_{dim-1,r} x .. x F_{0,r}
 * with factors F_{d,r} of m[d] x n[d] (dim = 2 or 3, rank <= 4) by `iterations` alternating
 * least-squares sweeps (rank^2 + 10 in the reference) from the initial factors given in
 * `factors`, which receives the result. mats: count x prod(m) x prod(n), row-major, direction 0
 * fastest in rows and columns; factors: per matrix, per direction d, per term r an m[d] x n[d]
 * row-major block (device FP64). */
int tpss_kronecker_approx(const double *mats, int64_t count, int dim, const int *m, const int *n,
                          int rank, int iterations, double *factors, void *stream);
/* The local inverses a preconditioner applies, as dense matrices: patches [first, first + count),
 * count x n_loc x n_loc row-major device FP64 (S diag(1/sum lambda) S^T of its fast-diagonalization
 * tables, or the stored dense inverses of TPSS_LOCAL_EXACT). TensorProductMatrix::as_inverse_table
 * for the separable state (tensor_product_matrix.h), without the damping. */
int tpss_precond_local_inverse(const tpss_precond *p, int64_t first, int64_t count, double *out);
/* Measured local inverse error (no counterpart in the reference): err[i] (host) =
 * ||A_j^-1 - B_j||_F / ||A_j^-1||_F for the patches j = first + i, A_j the exact patch matrix
 * of the mapped level operator `op` (inverted in FP64 on the GPU) and B_j the preconditioner's
 * local inverse (tpss_precond_local_inverse). */
int tpss_local_inverse_error(const tpss_precond *p, const tpss_operator *op, int64_t first,
                             int64_t count, double *err);

int tpss_diag_fma_peak(int precision, int iters, double *flops_per_second, void *stream);

const char *tpss_last_error(void);
/* Library version string. */
const char *tpss_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TPSS_GPU_H */
