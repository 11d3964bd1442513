/*
 * tpss_oracle.c -- CPU oracle for the TPSS Schwarz-smoother hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library under tpss_gb300/)
 * links, loads or calls this file.  It is loaded by tests/, by __graft_entry__.smoke() and
 * by bench.py's CPU-baseline leg, and only there as the checker / the timed CPU baseline.
 *
 * It is a plain-C, FP64 restatement of the reference algorithm (jwitte08/TPSS, which is
 * header-only C++ on top of deal.II; deal.II is not available, so its arithmetic on the path
 * is restated from the published method):
 *
 *  - 1-D shape data of FE_DGQ(k): Lagrange polynomials on the k+1 Gauss-Lobatto points,
 *    integrated with the (k+1)-point Gauss rule (FDEvaluation, TPSS/fd_evaluation.h:33-446,
 *    TPSS/fd_evaluation.templates.h:1-102).
 *  - 1-D patch matrices of the fast-diagonalization local solvers: cell mass and Laplace
 *    (apps/common_integrator.h:159-192, 300-343), SIPG face and interface terms
 *    (apps/common_integrator.h:194-293) with penalty 2*gamma*(0.5/h_l+0.5/h_r),
 *    gamma = k(k+1) (apps/common_integrator.h:30-37) and average factor 1 on the physical
 *    boundary, 1/2 elsewhere (TPSS/fd_evaluation.h:651-688), assembled as in
 *    FDEvaluation::patch_action (TPSS/fd_evaluation.templates.h:168-281) and selected by
 *    FD::MatrixIntegrator::assemble_subspace_inverses (apps/laplace_integrator.h:226-250).
 *  - The separable local solver (deal.II TensorProductMatrixSymmetricSum, selected at
 *    apps/poisson_problem.h:77): per direction the generalized eigenproblem
 *    A_d s = lambda M_d s with S_d^T M_d S_d = I, solved here by Cholesky of M_d followed by
 *    cyclic Jacobi (Golub & Van Loan, Matrix Computations, 4th ed., Alg. 8.5.3), and the
 *    inverse u = (S_d x..x S_1) (Lambda_1 (+) .. (+) Lambda_d)^-1 (S_d x..x S_1)^T r applied
 *    by sum factorization with direction 0 running fastest (TPSS/tensors.h:63-82, 760-795).
 *  - Patch layout: vertex patches around interior vertices with their 2^d cells in
 *    lexicographic order (TPSS/patch_info.templates.h:176-409, esp. 389-402), cell patches
 *    (patch_info.templates.h:59-173); patch-local DG index cell_no*(k+1)+i
 *    (TPSS/dof_info.h:358-369); tiled 2^d-coloring of vertex patches (apps/coloring.h:347-401);
 *    interior patches before boundary patches within a color (patch_info.templates.h:605-680).
 *  - Additive and multiplicative Schwarz vmult with relaxation and RAS weights
 *    (preconditioner/schwarz_preconditioner.templates.h:126-165, 585-732, .h:532-567).
 *  - Matrix-free SIPG operator (apps/laplace_integrator.h:613-743), written as the Kronecker
 *    sum of global 1-D operators, which is exact on Cartesian meshes.
 *  - DG level transfer (polynomial embedding), V-cycle, coarse CG, PCG with
 *    deal.II Multigrid / SolverCG / ReductionControl semantics
 *    (apps/poisson_problem.h:642-755, apps/multigrid.h:137-197,
 *    smoother/smoother_richardson.h:118-156, apps/postprocess.h:41-60).
 *
 * Parity pins: the reference ships no golden vectors for this path (its tests draw unseeded
 * rand() values).  The oracle is pinned by the reference's own relations, restated in tests/:
 * gather/scatter partition of unity (tests/patch_transfer.cc:217-247), FD local matrix equals
 * the submatrix of the level matrix (tests/apps_laplace_integrator.cc:55-115), Kronecker-sum
 * inverse against the explicit matrix (tests/tensor_product_matrix.cc:147-345) and the CG+GMG
 * iteration bounds (tests/apps_poisson.cc:87-135).
 *
 * Build: oracle/Makefile (gcc -O3 -fopenmp -ffp-contract=off, no -march flags so that x86
 * and Arm give the same rounding).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAXN 32 /* largest 1-D patch size handled (2(k+1) with k <= 15) */

/* SIPG penalty mode.  0: the reference's sigma = ip*gamma*(1/h_l+1/h_r)/2 inside and
 * 2*ip*gamma/h on Dirichlet faces, gamma = k(k+1) (apps/common_integrator.h:30-37).
 * 1: sigma = ip*2(k+1)^2*(1/h_l+1/h_r)/2 inside and ip*2(k+1)^2/h on Dirichlet faces (the
 * "2(k+1)^2/h" penalty of the 2D DGQ3 benchmark problem; no counterpart in the reference).
 * Both are written with gamma = k(k+1) and per-face-kind ip factors. */
static int g_penalty_mode = 0;

void or_set_penalty_mode(int mode) { g_penalty_mode = mode; }

static void penalty_factors(double ip, int k, double *ip_in, double *ip_bd)
{
  const double gamma = (k == 0) ? 1.0 : (double)k * (k + 1.0), kp = k + 1.0;
  if(g_penalty_mode == 1)
  {
    *ip_in = ip * 2.0 * kp * kp / gamma;
    *ip_bd = ip * kp * kp / gamma;
  }
  else
  {
    *ip_in = ip;
    *ip_bd = ip;
  }
}

/* ===================================================================================== */
/*                               1-D quadrature and shape data                            */
/* ===================================================================================== */

/* Legendre polynomial P_n and its derivative on [-1,1]. */
static void legendre_p(int n, double x, double *p, double *dp)
{
  double p0 = 1.0, p1 = x;
  if(n == 0)
  {
    *p = 1.0;
    *dp = 0.0;
    return;
  }
  for(int j = 2; j <= n; ++j)
  {
    double p2 = ((2.0 * j - 1.0) * x * p1 - (j - 1.0) * p0) / j;
    p0 = p1;
    p1 = p2;
  }
  *p = p1;
  /* derivative from the recurrence n (x P_n - P_{n-1}) / (x^2-1), valid for |x|<1 */
  *dp = n * (x * p1 - p0) / (x * x - 1.0);
}

static void sort_asc(int n, double *x, double *w)
{
  for(int i = 1; i < n; ++i)
    for(int j = i; j > 0 && x[j] < x[j - 1]; --j)
    {
      double t = x[j]; x[j] = x[j - 1]; x[j - 1] = t;
      if(w) { t = w[j]; w[j] = w[j - 1]; w[j - 1] = t; }
    }
}

/* n-point Gauss-Legendre rule on [0,1] (deal.II QGauss<1>(n)). */
int or_gauss(int n, double *x, double *w)
{
  if(n < 1 || n > 64) return -1;
  for(int i = 0; i < n; ++i)
  {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5));
    double p, dp;
    for(int it = 0; it < 100; ++it)
    {
      legendre_p(n, z, &p, &dp);
      double dz = p / dp;
      z -= dz;
      if(fabs(dz) < 1e-17) break;
    }
    legendre_p(n, z, &p, &dp);
    x[i] = 0.5 * (z + 1.0);
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp); /* 2/((1-z^2)P'^2) scaled by 1/2 */
  }
  sort_asc(n, x, w);
  return 0;
}

/* n-point Gauss-Lobatto nodes on [0,1]: endpoints and the roots of P'_{n-1}. */
int or_gauss_lobatto(int n, double *x)
{
  if(n < 2 || n > 64) return -1;
  const int m = n - 1;
  x[0] = 0.0;
  x[n - 1] = 1.0;
  for(int i = 1; i < m; ++i)
  {
    double z = -cos(M_PI * i / m);
    for(int it = 0; it < 200; ++it)
    {
      double p, dp;
      legendre_p(m, z, &p, &dp);
      /* Legendre ODE: (1-z^2) P'' = 2 z P' - m(m+1) P */
      double ddp = (2.0 * z * dp - m * (m + 1.0) * p) / (1.0 - z * z);
      double dz = dp / ddp;
      z -= dz;
      if(fabs(dz) < 1e-17) break;
    }
    x[i] = 0.5 * (z + 1.0);
  }
  sort_asc(n, x, NULL);
  return 0;
}

/* Lagrange basis on nodes z[0..np) evaluated at x: val[i], der[i]. */
void or_lagrange(int np, const double *z, double x, double *val, double *der)
{
  for(int i = 0; i < np; ++i)
  {
    double v = 1.0;
    for(int j = 0; j < np; ++j)
      if(j != i) v *= (x - z[j]) / (z[i] - z[j]);
    val[i] = v;
    double d = 0.0;
    for(int l = 0; l < np; ++l)
    {
      if(l == i) continue;
      double t = 1.0 / (z[i] - z[l]);
      for(int j = 0; j < np; ++j)
        if(j != i && j != l) t *= (x - z[j]) / (z[i] - z[j]);
      d += t;
    }
    der[i] = d;
  }
}

/* Unit-interval shape data of FE_DGQ(k) with k+1 Gauss points:
 * val[i*(k+1)+q] = phi_i(x_q), grad[...] = phi_i'(x_q), face values/gradients at 0 and 1. */
typedef struct
{
  int k, np;
  double qx[OR_MAXN], qw[OR_MAXN];
  double nodes[OR_MAXN];
  double val[OR_MAXN * OR_MAXN], grad[OR_MAXN * OR_MAXN];
  double fval[2][OR_MAXN], fgrad[2][OR_MAXN];
} shape1d;

static void shape1d_init(shape1d *s, int k)
{
  s->k = k;
  s->np = k + 1;
  or_gauss(k + 1, s->qx, s->qw);
  if(k == 0)
    s->nodes[0] = 0.5;
  else
    or_gauss_lobatto(k + 1, s->nodes);
  double v[OR_MAXN], d[OR_MAXN];
  for(int q = 0; q < k + 1; ++q)
  {
    if(k == 0) { v[0] = 1.0; d[0] = 0.0; }
    else or_lagrange(k + 1, s->nodes, s->qx[q], v, d);
    for(int i = 0; i < k + 1; ++i)
    {
      s->val[i * (k + 1) + q] = v[i];
      s->grad[i * (k + 1) + q] = d[i];
    }
  }
  for(int f = 0; f < 2; ++f)
  {
    if(k == 0) { v[0] = 1.0; d[0] = 0.0; }
    else or_lagrange(k + 1, s->nodes, (double)f, v, d);
    for(int i = 0; i < k + 1; ++i)
    {
      s->fval[f][i] = v[i];
      s->fgrad[f][i] = d[i];
    }
  }
}

/* Exported for tests: shape data of FE_DGQ(k) (sizes (k+1)^2, (k+1)^2, 2(k+1), 2(k+1)). */
int or_shape_data(int k, double *qx, double *qw, double *nodes, double *val, double *grad,
                  double *fval, double *fgrad)
{
  if(k < 0 || k + 1 > OR_MAXN) return -1;
  shape1d s;
  shape1d_init(&s, k);
  const int np = k + 1;
  memcpy(qx, s.qx, sizeof(double) * np);
  memcpy(qw, s.qw, sizeof(double) * np);
  memcpy(nodes, s.nodes, sizeof(double) * np);
  memcpy(val, s.val, sizeof(double) * np * np);
  memcpy(grad, s.grad, sizeof(double) * np * np);
  for(int f = 0; f < 2; ++f)
  {
    memcpy(fval + f * np, s.fval[f], sizeof(double) * np);
    memcpy(fgrad + f * np, s.fgrad[f], sizeof(double) * np);
  }
  return 0;
}

/* ===================================================================================== */
/*                       1-D patch matrices of the FD local solvers                       */
/* ===================================================================================== */

/* Assemble the 1-D mass M and SIPG-Laplace A (n x n, n = ncp*(k+1)) of a DG patch with
 * ncp = 1 (cell patch) or 2 (vertex patch) cells of widths h[0..ncp), with the patch's
 * lower/upper face at the physical boundary when bdry_lo/bdry_hi are set.  ip is the
 * EquationData ip_factor used for face and interface penalties. */
int or_patch_matrices_1d(int k, int ncp, const double *h, int bdry_lo, int bdry_hi, double ip,
                         double *M, double *A)
{
  if(ncp < 1 || ncp > 2 || k < 0 || ncp * (k + 1) > OR_MAXN) return -1;
  shape1d s;
  shape1d_init(&s, k);
  const int np = k + 1, n = ncp * np;
  const double gamma = (k == 0) ? 1.0 : (double)k * (k + 1.0);
  double ip_in, ip_bd;
  penalty_factors(ip, k, &ip_in, &ip_bd);
  memset(M, 0, sizeof(double) * n * n);
  memset(A, 0, sizeof(double) * n * n);
  for(int c = 0; c < ncp; ++c)
  {
    const double hc = h[c];
    /* cell mass and Laplace */
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        double m = 0.0, l = 0.0;
        for(int q = 0; q < np; ++q)
        {
          m += s.val[i * np + q] * s.val[j * np + q] * s.qw[q] * hc;
          l += (s.grad[i * np + q] / hc) * (s.grad[j * np + q] / hc) * s.qw[q] * hc;
        }
        M[(c * np + i) * n + c * np + j] += m;
        A[(c * np + i) * n + c * np + j] += l;
      }
    /* both faces of the cell (including the patch-interior interface, with factor 1/2) */
    for(int f = 0; f < 2; ++f)
    {
      const double normal = (f == 0) ? -1.0 : 1.0;
      int at_bdry = 0;
      const int interior_face = (ncp == 2) && ((c == 0 && f == 1) || (c == 1 && f == 0));
      if(!interior_face)
        at_bdry = (f == 0) ? bdry_lo : bdry_hi;
      const double avg = at_bdry ? 1.0 : 0.5;
      const double penalty = (at_bdry ? ip_bd : ip_in) * avg * 2.0 * gamma * (0.5 / hc + 0.5 / hc);
      for(int i = 0; i < np; ++i)
      {
        const double v = s.fval[f][i], dv = s.fgrad[f][i] / hc;
        for(int j = 0; j < np; ++j)
        {
          const double u = s.fval[f][j], du = s.fgrad[f][j] / hc;
          double val = -avg * (v * normal * du + dv * u * normal);
          val += penalty * v * u * normal * normal;
          A[(c * np + i) * n + c * np + j] += val;
        }
      }
    }
  }
  if(ncp == 2)
  {
    /* interface between cell 0 (face 1) and cell 1 (face 0) */
    const double n0 = 1.0, n1 = -1.0;
    const double h0 = h[0], h1 = h[1];
    const double penalty = ip_in * 0.5 * 2.0 * gamma * (0.5 / h0 + 0.5 / h1);
    for(int i = 0; i < np; ++i)
    {
      const double v0 = s.fval[1][i], dv0 = s.fgrad[1][i] / h0;
      const double v1 = s.fval[0][i], dv1 = s.fgrad[0][i] / h1;
      for(int j = 0; j < np; ++j)
      {
        const double u0 = s.fval[1][j], du0 = s.fgrad[1][j] / h0;
        const double u1 = s.fval[0][j], du1 = s.fgrad[0][j] / h1;
        double v01 = -0.5 * (v0 * n0 * du1 + dv0 * u1 * n1) + penalty * v0 * u1 * n0 * n1;
        double v10 = -0.5 * (v1 * n1 * du0 + dv1 * u0 * n0) + penalty * v1 * u0 * n1 * n0;
        A[(0 * np + i) * n + 1 * np + j] += v01;
        A[(1 * np + i) * n + 0 * np + j] += v10;
      }
    }
  }
  return 0;
}

/* ===================================================================================== */
/*                         generalized symmetric eigenproblem                             */
/* ===================================================================================== */

/* Solve A s = lambda M s for symmetric A and s.p.d. M (n x n, row-major).  On return
 * S[i*n+j] = component i of eigenvector j with S^T M S = I and lam ascending. */
int or_gen_eig(int n, const double *A, const double *M, double *S, double *lam)
{
  if(n < 1 || n > OR_MAXN) return -1;
  double L[OR_MAXN * OR_MAXN], C[OR_MAXN * OR_MAXN], X[OR_MAXN * OR_MAXN], V[OR_MAXN * OR_MAXN];
  /* Cholesky M = L L^T */
  memset(L, 0, sizeof(L));
  for(int j = 0; j < n; ++j)
  {
    double d = M[j * n + j];
    for(int p = 0; p < j; ++p) d -= L[j * n + p] * L[j * n + p];
    if(!(d > 0.0)) return -2;
    L[j * n + j] = sqrt(d);
    for(int i = j + 1; i < n; ++i)
    {
      double t = M[i * n + j];
      for(int p = 0; p < j; ++p) t -= L[i * n + p] * L[j * n + p];
      L[i * n + j] = t / L[j * n + j];
    }
  }
  /* X = L^{-1} A  (column by column forward substitution) */
  for(int c = 0; c < n; ++c)
    for(int i = 0; i < n; ++i)
    {
      double t = A[i * n + c];
      for(int p = 0; p < i; ++p) t -= L[i * n + p] * X[p * n + c];
      X[i * n + c] = t / L[i * n + i];
    }
  /* C = X L^{-T} = (L^{-1} X^T)^T */
  for(int r = 0; r < n; ++r)
    for(int i = 0; i < n; ++i)
    {
      double t = X[r * n + i];
      for(int p = 0; p < i; ++p) t -= L[i * n + p] * C[r * n + p];
      C[r * n + i] = t / L[i * n + i];
    }
  for(int i = 0; i < n; ++i)
    for(int j = i + 1; j < n; ++j)
    {
      double t = 0.5 * (C[i * n + j] + C[j * n + i]);
      C[i * n + j] = C[j * n + i] = t;
    }
  /* cyclic Jacobi */
  for(int i = 0; i < n * n; ++i) V[i] = 0.0;
  for(int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for(int sweep = 0; sweep < 100; ++sweep)
  {
    double off = 0.0, tot = 0.0;
    for(int i = 0; i < n; ++i)
      for(int j = 0; j < n; ++j)
      {
        tot += C[i * n + j] * C[i * n + j];
        if(i != j) off += C[i * n + j] * C[i * n + j];
      }
    if(off <= 1e-32 * tot) break;
    for(int p = 0; p < n - 1; ++p)
      for(int q = p + 1; q < n; ++q)
      {
        const double apq = C[p * n + q];
        if(apq == 0.0) continue;
        const double tau = (C[q * n + q] - C[p * n + p]) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for(int k = 0; k < n; ++k) /* C = C J */
        {
          const double ckp = C[k * n + p], ckq = C[k * n + q];
          C[k * n + p] = c * ckp - s * ckq;
          C[k * n + q] = s * ckp + c * ckq;
        }
        for(int k = 0; k < n; ++k) /* C = J^T C */
        {
          const double cpk = C[p * n + k], cqk = C[q * n + k];
          C[p * n + k] = c * cpk - s * cqk;
          C[q * n + k] = s * cpk + c * cqk;
        }
        for(int k = 0; k < n; ++k) /* V = V J */
        {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  /* S = L^{-T} V (back substitution per column) */
  for(int c = 0; c < n; ++c)
    for(int i = n - 1; i >= 0; --i)
    {
      double t = V[i * n + c];
      for(int p = i + 1; p < n; ++p) t -= L[p * n + i] * S[p * n + c];
      S[i * n + c] = t / L[i * n + i];
    }
  for(int i = 0; i < n; ++i) lam[i] = C[i * n + i];
  /* sort ascending, permuting columns of S */
  for(int i = 1; i < n; ++i)
    for(int j = i; j > 0 && lam[j] < lam[j - 1]; --j)
    {
      double t = lam[j]; lam[j] = lam[j - 1]; lam[j - 1] = t;
      for(int r = 0; r < n; ++r)
      {
        t = S[r * n + j]; S[r * n + j] = S[r * n + j - 1]; S[r * n + j - 1] = t;
      }
    }
  return 0;
}

/* ===================================================================================== */
/*                             FD inverse by sum factorization                            */
/* ===================================================================================== */

static int ipow(int b, int e)
{
  int r = 1;
  while(e-- > 0) r *= b;
  return r;
}

/* out = (I x..x B x..x I) in along direction d (B n x n row-major, applied as out_a = sum_b
 * B[a][b] in_b); transpose_B uses B^T. */
static void apply_dir(int dim, int n, int d, const double *B, int transpose_B, const double *in,
                      double *out)
{
  const int stride = ipow(n, d), nouter = ipow(n, dim - 1 - d);
  for(int o = 0; o < nouter; ++o)
    for(int inner = 0; inner < stride; ++inner)
    {
      const int base = o * stride * n + inner;
      for(int a = 0; a < n; ++a)
      {
        double s = 0.0;
        for(int b = 0; b < n; ++b)
        {
          const double bab = transpose_B ? B[b * n + a] : B[a * n + b];
          s += bab * in[base + b * stride];
        }
        out[base + a * stride] = s;
      }
    }
}

/* u = S Lambda^{-1} S^T r with S = S_{d-1} x .. x S_0, Lambda = sum_d lambda_d. */
int or_fd_apply(int dim, int n, const double *const *S, const double *const *lam, const double *r,
                double *u)
{
  const int nl = ipow(n, dim);
  double *t0 = (double *)malloc(sizeof(double) * nl), *t1 = (double *)malloc(sizeof(double) * nl);
  if(!t0 || !t1) { free(t0); free(t1); return -1; }
  memcpy(t0, r, sizeof(double) * nl);
  for(int d = 0; d < dim; ++d)
  {
    apply_dir(dim, n, d, S[d], 1, t0, t1);
    double *t = t0; t0 = t1; t1 = t;
  }
  for(int i = 0; i < nl; ++i)
  {
    double l = 0.0;
    int rem = i;
    for(int d = 0; d < dim; ++d) { l += lam[d][rem % n]; rem /= n; }
    t0[i] /= l;
  }
  for(int d = 0; d < dim; ++d)
  {
    apply_dir(dim, n, d, S[d], 0, t0, t1);
    double *t = t0; t0 = t1; t1 = t;
  }
  memcpy(u, t0, sizeof(double) * nl);
  free(t0);
  free(t1);
  return 0;
}

/* Exported single-patch variant with S and lam packed per direction. */
int or_fd_apply_packed(int dim, int n, const double *S_packed, const double *lam_packed,
                       const double *r, double *u)
{
  const double *S[3], *L[3];
  for(int d = 0; d < dim; ++d)
  {
    S[d] = S_packed + d * n * n;
    L[d] = lam_packed + d * n;
  }
  return or_fd_apply(dim, n, S, L, r, u);
}

/* ===================================================================================== */
/*                              structured level and patches                              */
/* ===================================================================================== */

typedef struct
{
  int dim, k, np, ncell_dofs;
  int nc[3];
  const double *h[3];
  double ip;
  const int64_t *cell_start; /* first DoF of each lexicographic cell, NULL = lexicographic */
  int64_t n_cells, n_dofs;
} level_t;

static void level_init(level_t *L, int dim, int k, const int *nc, const double *hx,
                       const double *hy, const double *hz, double ip, const int64_t *cell_start)
{
  L->dim = dim;
  L->k = k;
  L->np = k + 1;
  L->ncell_dofs = ipow(k + 1, dim);
  L->n_cells = 1;
  for(int d = 0; d < 3; ++d)
  {
    L->nc[d] = d < dim ? nc[d] : 1;
    L->n_cells *= L->nc[d];
  }
  L->h[0] = hx;
  L->h[1] = hy;
  L->h[2] = hz;
  L->ip = ip;
  L->cell_start = cell_start;
  L->n_dofs = L->n_cells * L->ncell_dofs;
}

static inline int64_t cell_lex(const level_t *L, const int *c)
{
  return c[0] + (int64_t)L->nc[0] * (c[1] + (int64_t)L->nc[1] * c[2]);
}

static inline int64_t cell_first_dof(const level_t *L, int64_t cell)
{
  return L->cell_start ? L->cell_start[cell] : cell * L->ncell_dofs;
}

/* Patch list.  patch_variant: 0 = cell, 1 = vertex.  smoother_variant: 0 = additive,
 * 1 = multiplicative.  Output: lower cell coordinate of each patch (3 ints) and its color,
 * ordered by color, interior patches before boundary patches, lexicographic within a group.
 * Returns the number of patches (or the count needed when out arrays are NULL);
 * *n_colors receives the number of colors. */
int64_t or_patches(int dim, const int *nc_in, int patch_variant, int smoother_variant,
                   int32_t *lower, int32_t *color_out, int *n_colors)
{
  int nc[3] = {1, 1, 1};
  for(int d = 0; d < dim; ++d) nc[d] = nc_in[d];
  int nv[3] = {1, 1, 1}; /* patch anchors per direction */
  for(int d = 0; d < dim; ++d) nv[d] = patch_variant == 1 ? nc[d] - 1 : nc[d];
  if(patch_variant == 1)
    for(int d = 0; d < dim; ++d)
      if(nv[d] < 1) { *n_colors = 0; return 0; }
  int ncol;
  if(patch_variant == 1) ncol = 1 << dim;
  else ncol = smoother_variant == 0 ? 1 : 2;
  *n_colors = ncol;
  int64_t total = (int64_t)nv[0] * nv[1] * nv[2];
  if(!lower) return total;
  int64_t pos = 0;
  for(int col = 0; col < ncol; ++col)
    for(int pass = 0; pass < 2; ++pass) /* 0: interior, 1: boundary */
      for(int a2 = 0; a2 < nv[2]; ++a2)
        for(int a1 = 0; a1 < nv[1]; ++a1)
          for(int a0 = 0; a0 < nv[0]; ++a0)
          {
            int a[3] = {a0, a1, a2}, lo[3] = {0, 0, 0}, c = 0, bd = 0;
            for(int d = 0; d < dim; ++d)
            {
              if(patch_variant == 1)
              {
                const int v = a[d] + 1; /* interior vertex index */
                lo[d] = v - 1;
                c |= ((v % 2) == 0) << d;
                bd |= (lo[d] == 0) || (lo[d] + 1 == nc[d] - 1);
              }
              else
              {
                lo[d] = a[d];
                if(smoother_variant == 1) c ^= (a[d] & 1);
                bd |= (lo[d] == 0) || (lo[d] == nc[d] - 1);
              }
            }
            if(c != col || bd != pass) continue;
            lower[3 * pos + 0] = lo[0];
            lower[3 * pos + 1] = lo[1];
            lower[3 * pos + 2] = lo[2];
            color_out[pos] = col;
            ++pos;
          }
  return pos;
}

/* One 1-D FD problem (per patch and direction), cached by its defining data. */
typedef struct
{
  double h0, h1;
  int ncp, lo, hi;
  double S[OR_MAXN * OR_MAXN];
  double lam[OR_MAXN];
} fd1d_t;

typedef struct
{
  fd1d_t *items;
  int n, cap;
} fdcache_t;

static int fdcache_get(fdcache_t *C, int k, int ncp, double h0, double h1, int lo, int hi,
                       double ip)
{
  for(int i = 0; i < C->n; ++i)
  {
    fd1d_t *f = &C->items[i];
    if(f->ncp == ncp && f->h0 == h0 && f->h1 == h1 && f->lo == lo && f->hi == hi) return i;
  }
  if(C->n == C->cap)
  {
    C->cap = C->cap ? 2 * C->cap : 16;
    C->items = (fd1d_t *)realloc(C->items, sizeof(fd1d_t) * C->cap);
  }
  fd1d_t *f = &C->items[C->n];
  f->h0 = h0;
  f->h1 = h1;
  f->ncp = ncp;
  f->lo = lo;
  f->hi = hi;
  const int n = ncp * (k + 1);
  double M[OR_MAXN * OR_MAXN], A[OR_MAXN * OR_MAXN], hh[2] = {h0, h1};
  or_patch_matrices_1d(k, ncp, hh, lo, hi, ip, M, A);
  if(or_gen_eig(n, A, M, f->S, f->lam) != 0) return -1;
  return C->n++;
}

/* Per patch: its cells' first DoFs and its FD data indices. */
typedef struct
{
  int64_t P;
  int ncol, npc, n, nloc;
  int64_t *color_start; /* ncol+1 */
  int64_t *cell_first;  /* P * npc */
  int *fd;              /* P * dim */
  fdcache_t cache;
} patches_t;

static void patches_free(patches_t *T)
{
  free(T->color_start);
  free(T->cell_first);
  free(T->fd);
  free(T->cache.items);
}

static int patches_build(patches_t *T, const level_t *L, int patch_variant, int smoother_variant)
{
  memset(T, 0, sizeof(*T));
  const int dim = L->dim;
  int ncol;
  int64_t P = or_patches(dim, L->nc, patch_variant, smoother_variant, NULL, NULL, &ncol);
  int32_t *lower = (int32_t *)malloc(sizeof(int32_t) * 3 * (P ? P : 1));
  int32_t *color = (int32_t *)malloc(sizeof(int32_t) * (P ? P : 1));
  or_patches(dim, L->nc, patch_variant, smoother_variant, lower, color, &ncol);
  const int ncp = patch_variant == 1 ? 2 : 1;
  T->P = P;
  T->ncol = ncol;
  T->npc = ipow(ncp, dim);
  T->n = ncp * L->np;
  T->nloc = ipow(T->n, dim);
  T->color_start = (int64_t *)calloc(ncol + 1, sizeof(int64_t));
  T->cell_first = (int64_t *)malloc(sizeof(int64_t) * (P ? P : 1) * T->npc);
  T->fd = (int *)malloc(sizeof(int) * (P ? P : 1) * dim);
  for(int64_t p = 0; p < P; ++p) T->color_start[color[p] + 1]++;
  for(int c = 0; c < ncol; ++c) T->color_start[c + 1] += T->color_start[c];
  for(int64_t p = 0; p < P; ++p)
  {
    const int32_t *lo = lower + 3 * p;
    for(int cn = 0; cn < T->npc; ++cn)
    {
      int c[3] = {lo[0], lo[1], lo[2]}, rem = cn;
      for(int d = 0; d < dim; ++d) { c[d] += rem % ncp; rem /= ncp; }
      T->cell_first[p * T->npc + cn] = cell_first_dof(L, cell_lex(L, c));
    }
    for(int d = 0; d < dim; ++d)
    {
      const int c0 = lo[d], c1 = lo[d] + ncp - 1;
      const double h0 = L->h[d][c0], h1 = ncp == 2 ? L->h[d][c1] : 0.0;
      const int blo = c0 == 0, bhi = c1 == L->nc[d] - 1;
      int idx = fdcache_get(&T->cache, L->k, ncp, h0, h1, blo, bhi, L->ip);
      if(idx < 0) { free(lower); free(color); return -1; }
      T->fd[p * dim + d] = idx;
    }
  }
  free(lower);
  free(color);
  return 0;
}

/* patch-local index of DoF e of patch cell cn (lexicographic cell number) */
static inline int patch_index(int dim, int np, int ncp, int n, int cn, int e)
{
  int idx = 0, stride = 1, rc = cn, re = e;
  for(int d = 0; d < dim; ++d)
  {
    const int cd = rc % ncp, id = re % np;
    rc /= ncp;
    re /= np;
    idx += (cd * np + id) * stride;
    stride *= n;
  }
  return idx;
}

static void gather_patch(const level_t *L, const patches_t *T, int64_t p, int ncp,
                         const double *src, double *r)
{
  for(int cn = 0; cn < T->npc; ++cn)
  {
    const int64_t f = T->cell_first[p * T->npc + cn];
    for(int e = 0; e < L->ncell_dofs; ++e)
      r[patch_index(L->dim, L->np, ncp, T->n, cn, e)] = src[f + e];
  }
}

static void scatter_add_patch(const level_t *L, const patches_t *T, int64_t p, int ncp,
                              const double *u, double *dst)
{
  for(int cn = 0; cn < T->npc; ++cn)
  {
    const int64_t f = T->cell_first[p * T->npc + cn];
    for(int e = 0; e < L->ncell_dofs; ++e)
      dst[f + e] += u[patch_index(L->dim, L->np, ncp, T->n, cn, e)];
  }
}

/* dst += omega * sum_{p in color} R_p^T A_p^-1 R_p src (weights: optional RAS weights; keep:
 * optional RAS boolean flags, P * nloc). */
static void apply_color(const level_t *L, const patches_t *T, int color, int ncp, double omega,
                        const double *weights, const unsigned char *keep, const double *src,
                        double *dst)
{
  const int64_t b = T->color_start[color], e = T->color_start[color + 1];
  const int dim = L->dim, n = T->n;
#pragma omp parallel
  {
    double *r = (double *)malloc(sizeof(double) * T->nloc);
    double *u = (double *)malloc(sizeof(double) * T->nloc);
    double *w = weights ? (double *)malloc(sizeof(double) * T->nloc) : NULL;
#pragma omp for schedule(static)
    for(int64_t p = b; p < e; ++p)
    {
      gather_patch(L, T, p, ncp, src, r);
      const double *S[3], *lam[3];
      for(int d = 0; d < dim; ++d)
      {
        const fd1d_t *f = &T->cache.items[T->fd[p * dim + d]];
        S[d] = f->S;
        lam[d] = f->lam;
      }
      or_fd_apply(dim, n, S, lam, r, u);
      if(omega != 1.0)
        for(int i = 0; i < T->nloc; ++i) u[i] *= omega;
      if(weights)
      {
        gather_patch(L, T, p, ncp, weights, w);
        for(int i = 0; i < T->nloc; ++i) u[i] /= w[i];
      }
      if(keep)
        for(int i = 0; i < T->nloc; ++i)
          if(!keep[p * T->nloc + i]) u[i] = 0.0; /* rscatter_add: restricted DoFs are skipped */
      scatter_add_patch(L, T, p, ncp, u, dst);
    }
    free(r);
    free(u);
    free(w);
  }
}

/* RAS boolean flags (DoFInfo::compute_restricted_dofs_impl, TPSS/dof_info.templates.h:194-313):
 * of all occurrences (patch p, patch-local index i) of a global DoF only the one with the
 * smallest (distance to the patch centre, i, p) scatters.  DGQ distance: max over directions of
 * trunc(|n/2 - 1/2 - m_d|), m_d the patch-local 1-D index.  keep[p * nloc + i] = 1 for the
 * winners.  Vertex patches of an additive smoother only. */
static unsigned char *ras_boolean_flags(const level_t *L, const patches_t *T, int ncp)
{
  const int dim = L->dim, n = T->n, nloc = T->nloc;
  int64_t *best_p = (int64_t *)malloc(sizeof(int64_t) * L->n_dofs);
  int *best_i = (int *)malloc(sizeof(int) * L->n_dofs);
  int *best_d = (int *)malloc(sizeof(int) * L->n_dofs);
  for(int64_t g = 0; g < L->n_dofs; ++g) best_p[g] = -1;
  for(int64_t p = 0; p < T->P; ++p)
    for(int cn = 0; cn < T->npc; ++cn)
    {
      const int64_t f = T->cell_first[p * T->npc + cn];
      for(int e = 0; e < L->ncell_dofs; ++e)
      {
        const int i = patch_index(dim, L->np, ncp, n, cn, e);
        int dist = 0, rem = i;
        for(int d = 0; d < dim; ++d, rem /= n)
        {
          const double diff = fabs(0.5 * n - 0.5 - (double)(rem % n));
          const int t = (int)diff;
          if(t > dist) dist = t;
        }
        const int64_t g = f + e;
        const int better = best_p[g] < 0 || dist < best_d[g] || (dist == best_d[g] && i < best_i[g]) ||
                           (dist == best_d[g] && i == best_i[g] && p < best_p[g]);
        if(better)
        {
          best_p[g] = p;
          best_i[g] = i;
          best_d[g] = dist;
        }
      }
    }
  unsigned char *keep = (unsigned char *)calloc((size_t)T->P * nloc, 1);
  for(int64_t g = 0; g < L->n_dofs; ++g)
    if(best_p[g] >= 0) keep[best_p[g] * nloc + best_i[g]] = 1;
  free(best_p);
  free(best_i);
  free(best_d);
  return keep;
}

static void ras_weights(const level_t *L, const patches_t *T, int ncp, double *wgt)
{
  memset(wgt, 0, sizeof(double) * L->n_dofs);
  double *one = (double *)malloc(sizeof(double) * T->nloc);
  for(int i = 0; i < T->nloc; ++i) one[i] = 1.0;
  for(int64_t p = 0; p < T->P; ++p) scatter_add_patch(L, T, p, ncp, one, wgt);
  free(one);
}

/* ===================================================================================== */
/*                         SIPG operator (Kronecker sum, Cartesian)                       */
/* ===================================================================================== */

/* Per direction and cell: cell mass block and the three blocks (left, centre, right) of the
 * global 1-D SIPG matrix, (k+1)^2 each. */
typedef struct
{
  int k, np, nc;
  double *mass; /* nc * np^2 */
  double *blk;  /* nc * 3 * np^2 : [c][o+1] couples cell c (test) with c+o (trial) */
} op1d_t;

static void op1d_build(op1d_t *O, int k, int nc, const double *h, double ip)
{
  shape1d s;
  shape1d_init(&s, k);
  const int np = k + 1, q2 = np * np;
  const double gamma = (k == 0) ? 1.0 : (double)k * (k + 1.0);
  double ip_in, ip_bd;
  penalty_factors(ip, k, &ip_in, &ip_bd);
  O->k = k;
  O->np = np;
  O->nc = nc;
  O->mass = (double *)calloc((size_t)nc * q2, sizeof(double));
  O->blk = (double *)calloc((size_t)nc * 3 * q2, sizeof(double));
  for(int c = 0; c < nc; ++c)
  {
    const double hc = h[c];
    double *C = O->blk + ((size_t)c * 3 + 1) * q2;
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        double m = 0.0, l = 0.0;
        for(int q = 0; q < np; ++q)
        {
          m += s.val[i * np + q] * s.val[j * np + q] * s.qw[q] * hc;
          l += s.grad[i * np + q] * s.grad[j * np + q] * s.qw[q] / hc;
        }
        O->mass[(size_t)c * q2 + i * np + j] = m;
        C[i * np + j] += l;
      }
    /* boundary faces (Dirichlet): sigma = ip * 2 gamma / h */
    if(c == 0 || c == nc - 1)
    {
      for(int f = 0; f < 2; ++f)
      {
        if(f == 0 && c != 0) continue;
        if(f == 1 && c != nc - 1) continue;
        const double nrm = f == 0 ? -1.0 : 1.0;
        const double sigma = ip_bd * 2.0 * gamma * (0.5 / hc + 0.5 / hc);
        for(int i = 0; i < np; ++i)
          for(int j = 0; j < np; ++j)
          {
            const double v = s.fval[f][i], dv = s.fgrad[f][i] / hc;
            const double u = s.fval[f][j], du = s.fgrad[f][j] / hc;
            C[i * np + j] += sigma * u * v - nrm * du * v - u * nrm * dv;
          }
      }
    }
  }
  /* interior faces between c (left) and c+1 (right), normal +x */
  for(int c = 0; c + 1 < nc; ++c)
  {
    const double hl = h[c], hr = h[c + 1];
    const double sigma = ip_in * 0.5 * 2.0 * gamma * (0.5 / hl + 0.5 / hr);
    double *LL = O->blk + ((size_t)c * 3 + 1) * q2;
    double *LR = O->blk + ((size_t)c * 3 + 2) * q2;
    double *RL = O->blk + ((size_t)(c + 1) * 3 + 0) * q2;
    double *RR = O->blk + ((size_t)(c + 1) * 3 + 1) * q2;
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        /* test i, trial j; [w] = w_l(1) - w_r(0), {w'} = (w_l'(1) + w_r'(0))/2 */
        const double vl = s.fval[1][i], dvl = s.fgrad[1][i] / hl;
        const double vr = s.fval[0][i], dvr = s.fgrad[0][i] / hr;
        const double ul = s.fval[1][j], dul = s.fgrad[1][j] / hl;
        const double ur = s.fval[0][j], dur = s.fgrad[0][j] / hr;
        LL[i * np + j] += sigma * ul * vl - 0.5 * dul * vl - ul * 0.5 * dvl;
        LR[i * np + j] += -sigma * ur * vl - 0.5 * dur * vl + ur * 0.5 * dvl;
        RL[i * np + j] += -sigma * ul * vr + 0.5 * dul * vr - ul * 0.5 * dvr;
        RR[i * np + j] += sigma * ur * vr + 0.5 * dur * vr + ur * 0.5 * dvr;
      }
  }
}

static void op1d_free(op1d_t *O)
{
  free(O->mass);
  free(O->blk);
}

/* dst = A src for the SIPG operator on a structured level. */
static void sipg_apply(const level_t *L, const op1d_t *O, const double *src, double *dst)
{
  const int dim = L->dim, np = L->np, nd = L->ncell_dofs;
#pragma omp parallel
  {
    double *t0 = (double *)malloc(sizeof(double) * nd), *t1 = (double *)malloc(sizeof(double) * nd);
    double *acc = (double *)malloc(sizeof(double) * nd);
#pragma omp for schedule(static)
    for(int64_t cell = 0; cell < L->n_cells; ++cell)
    {
      int c[3] = {(int)(cell % L->nc[0]), (int)((cell / L->nc[0]) % L->nc[1]),
                  (int)(cell / ((int64_t)L->nc[0] * L->nc[1]))};
      for(int i = 0; i < nd; ++i) acc[i] = 0.0;
      for(int d = 0; d < dim; ++d)
        for(int o = -1; o <= 1; ++o)
        {
          const int cn = c[d] + o;
          if(cn < 0 || cn >= L->nc[d]) continue;
          int cc[3] = {c[0], c[1], c[2]};
          cc[d] = cn;
          const double *u = src + cell_first_dof(L, cell_lex(L, cc));
          memcpy(t0, u, sizeof(double) * nd);
          for(int e = 0; e < dim; ++e)
          {
            const double *B = e == d ? O[d].blk + ((size_t)c[d] * 3 + (o + 1)) * np * np
                                     : O[e].mass + (size_t)c[e] * np * np;
            apply_dir(dim, np, e, B, 0, t0, t1);
            double *t = t0; t0 = t1; t1 = t;
          }
          for(int i = 0; i < nd; ++i) acc[i] += t0[i];
        }
      memcpy(dst + cell_first_dof(L, cell), acc, sizeof(double) * nd);
    }
    free(t0);
    free(t1);
    free(acc);
  }
}

int or_sipg_vmult(int dim, int k, const int *nc, const double *hx, const double *hy,
                  const double *hz, double ip, const int64_t *cell_start, const double *src,
                  double *dst)
{
  level_t L;
  level_init(&L, dim, k, nc, hx, hy, hz, ip, cell_start);
  op1d_t O[3];
  for(int d = 0; d < dim; ++d) op1d_build(&O[d], k, L.nc[d], L.h[d], ip);
  sipg_apply(&L, O, src, dst);
  for(int d = 0; d < dim; ++d) op1d_free(&O[d]);
  return 0;
}

/* ===================================================================================== */
/*                                  Schwarz preconditioner                                */
/* ===================================================================================== */

typedef struct
{
  level_t L;
  patches_t T;
  op1d_t O[3];
  int patch_variant, smoother_variant, ncp;
  double omega;
  int reverse, symmetrized, use_ras; /* use_ras: 1 RAS weights, 2 RAS boolean weights */
  double *wgt;
  unsigned char *keep;
} schwarz_t;

static int schwarz_init(schwarz_t *S, int dim, int k, const int *nc, const double *hx,
                        const double *hy, const double *hz, double ip,
                        const int64_t *cell_start, int patch_variant, int smoother_variant,
                        double omega, int reverse, int symmetrized, int use_ras)
{
  memset(S, 0, sizeof(*S));
  level_init(&S->L, dim, k, nc, hx, hy, hz, ip, cell_start);
  if(patches_build(&S->T, &S->L, patch_variant, smoother_variant) != 0) return -1;
  S->patch_variant = patch_variant;
  S->smoother_variant = smoother_variant;
  S->ncp = patch_variant == 1 ? 2 : 1;
  S->omega = omega;
  S->reverse = reverse;
  S->symmetrized = symmetrized;
  S->use_ras = smoother_variant == 0 ? use_ras : 0;
  if(smoother_variant == 1)
    for(int d = 0; d < dim; ++d) op1d_build(&S->O[d], k, S->L.nc[d], S->L.h[d], ip);
  if(S->use_ras == 2)
  {
    if(patch_variant != 1) return -1; /* the reference: vertex patches only */
    S->keep = ras_boolean_flags(&S->L, &S->T, S->ncp);
  }
  else if(S->use_ras)
  {
    S->wgt = (double *)malloc(sizeof(double) * S->L.n_dofs);
    ras_weights(&S->L, &S->T, S->ncp, S->wgt);
  }
  return 0;
}

static void schwarz_free(schwarz_t *S)
{
  patches_free(&S->T);
  if(S->smoother_variant == 1)
    for(int d = 0; d < S->L.dim; ++d) op1d_free(&S->O[d]);
  free(S->wgt);
  free(S->keep);
}

/* Color sequence as SchwarzPreconditioner::get_color_sequence (schwarz_preconditioner.h:532-567). */
static int color_sequence(int ncol, int reverse, int symmetrized, int *seq)
{
  int n = 0;
  for(int c = 0; c < ncol; ++c) seq[n++] = reverse ? ncol - 1 - c : c;
  if(symmetrized)
    for(int i = ncol - 2; i >= 0; --i) seq[n++] = seq[i];
  return n;
}

static void schwarz_vmult(const schwarz_t *S, double *dst, const double *src)
{
  const int64_t N = S->L.n_dofs;
  memset(dst, 0, sizeof(double) * N);
  if(S->smoother_variant == 0)
  {
    for(int c = 0; c < S->T.ncol; ++c)
      apply_color(&S->L, &S->T, c, S->ncp, S->omega, S->wgt, S->keep, src, dst);
    return;
  }
  int seq[64];
  const int ns = color_sequence(S->T.ncol, S->reverse, S->symmetrized, seq);
  double *res = (double *)malloc(sizeof(double) * N);
  apply_color(&S->L, &S->T, seq[0], S->ncp, S->omega, NULL, NULL, src, dst);
  for(int i = 1; i < ns; ++i)
  {
    sipg_apply(&S->L, S->O, dst, res);
    for(int64_t j = 0; j < N; ++j) res[j] = src[j] - res[j];
    apply_color(&S->L, &S->T, seq[i], S->ncp, S->omega, NULL, NULL, res, dst);
  }
  free(res);
}

/* SchwarzPreconditioner::vmult on one structured level.  patch_variant 0 = cell, 1 = vertex;
 * smoother_variant 0 = additive, 1 = multiplicative.  Returns 0 on success. */
int or_schwarz_vmult(int dim, int k, const int *nc, const double *hx, const double *hy,
                     const double *hz, double ip, const int64_t *cell_start, int patch_variant,
                     int smoother_variant, double omega, int reverse, int symmetrized,
                     int use_ras, const double *src, double *dst)
{
  schwarz_t S;
  if(schwarz_init(&S, dim, k, nc, hx, hy, hz, ip, cell_start, patch_variant, smoother_variant,
                  omega, reverse, symmetrized, use_ras) != 0)
    return -1;
  schwarz_vmult(&S, dst, src);
  schwarz_free(&S);
  return 0;
}

/* Opaque handle variant for timing repeated applications (CPU baseline). */
void *or_schwarz_create(int dim, int k, const int *nc, const double *hx, const double *hy,
                        const double *hz, double ip, const int64_t *cell_start, int patch_variant,
                        int smoother_variant, double omega)
{
  schwarz_t *S = (schwarz_t *)malloc(sizeof(schwarz_t));
  if(schwarz_init(S, dim, k, nc, hx, hy, hz, ip, cell_start, patch_variant, smoother_variant,
                  omega, 0, 0, 0) != 0)
  {
    free(S);
    return NULL;
  }
  return S;
}

void or_schwarz_apply(void *h, double *dst, const double *src)
{
  schwarz_vmult((const schwarz_t *)h, dst, src);
}

/* Apply only the patches [p_begin, p_end) of the additive smoother (dst += ...); used to
 * time a bounded sample of a vmult. */
void or_schwarz_apply_range(void *h, int64_t p_begin, int64_t p_end, double *dst,
                            const double *src)
{
  const schwarz_t *S = (const schwarz_t *)h;
  for(int c = 0; c < S->T.ncol; ++c)
  {
    int64_t b = S->T.color_start[c], e = S->T.color_start[c + 1];
    if(b < p_begin) b = p_begin;
    if(e > p_end) e = p_end;
    if(b >= e) continue;
    patches_t sub = S->T;
    int64_t cs[2] = {b, e};
    sub.color_start = cs;
    sub.ncol = 1;
    apply_color(&S->L, &sub, 0, S->ncp, S->omega, NULL, NULL, src, dst);
  }
}

int64_t or_schwarz_n_patches(void *h) { return ((const schwarz_t *)h)->T.P; }

void or_schwarz_destroy(void *h)
{
  if(!h) return;
  schwarz_free((schwarz_t *)h);
  free(h);
}

int or_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int n)
{
#ifdef _OPENMP
  if(n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ===================================================================================== */
/*                      DG transfer, V-cycle, coarse CG and PCG (FP64)                    */
/* ===================================================================================== */

/* 1-D embedding of the coarse basis into child s: E[s][i*np+j] = phi_j((z_i + s)/2). */
static void embedding_1d(int k, double *E)
{
  shape1d s;
  shape1d_init(&s, k);
  const int np = k + 1;
  double v[OR_MAXN], d[OR_MAXN];
  for(int ch = 0; ch < 2; ++ch)
    for(int i = 0; i < np; ++i)
    {
      if(k == 0) { v[0] = 1.0; }
      else or_lagrange(np, s.nodes, 0.5 * (s.nodes[i] + ch), v, d);
      for(int j = 0; j < np; ++j) E[ch * np * np + i * np + j] = v[j];
    }
}

/* fine += P coarse (prolongate_add) or coarse += P^T fine (restrict_add) between structured
 * levels with lexicographic cells (nc_fine = 2 nc_coarse). */
static void transfer(int dim, int k, const int *ncc, const double *E, int restrict_mode,
                     double *coarse, double *fine)
{
  const int np = k + 1, nd = ipow(np, dim), nch = 1 << dim;
  int nf[3] = {1, 1, 1}, nc3[3] = {1, 1, 1};
  for(int d = 0; d < dim; ++d) { nc3[d] = ncc[d]; nf[d] = 2 * ncc[d]; }
  const int64_t ncells = (int64_t)nc3[0] * nc3[1] * nc3[2];
#pragma omp parallel
  {
    double *t0 = (double *)malloc(sizeof(double) * nd), *t1 = (double *)malloc(sizeof(double) * nd);
    double *acc = (double *)malloc(sizeof(double) * nd);
#pragma omp for schedule(static)
    for(int64_t cell = 0; cell < ncells; ++cell)
    {
      int c[3] = {(int)(cell % nc3[0]), (int)((cell / nc3[0]) % nc3[1]),
                  (int)(cell / ((int64_t)nc3[0] * nc3[1]))};
      if(restrict_mode)
        for(int i = 0; i < nd; ++i) acc[i] = 0.0;
      for(int ch = 0; ch < nch; ++ch)
      {
        int f[3] = {0, 0, 0}, sbit[3] = {0, 0, 0};
        for(int d = 0; d < dim; ++d) { sbit[d] = (ch >> d) & 1; f[d] = 2 * c[d] + sbit[d]; }
        const int64_t fcell = f[0] + (int64_t)nf[0] * (f[1] + (int64_t)nf[1] * f[2]);
        double *fu = fine + fcell * nd;
        if(restrict_mode)
        {
          memcpy(t0, fu, sizeof(double) * nd);
          for(int d = 0; d < dim; ++d)
          {
            apply_dir(dim, np, d, E + sbit[d] * np * np, 1, t0, t1);
            double *t = t0; t0 = t1; t1 = t;
          }
          for(int i = 0; i < nd; ++i) acc[i] += t0[i];
        }
        else
        {
          memcpy(t0, coarse + cell * nd, sizeof(double) * nd);
          for(int d = 0; d < dim; ++d)
          {
            apply_dir(dim, np, d, E + sbit[d] * np * np, 0, t0, t1);
            double *t = t0; t0 = t1; t1 = t;
          }
          for(int i = 0; i < nd; ++i) fu[i] += t0[i];
        }
      }
      if(restrict_mode)
        for(int i = 0; i < nd; ++i) coarse[cell * nd + i] += acc[i];
    }
    free(t0);
    free(t1);
    free(acc);
  }
}

int or_prolongate_add(int dim, int k, const int *nc_coarse, const double *coarse, double *fine)
{
  double E[2 * OR_MAXN * OR_MAXN];
  embedding_1d(k, E);
  transfer(dim, k, nc_coarse, E, 0, (double *)coarse, fine);
  return 0;
}

int or_restrict_add(int dim, int k, const int *nc_coarse, double *coarse, const double *fine)
{
  double E[2 * OR_MAXN * OR_MAXN];
  embedding_1d(k, E);
  transfer(dim, k, nc_coarse, E, 1, coarse, (double *)fine);
  return 0;
}

static double dot(int64_t n, const double *a, const double *b)
{
  double s = 0.0;
  for(int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

typedef struct
{
  int dim, k, nlev, n_rep;
  level_t L[16];
  op1d_t O[16][3];
  schwarz_t S[16];
  double *h[16][3];
  double *E;
  double *x[16], *b[16], *t[16], *r[16];
  int coarse_iters;
} mg_t;

/* V-cycle on level l: x = MG_l b (deal.II Multigrid::level_v_step with SmootherRichardson,
 * one pre- and one post-smoothing step, relaxation inside the Schwarz preconditioner). */
static void coarse_cg(mg_t *G, double *x, const double *b)
{
  level_t *L = &G->L[0];
  const int64_t N = L->n_dofs;
  double *r = G->r[0], *p = (double *)malloc(sizeof(double) * N), *Ap = G->t[0];
  memset(x, 0, sizeof(double) * N);
  memcpy(r, b, sizeof(double) * N);
  double rr = dot(N, r, r);
  int it = 0;
  if(sqrt(rr) > 1e-12)
  {
    memcpy(p, r, sizeof(double) * N);
    for(it = 1; it <= N; ++it)
    {
      sipg_apply(L, G->O[0], p, Ap);
      const double alpha = rr / dot(N, p, Ap);
      for(int64_t i = 0; i < N; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
      const double rr_new = dot(N, r, r);
      if(sqrt(rr_new) <= 1e-12) break;
      const double beta = rr_new / rr;
      rr = rr_new;
      for(int64_t i = 0; i < N; ++i) p[i] = r[i] + beta * p[i];
    }
  }
  G->coarse_iters += it;
  free(p);
}

static void vcycle(mg_t *G, int l)
{
  level_t *L = &G->L[l];
  const int64_t N = L->n_dofs;
  double *x = G->x[l], *b = G->b[l], *t = G->t[l], *r = G->r[l];
  if(l == 0)
  {
    coarse_cg(G, x, b);
    return;
  }
  /* pre-smoothing from zero: x = P b */
  schwarz_vmult(&G->S[l], x, b);
  /* residual and restriction */
  sipg_apply(L, G->O[l], x, t);
  for(int64_t i = 0; i < N; ++i) t[i] = b[i] - t[i];
  memset(G->b[l - 1], 0, sizeof(double) * G->L[l - 1].n_dofs);
  transfer(G->dim, G->k, G->L[l - 1].nc, G->E, 1, G->b[l - 1], t);
  vcycle(G, l - 1);
  transfer(G->dim, G->k, G->L[l - 1].nc, G->E, 0, G->x[l - 1], x);
  /* post-smoothing: x += P (b - A x) */
  sipg_apply(L, G->O[l], x, t);
  for(int64_t i = 0; i < N; ++i) t[i] = b[i] - t[i];
  schwarz_vmult(&G->S[l], r, t);
  for(int64_t i = 0; i < N; ++i) x[i] += r[i];
}

/* Solve A u = f on the unit cube with n_rep^dim root cells refined to nc_fine cells per
 * direction (nc_fine = n_rep * 2^L), DG Q_k, SIPG (ip factor), by CG preconditioned with one
 * V-cycle (additive or multiplicative Schwarz smoother on levels 1..L, coarse CG to 1e-12 on
 * level 0).  Stops at ||r|| <= max(abs_tol, rel_tol ||r_0||) or max_iter.  Returns the
 * iteration count (or -1) and fills res_history[0..iters]. */
int or_mg_cg_solve(int dim, int k, int n_rep, int nc_fine, double ip, int patch_variant,
                   int smoother_variant, double omega, double rel_tol, double abs_tol,
                   int max_iter, const double *f, double *u, double *res_history)
{
  mg_t G;
  memset(&G, 0, sizeof(G));
  G.dim = dim;
  G.k = k;
  G.n_rep = n_rep;
  int nl = 0;
  for(int nc = n_rep; nc <= nc_fine; nc *= 2) ++nl;
  if(nl < 1 || nl > 16 || (n_rep << (nl - 1)) != nc_fine) return -1;
  G.nlev = nl;
  G.E = (double *)malloc(sizeof(double) * 2 * OR_MAXN * OR_MAXN);
  embedding_1d(k, G.E);
  for(int l = 0; l < nl; ++l)
  {
    int nc[3] = {n_rep << l, n_rep << l, n_rep << l};
    for(int d = 0; d < dim; ++d)
    {
      G.h[l][d] = (double *)malloc(sizeof(double) * nc[d]);
      for(int c = 0; c < nc[d]; ++c) G.h[l][d][c] = 1.0 / nc[d];
    }
    level_init(&G.L[l], dim, k, nc, G.h[l][0], G.h[l][1], dim == 3 ? G.h[l][2] : NULL, ip,
               NULL);
    for(int d = 0; d < dim; ++d) op1d_build(&G.O[l][d], k, nc[d], G.h[l][d], ip);
    if(l > 0)
      schwarz_init(&G.S[l], dim, k, nc, G.h[l][0], G.h[l][1], dim == 3 ? G.h[l][2] : NULL, ip,
                   NULL, patch_variant, smoother_variant, omega, 0, 0, 0);
    const int64_t N = G.L[l].n_dofs;
    G.x[l] = (double *)calloc(N, sizeof(double));
    G.b[l] = (double *)calloc(N, sizeof(double));
    G.t[l] = (double *)calloc(N, sizeof(double));
    G.r[l] = (double *)calloc(N, sizeof(double));
  }
  const int top = nl - 1;
  level_t *L = &G.L[top];
  const int64_t N = L->n_dofs;
  double *r = (double *)malloc(sizeof(double) * N), *p = (double *)malloc(sizeof(double) * N);
  double *Ap = (double *)malloc(sizeof(double) * N), *z = (double *)malloc(sizeof(double) * N);
  memset(u, 0, sizeof(double) * N);
  memcpy(r, f, sizeof(double) * N);
  double res = sqrt(dot(N, r, r));
  res_history[0] = res;
  const double tol = fmax(abs_tol, rel_tol * res);
  int it = 0, converged = res <= tol;
  if(!converged)
  {
    memcpy(G.b[top], r, sizeof(double) * N);
    vcycle(&G, top);
    memcpy(z, G.x[top], sizeof(double) * N);
    memcpy(p, z, sizeof(double) * N);
    double rz = dot(N, r, z);
    for(it = 1; it <= max_iter; ++it)
    {
      sipg_apply(L, G.O[top], p, Ap);
      const double alpha = rz / dot(N, p, Ap);
      for(int64_t i = 0; i < N; ++i) { u[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
      res = sqrt(dot(N, r, r));
      res_history[it] = res;
      if(res <= tol) { converged = 1; break; }
      memcpy(G.b[top], r, sizeof(double) * N);
      vcycle(&G, top);
      memcpy(z, G.x[top], sizeof(double) * N);
      const double rz_new = dot(N, r, z);
      const double beta = rz_new / rz;
      rz = rz_new;
      for(int64_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
    }
  }
  free(r); free(p); free(Ap); free(z);
  for(int l = 0; l < nl; ++l)
  {
    for(int d = 0; d < dim; ++d) { op1d_free(&G.O[l][d]); free(G.h[l][d]); }
    if(l > 0) schwarz_free(&G.S[l]);
    free(G.x[l]); free(G.b[l]); free(G.t[l]); free(G.r[l]);
  }
  free(G.E);
  return converged ? it : -1;
}

/* ===================================================================================== */
/*                       Kronecker SVD (low Kronecker-rank approximation)                */
/* ===================================================================================== */

/* One-sided Jacobi SVD (Hestenes) of the m x n row-major matrix A: on return A holds U*S
 * (column j = sigma_j u_j), V (n x n) the right singular vectors, s the singular values,
 * all sorted by descending sigma. */
static void svd_onesided(int m, int n, double *A, double *V, double *s)
{
  for(int i = 0; i < n * n; ++i) V[i] = 0.0;
  for(int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for(int sweep = 0; sweep < 100; ++sweep)
  {
    int rotated = 0;
    for(int p = 0; p < n - 1; ++p)
      for(int q = p + 1; q < n; ++q)
      {
        double al = 0.0, be = 0.0, ga = 0.0;
        for(int i = 0; i < m; ++i)
        {
          al += A[i * n + p] * A[i * n + p];
          be += A[i * n + q] * A[i * n + q];
          ga += A[i * n + p] * A[i * n + q];
        }
        if(fabs(ga) <= 1e-15 * sqrt(al * be) || ga == 0.0) continue;
        rotated = 1;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
        for(int i = 0; i < m; ++i)
        {
          const double ap = A[i * n + p], aq = A[i * n + q];
          A[i * n + p] = c * ap - sn * aq;
          A[i * n + q] = sn * ap + c * aq;
        }
        for(int i = 0; i < n; ++i)
        {
          const double vp = V[i * n + p], vq = V[i * n + q];
          V[i * n + p] = c * vp - sn * vq;
          V[i * n + q] = sn * vp + c * vq;
        }
      }
    if(!rotated) break;
  }
  for(int j = 0; j < n; ++j)
  {
    double nn = 0.0;
    for(int i = 0; i < m; ++i) nn += A[i * n + j] * A[i * n + j];
    s[j] = sqrt(nn);
  }
  /* sort descending (selection on columns) */
  for(int a = 0; a < n; ++a)
  {
    int b = a;
    for(int j = a + 1; j < n; ++j)
      if(s[j] > s[b]) b = j;
    if(b == a) continue;
    double t = s[a]; s[a] = s[b]; s[b] = t;
    for(int i = 0; i < m; ++i) { t = A[i * n + a]; A[i * n + a] = A[i * n + b]; A[i * n + b] = t; }
    for(int i = 0; i < n; ++i) { t = V[i * n + a]; V[i * n + a] = V[i * n + b]; V[i * n + b] = t; }
  }
}

/* Best Kronecker rank-r approximation M ~ sum_r B_r (x) A_r (TPSS/kroneckersvd.h:207-296,
 * compute_ksvd; "big" B_r is bm x bn, "small" A_r is sm x sn, M = (bm sm) x (bn sn)).  As in the
 * reference, the rearranged matrix R[(k,l),(i,j)] = M[k sm + i][l sn + j] (Van Loan & Pitsianis)
 * is decomposed by an SVD and sigma_r is split as sqrt(sigma_r) on both factors; here the SVD is
 * a one-sided Jacobi SVD instead of the reference's Lanczos bidiagonalization.  Signs: the first
 * nonzero entry of each A_r is made positive.  B: rank * bm*bn, A: rank * sm*sn. */
int or_ksvd(int bm, int bn, int sm, int sn, const double *M, int rank, double *B, double *A)
{
  const int rows = bm * bn, cols = sm * sn;
  if(rank < 1 || rank > (rows < cols ? rows : cols)) return -1;
  double *R = (double *)malloc(sizeof(double) * rows * cols);
  double *V = (double *)malloc(sizeof(double) * cols * cols);
  double *s = (double *)malloc(sizeof(double) * cols);
  const int ld = bn * sn;
  for(int k = 0; k < bm; ++k)
    for(int l = 0; l < bn; ++l)
      for(int i = 0; i < sm; ++i)
        for(int j = 0; j < sn; ++j)
          R[(k * bn + l) * cols + i * sn + j] = M[(k * sm + i) * ld + l * sn + j];
  svd_onesided(rows, cols, R, V, s);
  for(int r = 0; r < rank; ++r)
  {
    const double rs = sqrt(s[r]);
    double sign = 1.0;
    for(int j = 0; j < cols; ++j)
      if(fabs(V[j * cols + r]) > 1e-14) { sign = V[j * cols + r] > 0 ? 1.0 : -1.0; break; }
    for(int j = 0; j < cols; ++j) A[r * cols + j] = sign * V[j * cols + r] * rs;
    for(int i = 0; i < rows; ++i) B[r * rows + i] = s[r] > 0 ? sign * R[i * cols + r] / s[r] * rs : 0.0;
  }
  free(R);
  free(V);
  free(s);
  return 0;
}

/* Diagonal variant (TPSS/kroneckersvd.h:412-490): M = diag(d), d of length bm*sm; the
 * factors are diagonal, B_r = diag(u_r sqrt(sigma_r)), A_r = diag(v_r sqrt(sigma_r)).
 * Outputs the diagonals: B: rank * bm, A: rank * sm. */
int or_ksvd_diag(int bm, int sm, const double *d, int rank, double *B, double *A)
{
  if(rank < 1 || rank > (bm < sm ? bm : sm)) return -1;
  double *R = (double *)malloc(sizeof(double) * bm * sm);
  double *V = (double *)malloc(sizeof(double) * sm * sm);
  double *s = (double *)malloc(sizeof(double) * sm);
  memcpy(R, d, sizeof(double) * bm * sm);
  svd_onesided(bm, sm, R, V, s);
  for(int r = 0; r < rank; ++r)
  {
    const double rs = sqrt(s[r]);
    double sign = 1.0;
    for(int j = 0; j < sm; ++j)
      if(fabs(V[j * sm + r]) > 1e-14) { sign = V[j * sm + r] > 0 ? 1.0 : -1.0; break; }
    for(int j = 0; j < sm; ++j) A[r * sm + j] = sign * V[j * sm + r] * rs;
    for(int i = 0; i < bm; ++i) B[r * bm + i] = s[r] > 0 ? sign * R[i * sm + r] / s[r] * rs : 0.0;
  }
  free(R);
  free(V);
  free(s);
  return 0;
}

/* ===================================================================================== */
/*                         surrogate patches on distorted meshes                         */
/* ===================================================================================== */

/* Trilinear (bilinear) map of a cell with vertex coordinates X[2^dim][dim] (lexicographic
 * vertex order), evaluated at reference point xi. */
static void cell_map(int dim, const double *X, const double *xi, double *x)
{
  for(int c = 0; c < dim; ++c) x[c] = 0.0;
  for(int v = 0; v < (1 << dim); ++v)
  {
    double w = 1.0;
    for(int d = 0; d < dim; ++d) w *= ((v >> d) & 1) ? xi[d] : 1.0 - xi[d];
    for(int c = 0; c < dim; ++c) x[c] += w * X[v * dim + c];
  }
}

/* Average arc lengths between opposite faces of one cell (MappingInfo::compute_average_scaling,
 * TPSS/mapping_info.templates.h:42-240, use_arc_length = true): nq Gauss-Lobatto points per
 * direction; h_d = sum over face points of weight * length of the polyline through the nq
 * points of the fibre in direction d. */
static void cell_arc_lengths(int dim, const double *X, int nq, double *h)
{
  double z[32], wq[32];
  or_gauss_lobatto(nq, z);
  /* Gauss-Lobatto weights on [0,1]: w_i = 1/(n(n-1) P_{n-1}(x_i)^2) on [-1,1], halved */
  for(int i = 0; i < nq; ++i)
  {
    double p, dp;
    legendre_p(nq - 1, 2.0 * z[i] - 1.0, &p, &dp);
    if(i == 0 || i == nq - 1) p = (i == 0 && ((nq - 1) % 2)) ? -1.0 : 1.0;
    wq[i] = 1.0 / (nq * (nq - 1.0) * p * p);
  }
  for(int d = 0; d < dim; ++d)
  {
    double acc = 0.0;
    const int nf = dim == 2 ? nq : nq * nq;
    for(int f = 0; f < nf; ++f)
    {
      int fi[2] = {f % nq, f / nq};
      double wf = 1.0;
      for(int t = 0; t < dim - 1; ++t) wf *= wq[fi[t]];
      double len = 0.0, prev[3] = {0, 0, 0};
      for(int i = 0; i < nq; ++i)
      {
        double xi[3] = {0, 0, 0}, x[3];
        int t = 0;
        for(int e = 0; e < dim; ++e) xi[e] = e == d ? z[i] : z[fi[t++]];
        cell_map(dim, X, xi, x);
        if(i > 0)
        {
          double dd = 0.0;
          for(int c = 0; c < dim; ++c) dd += (x[c] - prev[c]) * (x[c] - prev[c]);
          len += sqrt(dd);
        }
        for(int c = 0; c < dim; ++c) prev[c] = x[c];
      }
      acc += wf * len;
    }
    h[d] = acc;
  }
}

/* Surrogate 1-D cell widths of every vertex patch of a structured mesh with distorted
 * vertex coordinates coords[(nx+1)(ny+1)(nz+1)][dim] (lexicographic vertices): for patch p and
 * direction d, out[(p*dim + d)*2 + c] = mean over the 2^(dim-1) patch cells with 1-D index c
 * of their arc length in direction d.  Patches in the oracle's order (or_patches). */
int or_surrogate_h(int dim, const int *nc_in, const double *coords, int nq, double *out)
{
  int nc[3] = {1, 1, 1};
  for(int d = 0; d < dim; ++d) nc[d] = nc_in[d];
  int ncol;
  int64_t P = or_patches(dim, nc, 1, 0, NULL, NULL, &ncol);
  int32_t *lower = (int32_t *)malloc(sizeof(int32_t) * 3 * (P ? P : 1));
  int32_t *color = (int32_t *)malloc(sizeof(int32_t) * (P ? P : 1));
  or_patches(dim, nc, 1, 0, lower, color, &ncol);
  const int nv0 = nc[0] + 1, nv1 = nc[1] + 1;
  for(int64_t p = 0; p < P; ++p)
  {
    double hsum[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for(int cn = 0; cn < (1 << dim); ++cn)
    {
      int c[3] = {lower[3 * p], lower[3 * p + 1], lower[3 * p + 2]};
      for(int d = 0; d < dim; ++d) c[d] += (cn >> d) & 1;
      double X[8 * 3];
      for(int v = 0; v < (1 << dim); ++v)
      {
        int vi[3] = {c[0], c[1], c[2]};
        for(int d = 0; d < dim; ++d) vi[d] += (v >> d) & 1;
        const int64_t vid = vi[0] + (int64_t)nv0 * (vi[1] + (int64_t)nv1 * vi[2]);
        for(int d = 0; d < dim; ++d) X[v * dim + d] = coords[vid * dim + d];
      }
      double h[3];
      cell_arc_lengths(dim, X, nq, h);
      for(int d = 0; d < dim; ++d) hsum[d][(cn >> d) & 1] += h[d] / (1 << (dim - 1));
    }
    for(int d = 0; d < dim; ++d)
      for(int c = 0; c < 2; ++c) out[(p * dim + d) * 2 + c] = hsum[d][c];
  }
  free(lower);
  free(color);
  return 0;
}

/* Additive vertex-patch Schwarz vmult with per-patch surrogate widths hp[(p*dim+d)*2+c]
 * (one FD problem per patch and direction), lexicographic cells. */
int or_schwarz_vmult_surrogate(int dim, int k, const int *nc_in, const double *hp, double ip,
                               double omega, const double *src, double *dst)
{
  int nc[3] = {1, 1, 1};
  for(int d = 0; d < dim; ++d) nc[d] = nc_in[d];
  double *hx = (double *)malloc(sizeof(double) * nc[0]);
  double *hy = (double *)malloc(sizeof(double) * nc[1]);
  double *hz = (double *)malloc(sizeof(double) * nc[2]);
  for(int c = 0; c < nc[0]; ++c) hx[c] = 1.0 / nc[0];
  for(int c = 0; c < nc[1]; ++c) hy[c] = 1.0 / nc[1];
  for(int c = 0; c < nc[2]; ++c) hz[c] = 1.0 / nc[2];
  level_t L;
  level_init(&L, dim, k, nc, hx, hy, hz, ip, NULL);
  patches_t T;
  patches_build(&T, &L, 1, 0);
  /* replace the FD entries by per-patch surrogate problems */
  free(T.cache.items);
  memset(&T.cache, 0, sizeof(T.cache));
  for(int64_t p = 0; p < T.P; ++p)
  {
    int32_t lo[3];
    /* recover the patch's lower cell from its first cell start */
    const int64_t cell0 = T.cell_first[p * T.npc] / L.ncell_dofs;
    lo[0] = (int32_t)(cell0 % nc[0]);
    lo[1] = (int32_t)((cell0 / nc[0]) % nc[1]);
    lo[2] = (int32_t)(cell0 / ((int64_t)nc[0] * nc[1]));
    for(int d = 0; d < dim; ++d)
    {
      /* always a new entry (no key sharing): index = p*dim + d */
      if(T.cache.n == T.cache.cap)
      {
        T.cache.cap = T.cache.cap ? 2 * T.cache.cap : 64;
        T.cache.items = (fd1d_t *)realloc(T.cache.items, sizeof(fd1d_t) * T.cache.cap);
      }
      fd1d_t *f = &T.cache.items[T.cache.n];
      const double hh[2] = {hp[(p * dim + d) * 2], hp[(p * dim + d) * 2 + 1]};
      const int blo = lo[d] == 0, bhi = lo[d] + 1 == nc[d] - 1;
      double M[OR_MAXN * OR_MAXN], A[OR_MAXN * OR_MAXN];
      or_patch_matrices_1d(k, 2, hh, blo, bhi, ip, M, A);
      if(or_gen_eig(2 * (k + 1), A, M, f->S, f->lam) != 0) return -1;
      f->ncp = 2;
      f->h0 = hh[0];
      f->h1 = hh[1];
      f->lo = blo;
      f->hi = bhi;
      T.fd[p * dim + d] = T.cache.n++;
    }
  }
  memset(dst, 0, sizeof(double) * L.n_dofs);
  for(int c = 0; c < T.ncol; ++c) apply_color(&L, &T, c, 2, omega, NULL, NULL, src, dst);
  patches_free(&T);
  free(hx);
  free(hy);
  free(hz);
  return 0;
}
