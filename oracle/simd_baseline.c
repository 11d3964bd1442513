/*
 * simd_baseline.c -- the timed CPU baseline of the Schwarz smoother: the reference's CPU path
 * restated with SIMD "macro patches".
 *
 * BENCH / TEST INFRASTRUCTURE ONLY.  bench.py's cpu_baseline leg and its reference arm time
 * it; tests/ check it against the strict oracle.  Nothing in the product links, loads or calls
 * it.
 *
 * The reference applies its smoother with deal.II's VectorizedArray: SubdomainHandler batches
 * the patches of a color into macro patches of VectorizedArray::size() lanes
 * (TPSS/patch_worker.h:497-611; empty lanes repeat lane 0, patch_worker.h:476-483), and per
 * macro patch SchwarzPreconditioner::apply_local_solvers
 * (preconditioner/schwarz_preconditioner.templates.h:585-662) gathers the lanes' DoFs
 * (PatchTransfer::gather, TPSS/patch_transfer.templates.h:3-23), applies the macro patch's own
 * TensorProductMatrixSymmetricSum inverse with lane-wise eigenvectors and eigenvalues (a dense
 * n x n contraction per direction, S^T ... divide by the eigenvalue sums ... S), scales by the
 * relaxation and scatter-adds the filled lanes (patch_transfer.templates.h:54-95).  Threads
 * share the macro patches of one color (the reference's TBB parloop over a race-free coloring,
 * subdomain_handler.templates.h:210-235).
 *
 * Here a macro patch holds VL = 8 lanes in GCC vector-extension registers (8 FP64 lanes, the
 * AVX-512 width of the reference's -march=native builds; the compiler maps them to the host's
 * vector unit: 4 x 128-bit NEON/SVE registers on Grace, whose SVE vectors are 128-bit, so an
 * -mcpu flag would not widen them).  Compiled with -O3 and contraction on (FMA), unlike the
 * strict oracle (-ffp-contract=off), which stays the checker.  The patch layout, colors and
 * 1-D eigenproblems come from the oracle's own code, included below.
 */
#include "tpss_oracle.c"

#define VL 8
typedef double vd __attribute__((vector_size(VL * sizeof(double))));

typedef struct
{
  schwarz_t S;
  int64_t n_macro;
  int64_t *color_macro; /* first macro patch of each color, ncol + 1 */
  int64_t *mp_first;    /* first patch of each macro patch */
  int *mp_lanes;        /* filled lanes */
  vd *Smat;             /* per macro patch and direction: n x n lane-wise eigenvectors */
  vd *lam;              /* per macro patch and direction: n lane-wise eigenvalues */
} simd_t;

/* out[.. i ..] = sum_m B(i, m) in[.. m ..] along direction d; B(i, m) = S[m][i] (forward, S^T)
 * or S[i][m] (backward).  Inlined with compile-time n, dim, d and transpose (deal.II's
 * sum-factorization kernels are templates on the same sizes), so the loops over i and m unroll
 * and the accumulators stay in registers. */
static inline __attribute__((always_inline)) void vd_dir(const int dim, const int n, const int d,
                                                        const vd *restrict S, const int transpose,
                                                        const vd *restrict in, vd *restrict out)
{
  const int stride = ipow(n, d), nouter = ipow(n, dim - 1 - d);
  for(int o = 0; o < nouter; ++o)
    for(int inner = 0; inner < stride; ++inner)
    {
      const int base = o * stride * n + inner;
      vd x[16];
      for(int m = 0; m < n; ++m) x[m] = in[base + m * stride];
      for(int i = 0; i < n; ++i)
      {
        vd acc = {0};
        for(int m = 0; m < n; ++m) acc += (transpose ? S[m * n + i] : S[i * n + m]) * x[m];
        out[base + i * stride] = acc;
      }
    }
}

#define VD_DIR_CASES(DIM, D, T)                                                                       \
  switch(n)                                                                                           \
  {                                                                                                   \
  case 2: vd_dir(DIM, 2, D, S, T, in, out); break;                                                    \
  case 3: vd_dir(DIM, 3, D, S, T, in, out); break;                                                    \
  case 4: vd_dir(DIM, 4, D, S, T, in, out); break;                                                    \
  case 5: vd_dir(DIM, 5, D, S, T, in, out); break;                                                    \
  case 6: vd_dir(DIM, 6, D, S, T, in, out); break;                                                    \
  case 7: vd_dir(DIM, 7, D, S, T, in, out); break;                                                    \
  case 8: vd_dir(DIM, 8, D, S, T, in, out); break;                                                    \
  case 10: vd_dir(DIM, 10, D, S, T, in, out); break;                                                  \
  case 12: vd_dir(DIM, 12, D, S, T, in, out); break;                                                  \
  case 14: vd_dir(DIM, 14, D, S, T, in, out); break;                                                  \
  case 16: vd_dir(DIM, 16, D, S, T, in, out); break;                                                  \
  default: break;                                                                                     \
  }

static void vd_apply_dir(int dim, int n, int d, const vd *restrict S, int transpose,
                         const vd *restrict in, vd *restrict out)
{
  if(dim == 2)
  {
    if(d == 0) { if(transpose) { VD_DIR_CASES(2, 0, 1) } else { VD_DIR_CASES(2, 0, 0) } }
    else { if(transpose) { VD_DIR_CASES(2, 1, 1) } else { VD_DIR_CASES(2, 1, 0) } }
  }
  else
  {
    if(d == 0) { if(transpose) { VD_DIR_CASES(3, 0, 1) } else { VD_DIR_CASES(3, 0, 0) } }
    else if(d == 1) { if(transpose) { VD_DIR_CASES(3, 1, 1) } else { VD_DIR_CASES(3, 1, 0) } }
    else { if(transpose) { VD_DIR_CASES(3, 2, 1) } else { VD_DIR_CASES(3, 2, 0) } }
  }
}

static void simd_macro(const simd_t *H, int64_t mp, const double *src, double *dst, vd *r, vd *t)
{
  const level_t *L = &H->S.L;
  const patches_t *T = &H->S.T;
  const int dim = L->dim, n = T->n, nloc = T->nloc, npc = T->npc, cd = L->ncell_dofs, np = L->np;
  const int ncp = H->S.ncp;
  const int64_t p0 = H->mp_first[mp];
  const int lanes = H->mp_lanes[mp];
  for(int l = 0; l < VL; ++l)
  {
    const int64_t p = p0 + (l < lanes ? l : 0);
    for(int cn = 0; cn < npc; ++cn)
    {
      const int64_t f = T->cell_first[p * npc + cn];
      for(int e = 0; e < cd; ++e) r[patch_index(dim, np, ncp, n, cn, e)][l] = src[f + e];
    }
  }
  const vd *S = H->Smat + (size_t)mp * dim * n * n;
  const vd *lam = H->lam + (size_t)mp * dim * n;
  for(int d = 0; d < dim; ++d)
  {
    vd_apply_dir(dim, n, d, S + (size_t)d * n * n, 1, r, t);
    vd *x = r; r = t; t = x;
  }
  const vd om = {H->S.omega, H->S.omega, H->S.omega, H->S.omega, H->S.omega, H->S.omega, H->S.omega,
                 H->S.omega};
  for(int i = 0; i < nloc; ++i)
  {
    vd l = {0};
    int rem = i;
    for(int d = 0; d < dim; ++d, rem /= n) l += lam[d * n + rem % n];
    r[i] /= l;
  }
  for(int d = 0; d < dim; ++d)
  {
    vd_apply_dir(dim, n, d, S + (size_t)d * n * n, 0, r, t);
    vd *x = r; r = t; t = x;
  }
  for(int l = 0; l < lanes; ++l)
  {
    const int64_t p = p0 + l;
    for(int cn = 0; cn < npc; ++cn)
    {
      const int64_t f = T->cell_first[p * npc + cn];
      for(int e = 0; e < cd; ++e) dst[f + e] += (om * r[patch_index(dim, np, ncp, n, cn, e)])[l];
    }
  }
}

/* Additive smoother of one structured level (vertex or cell patches), relaxation omega. */
void *or_simd_create(int dim, int k, const int *nc, int patch_variant, double omega)
{
  simd_t *H = (simd_t *)calloc(1, sizeof(simd_t));
  double *h[3];
  for(int d = 0; d < 3; ++d)
  {
    const int m = d < dim ? nc[d] : 1;
    h[d] = (double *)malloc(sizeof(double) * m);
    for(int c = 0; c < m; ++c) h[d][c] = 1.0 / m;
  }
  const int rc = schwarz_init(&H->S, dim, k, nc, h[0], h[1], h[2], 1.0, NULL, patch_variant, 0, omega, 0, 0, 0);
  /* level_init keeps pointers to h: they live as long as the handle (freed in destroy) */
  if(rc != 0)
  {
    free(H);
    return NULL;
  }
  const patches_t *T = &H->S.T;
  const int n = T->n;
  H->color_macro = (int64_t *)malloc(sizeof(int64_t) * (T->ncol + 1));
  int64_t nm = 0;
  for(int c = 0; c < T->ncol; ++c)
  {
    H->color_macro[c] = nm;
    nm += (T->color_start[c + 1] - T->color_start[c] + VL - 1) / VL;
  }
  H->color_macro[T->ncol] = nm;
  H->n_macro = nm;
  H->mp_first = (int64_t *)malloc(sizeof(int64_t) * (nm > 0 ? nm : 1));
  H->mp_lanes = (int *)malloc(sizeof(int) * (nm > 0 ? nm : 1));
  H->Smat = (vd *)aligned_alloc(64, sizeof(vd) * ((size_t)(nm > 0 ? nm : 1) * dim * n * n));
  H->lam = (vd *)aligned_alloc(64, sizeof(vd) * ((size_t)(nm > 0 ? nm : 1) * dim * n));
  for(int c = 0; c < T->ncol; ++c)
    for(int64_t m = H->color_macro[c]; m < H->color_macro[c + 1]; ++m)
    {
      const int64_t p0 = T->color_start[c] + (m - H->color_macro[c]) * VL;
      const int64_t left = T->color_start[c + 1] - p0;
      H->mp_first[m] = p0;
      H->mp_lanes[m] = left < VL ? (int)left : VL;
      for(int l = 0; l < VL; ++l)
      {
        const int64_t p = p0 + (l < H->mp_lanes[m] ? l : 0);
        for(int d = 0; d < dim; ++d)
        {
          const fd1d_t *f = &T->cache.items[T->fd[p * dim + d]];
          for(int i = 0; i < n * n; ++i) H->Smat[((size_t)m * dim + d) * n * n + i][l] = f->S[i];
          for(int i = 0; i < n; ++i) H->lam[((size_t)m * dim + d) * n + i][l] = f->lam[i];
        }
      }
    }
  return H;
}

int64_t or_simd_n_patches(void *h) { return ((simd_t *)h)->S.T.P; }

/* dst += the contributions of the patches [p_begin, p_end) (storage order, whole macro
 * patches: those whose first patch lies in the range); p_begin = 0, p_end = P after zeroing
 * dst is one vmult. */
void or_simd_apply_range(void *h, int64_t p_begin, int64_t p_end, double *dst, const double *src)
{
  const simd_t *H = (const simd_t *)h;
  const patches_t *T = &H->S.T;
  const int nloc = T->nloc;
  for(int c = 0; c < T->ncol; ++c)
  {
    const int64_t mb = H->color_macro[c], me = H->color_macro[c + 1];
#pragma omp parallel
    {
      vd *r = (vd *)aligned_alloc(64, sizeof(vd) * nloc);
      vd *t = (vd *)aligned_alloc(64, sizeof(vd) * nloc);
#pragma omp for schedule(static)
      for(int64_t m = mb; m < me; ++m)
        if(H->mp_first[m] >= p_begin && H->mp_first[m] < p_end) simd_macro(H, m, src, dst, r, t);
      free(r);
      free(t);
    }
  }
}

void or_simd_apply(void *h, double *dst, const double *src)
{
  const simd_t *H = (const simd_t *)h;
  memset(dst, 0, sizeof(double) * H->S.L.n_dofs);
  or_simd_apply_range(h, 0, H->S.T.P, dst, src);
}

void or_simd_destroy(void *h)
{
  simd_t *H = (simd_t *)h;
  if(!H) return;
  for(int d = 0; d < 3; ++d) free((void *)H->S.L.h[d]);
  schwarz_free(&H->S);
  free(H->color_macro);
  free(H->mp_first);
  free(H->mp_lanes);
  free(H->Smat);
  free(H->lam);
  free(H);
}
