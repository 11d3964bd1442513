// precond.cu -- SchwarzPreconditioner and SchwarzSmoother on the GPU.
//
// initialize (preconditioner/schwarz_preconditioner.templates.h:1-60): the 1-D SIPG
// mass/Laplace matrices of every distinct (h_left, h_right, boundary flags) patch direction are
// assembled on the host and their generalized eigenproblems are solved in FP64 on the GPU
// (compute_inverses, templates:101-123); the FD tables are kept in FP64 and FP32.
// vmult (templates:209-239): additive = dst := 0 then one fused kernel per color
// (additive_schwarz_operation, templates:665-688); multiplicative = residual update with the
// level operator between colors in the color sequence of get_color_sequence
// (schwarz_preconditioner.h:532-567, templates:691-732).
#include <chrono>
#include <cmath>
#include <cstring>

#include "internal.h"

namespace tpss
{

namespace
{
const char *kTimerNames[5] = {"[SchwarzPrecond] Update residuals:", "[SchwarzPrecond] Apply inverses:",
                              "[SchwarzPrecond] Compute inverses:",
                              "[SchwarzPrecond] Copy Locally Owned:", "[SchwarzPrecond] Step:"};

int pad_to(int n, int w) { return (n + w - 1) / w * w; }

// Mirror-symmetric 1-D problems (two equal cells, equal boundary flags) commute with the flip
// J: i -> n-1-i.  Their generalized eigenproblem splits into an even and an odd half problem
// in the bases e_j = (delta_j + delta_{n-1-j})/sqrt(2) and o_j = (delta_j - delta_{n-1-j})/sqrt(2),
// which lets the kernels contract with two h x h matrices (h = n/2) instead of one n x n.
// The resulting inverse is the same operator; only the rounding differs.
void build_even_odd(const tpss_layout &L, FdTables &T, const std::vector<double> &Ms,
                    const std::vector<double> &As, bool keyed)
{
  const int n = L.n, nn = n * n;
  T.lam_kernel = T.lam_host;  // mirror-symmetric entries are overwritten below
  std::vector<int32_t> sym(T.n_entries, 0);
  if(keyed && L.ncp == 2 && n % 2 == 0)
    for(int e = 0; e < T.n_entries; ++e)
    {
      const auto &k = L.fd_keys[e];
      sym[e] = k.h0 == k.h1 && k.lo == k.hi;
    }
  const int h = n / 2;
  T.hpad32 = pad_to(h, 4);
  T.hpad64 = pad_to(h, 2);
  const int npad = T.npad32, hp = T.hpad32;
  const int es = 4 * h * hp + npad;
  const int hp64 = T.hpad64, es64 = 4 * h * hp64 + T.npad64;
  std::vector<int> ids;
  for(int e = 0; e < T.n_entries; ++e)
    if(sym[e]) ids.push_back(e);
  std::vector<float> tab((size_t)std::max<size_t>(1, (size_t)T.n_entries) * es, 0.f);
  std::vector<double> tab64((size_t)std::max<size_t>(1, (size_t)T.n_entries) * es64, 0.0);
  if(!ids.empty())
  {
    const double r2 = 1.0 / std::sqrt(2.0);
    const int hh = h * h;
    std::vector<double> Mh(2 * ids.size() * hh), Ah(2 * ids.size() * hh);
    for(size_t u = 0; u < ids.size(); ++u)
    {
      const double *M = &Ms[(size_t)ids[u] * nn], *A = &As[(size_t)ids[u] * nn];
      for(int par = 0; par < 2; ++par)  // 0: even, 1: odd
      {
        const double sg = par == 0 ? 1.0 : -1.0;
        double *Mo = &Mh[(2 * u + par) * hh], *Ao = &Ah[(2 * u + par) * hh];
        for(int a = 0; a < h; ++a)
          for(int b = 0; b < h; ++b)
          {
            // x_a^T X x_b with x_a = (delta_a + sg delta_{n-1-a})/sqrt(2)
            auto proj = [&](const double *X) {
              const int a2 = n - 1 - a, b2 = n - 1 - b;
              return 0.5 * (X[a * n + b] + sg * X[a * n + b2] + sg * X[a2 * n + b] + X[a2 * n + b2]);
            };
            Mo[a * h + b] = proj(M);
            Ao[a * h + b] = proj(A);
          }
      }
    }
    std::vector<double> Sh, lamh;
    gen_eig_batched(h, (int)(2 * ids.size()), Mh, Ah, Sh, lamh);
    for(size_t u = 0; u < ids.size(); ++u)
    {
      float *E = &tab[(size_t)ids[u] * es];
      double *E64 = &tab64[(size_t)ids[u] * es64];
      for(int par = 0; par < 2; ++par)
      {
        const double *S = &Sh[(2 * u + par) * hh];
        for(int i = 0; i < h; ++i)
          for(int k = 0; k < h; ++k)
          {
            E[(par * h + k) * hp + i] = float(S[i * h + k] * r2);          // Se^T / So^T rows
            E[(2 * h + par * h + i) * hp + k] = float(S[i * h + k] * r2);  // Se / So rows
            E64[(par * h + k) * hp64 + i] = S[i * h + k] * r2;
            E64[(2 * h + par * h + i) * hp64 + k] = S[i * h + k] * r2;
          }
        for(int k = 0; k < h; ++k)
        {
          E[4 * h * hp + par * h + k] = float(lamh[(2 * u + par) * h + k]);
          E64[4 * h * hp64 + par * h + k] = lamh[(2 * u + par) * h + k];
          T.lam_kernel[(size_t)ids[u] * n + par * h + k] = lamh[(2 * u + par) * h + k];
        }
      }
    }
  }
  T.fd32_eo.upload(tab.data(), tab.size());
  T.fd64_eo.upload(tab64.data(), tab64.size());
  T.has_eo = !ids.empty();
  T.sym.upload(sym.data(), sym.size());
}

// 1 / (lambda_0 + .. + lambda_{dim-1}) for every combination of keyed entries, in the order the
// kernels read the eigenvalues (T.lam_kernel), summed as the kernels sum them (directions
// 0..dim-2 first, then the last)
void build_reciprocals(const tpss_layout &L, FdTables &T)
{
  const int n = L.n, dim = L.dim, E = T.n_entries;
  const int64_t nloc = ipow(n, dim);
  // E^dim n^dim values, at most 4 Mi (checked in floating point: E can be large on distorted
  // levels, whose surrogate patches have many distinct 1-D problems)
  if(E == 0 || std::pow(double(E), dim) * double(nloc) > double(int64_t(1) << 22)) return;
  const int64_t combos = ipow(E, dim);
  std::vector<double> r64((size_t)(combos * nloc));
  std::vector<float> r32(r64.size());
  for(int64_t c = 0; c < combos; ++c)
  {
    int e[3] = {0, 0, 0};
    for(int d = 0, rem = (int)c; d < dim; ++d, rem /= E) e[d] = rem % E;
    for(int64_t i = 0; i < nloc; ++i)
    {
      int id[3] = {0, 0, 0};
      for(int d = 0, rem = (int)i; d < dim; ++d, rem /= n) id[d] = rem % n;
      double lsum = 0.0;
      for(int d = 0; d < dim - 1; ++d) lsum += T.lam_kernel[(size_t)e[d] * n + id[d]];
      const double sum = lsum + T.lam_kernel[(size_t)e[dim - 1] * n + id[dim - 1]];
      r64[(size_t)(c * nloc + i)] = 1.0 / sum;
      r32[(size_t)(c * nloc + i)] = float(1.0 / sum);
    }
  }
  T.rcp64.upload(r64.data(), r64.size());
  T.rcp32.upload(r32.data(), r32.size());
  T.rcp_E = E;
}

}  // namespace

// 1-D patch matrices (mass, SIPG Laplace) of every FD key of the layout
void key_matrices(const tpss_layout &L, Penalty ip, std::vector<double> &Ms, std::vector<double> &As)
{
  const int n = L.n, nn = n * n, ne = (int)L.fd_keys.size();
  const Shape1D shape = make_shape_1d(L.k);
  Ms.assign((size_t)ne * nn, 0.0);
  As.assign((size_t)ne * nn, 0.0);
  for(int e = 0; e < ne; ++e)
  {
    const auto &key = L.fd_keys[e];
    const double h[2] = {key.h0, key.h1};
    patch_matrices_1d(shape, L.ncp, h, key.lo != 0, key.hi != 0, ip, &Ms[(size_t)e * nn],
                      &As[(size_t)e * nn]);
  }
}

// per patch and direction (entry p * dim + d): the 1-D matrices of the patch's FD key
std::vector<double> per_patch(const tpss_layout &L, const std::vector<double> &keyed)
{
  const size_t nn = (size_t)L.n * L.n;
  std::vector<double> out((size_t)L.P * L.dim * nn);
  for(int64_t i = 0; i < L.P * L.dim; ++i)
    std::copy_n(&keyed[(size_t)L.patch_fd_key[i] * nn], nn, &out[(size_t)i * nn]);
  return out;
}

// Replace, patch by patch, approximate 1-D problems whose Kronecker sum is not safely positive
// definite: the smallest eigenvalue of the sum, sum_d min_i lambda_(d,i), must stay at least half
// of the surrogate's, else the patch keeps the surrogate problems. Returns the patch count.
int64_t keep_definite(const tpss_layout &L, const std::vector<double> &Mp, std::vector<double> &Ap,
                      const std::vector<double> &Asur)
{
  const int n = L.n, nn = n * n, dim = L.dim;
  const int ne = (int)(L.P * dim);
  std::vector<double> S, lam, Ss, lams;
  gen_eig_batched(n, ne, Mp, Ap, S, lam);
  gen_eig_batched(n, ne, Mp, Asur, Ss, lams);
  int64_t count = 0;
  for(int64_t p = 0; p < L.P; ++p)
  {
    double snew = 0.0, ssur = 0.0;
    bool finite = true;
    for(int d = 0; d < dim; ++d)
    {
      const double *a = &lam[((size_t)p * dim + d) * n], *b = &lams[((size_t)p * dim + d) * n];
      double ma = a[0], mb = b[0];
      for(int i = 0; i < n; ++i)
      {
        finite = finite && std::isfinite(a[i]);
        ma = std::min(ma, a[i]);
        mb = std::min(mb, b[i]);
      }
      snew += ma;
      ssur += mb;
    }
    if(!(finite && snew >= 0.5 * ssur))
    {
      ++count;
      std::copy_n(&Asur[(size_t)p * dim * nn], (size_t)dim * nn, &Ap[(size_t)p * dim * nn]);
    }
  }
  return count;
}

namespace
{
// FD tables of the layout's keys, or (patchM, patchA given) of one 1-D problem per patch and
// direction
std::shared_ptr<FdTables> build_tables(const tpss_layout &L, Penalty ip, bool ras,
                                       const std::vector<double> *patchM = nullptr,
                                       const std::vector<double> *patchA = nullptr)
{
  auto t0 = std::chrono::steady_clock::now();
  auto T = std::make_shared<FdTables>();
  T->layout = &L;
  T->n = L.n;
  T->npad32 = pad_to(L.n, 4);
  T->npad64 = pad_to(L.n, 2);
  const int n = L.n, nn = n * n;
  std::vector<double> Ms, As;
  const bool keyed = patchM == nullptr;
  if(keyed)
  {
    key_matrices(L, ip, Ms, As);
    T->n_entries = (int)L.fd_keys.size();
  }
  else
  {
    TPSS_REQUIRE(L.P * L.dim < (int64_t)INT32_MAX, "too many patches");
    Ms = *patchM;
    As = *patchA;
    T->n_entries = (int)(L.P * L.dim);
    std::vector<int32_t> map((size_t)L.P * L.dim);
    for(size_t i = 0; i < map.size(); ++i) map[i] = (int32_t)i;
    T->own_fd.upload(map.data(), map.size());
  }
  gen_eig_batched(n, T->n_entries, Ms, As, T->S_host, T->lam_host);
  // kernel tables: [S^T n x npad][S n x npad][lambda npad]
  auto fill = [&](auto *dummy, int npad, std::vector<std::remove_pointer_t<decltype(dummy)>> &out) {
    using V = std::remove_pointer_t<decltype(dummy)>;
    const int es = (2 * n + 1) * npad;
    out.assign((size_t)T->n_entries * es, V(0));
    for(int e = 0; e < T->n_entries; ++e)
    {
      const double *S = &T->S_host[(size_t)e * nn], *lam = &T->lam_host[(size_t)e * n];
      V *E = &out[(size_t)e * es];
      for(int i = 0; i < n; ++i)
        for(int m = 0; m < n; ++m)
        {
          E[i * npad + m] = V(S[m * n + i]);              // S^T
          E[n * npad + i * npad + m] = V(S[i * n + m]);   // S
        }
      for(int i = 0; i < n; ++i) E[2 * n * npad + i] = V(lam[i]);
    }
  };
  std::vector<double> t64;
  std::vector<float> t32;
  fill((double *)nullptr, T->npad64, t64);
  fill((float *)nullptr, T->npad32, t32);
  T->fd64.upload(t64.data(), t64.size());
  T->fd32.upload(t32.data(), t32.size());
  build_even_odd(L, *T, Ms, As, keyed);
  if(keyed) build_reciprocals(L, *T);
  if(ras)
  {
    // RAS weights: 1 / (number of patches sharing the cell), the gathered "appearances" of
    // compute_ras_weights (schwarz_preconditioner.templates.h:126-165); DG DoFs of a cell
    // all have the same count.
    std::vector<float> w((size_t)L.P * L.npc);
    const std::vector<int64_t> &first = L.patch_first;
    std::vector<int32_t> mult_by_block(L.n_cells);
    for(int64_t c = 0; c < L.n_cells; ++c)
      mult_by_block[L.cell_start[c] / L.cell_dofs] = L.cell_multiplicity[c];
    for(size_t i = 0; i < w.size(); ++i) w[i] = 1.0f / float(mult_by_block[first[i] / L.cell_dofs]);
    T->ras_w.upload(w.data(), w.size());
  }
  T->setup_seconds =
    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return T;
}

// local solvers of a preconditioner according to desc.local_solver
std::shared_ptr<FdTables> build_local_solvers(const tpss_layout &L, const tpss_operator *op,
                                              const tpss_precond_desc &d)
{
  const bool ras = d.use_ras_weights != 0;
  const Penalty pen = make_penalty(d.ip_factor, d.penalty_mode, L.k);
  switch(d.local_solver)
  {
  case TPSS_LOCAL_EXACT:
  {
    check_exact_local(L, op);
    auto t0 = std::chrono::steady_clock::now();
    auto T = std::make_shared<FdTables>();
    T->layout = &L;
    T->n = L.n;
    T->dense = true;
    build_dense_inverses(L, *op, d.precision == TPSS_FP32, T->dense64, T->dense32);
    T->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return T;
  }
  case TPSS_LOCAL_KSUM:
  {
    check_exact_local(L, op);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> Mk, Ak;
    key_matrices(L, pen, Mk, Ak);
    const std::vector<double> Mp = per_patch(L, Mk);
    std::vector<double> Ap = ksum_fit(L, *op, Mp);
    const int64_t kept = keep_definite(L, Mp, Ap, per_patch(L, Ak));
    auto T = build_tables(L, pen, ras, &Mp, &Ap);
    T->learned_fallbacks = kept;
    T->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return T;
  }
  case TPSS_LOCAL_LEARNED:
    return build_learned_tables(L, d, [&](const std::vector<double> *Mp, const std::vector<double> *Ap) {
      return build_tables(L, pen, ras, Mp, Ap);
    });
  case TPSS_LOCAL_KSVD:
  {
    // Rank-2 Kronecker approximation X = F_(D-1),0 x .. x F_0,0 + F_(D-1),1 x .. x F_0,1 of the
    // exact patch matrix (ksvd_fit), inverted by simultaneous diagonalization of the two terms:
    // S_d^T F_d,0 S_d = I, S_d^T F_d,1 S_d = diag(mu_d) gives
    // X^-1 = S diag(1 / (1 + prod_d mu_d)) S^T, S = S_(D-1) x .. x S_0 -- fast diagonalization
    // with product-form eigenvalue combinations, which the kernels read from per-patch
    // reciprocal tables. A patch whose fit is not safely positive definite keeps its surrogate.
    check_exact_local(L, op);
    auto t0 = std::chrono::steady_clock::now();
    const int n = L.n, nn = n * n, dim = L.dim, nloc = L.nloc;
    std::vector<double> Mk, Ak;
    key_matrices(L, pen, Mk, Ak);
    const std::vector<double> Msur = per_patch(L, Mk), Asur = per_patch(L, Ak);
    const std::vector<double> F = ksvd_fit(L, *op, Msur, Asur, 14);  // rank^2 + 10 sweeps (compute_kcp)
    std::vector<double> F0((size_t)L.P * dim * nn), F1((size_t)L.P * dim * nn);
    for(int64_t p = 0; p < L.P; ++p)
      for(int dd = 0; dd < dim; ++dd)
      {
        const double *f = &F[((size_t)p * dim + dd) * 2 * nn];
        double *g0 = &F0[((size_t)p * dim + dd) * nn], *g1 = &F1[((size_t)p * dim + dd) * nn];
        double tr = 0.0;
        for(int i = 0; i < n; ++i) tr += f[i * n + i];
        const double sg = tr < 0.0 ? -1.0 : 1.0;  // sign pairs of term 0 so that every factor is positive
        for(int i = 0; i < n; ++i)
          for(int j = 0; j < n; ++j)
          {
            g0[i * n + j] = sg * 0.5 * (f[i * n + j] + f[j * n + i]);
            g1[i * n + j] = 0.5 * (f[nn + i * n + j] + f[nn + j * n + i]);
          }
      }
    std::vector<double> S, mu;
    std::vector<int> status;
    gen_eig_batched(n, (int)(L.P * dim), F0, F1, S, mu, &status);
    std::vector<char> use_ksvd((size_t)L.P, 1);
    for(int64_t p = 0; p < L.P; ++p)
    {
      // term 0 positive definite in every direction (after the sign flips, which must pair up)
      // and 1 + prod mu clearly positive
      for(int dd = 0; dd < dim; ++dd)
        if(status[(size_t)p * dim + dd]) use_ksvd[p] = 0;
      if(!use_ksvd[p]) continue;
      int flips = 0;
      for(int dd = 0; dd < dim; ++dd)
      {
        const double *f = &F[((size_t)p * dim + dd) * 2 * nn];
        double tr = 0.0;
        for(int i = 0; i < n; ++i) tr += f[i * n + i];
        flips += tr < 0.0;
      }
      double lo = 1e300, hi = 0.0;
      bool ok = flips % 2 == 0;
      for(int i = 0; i < nloc && ok; ++i)
      {
        double prod = 1.0;
        for(int dd = 0, rem = i; dd < dim; ++dd, rem /= n) prod *= mu[((size_t)p * dim + dd) * n + rem % n];
        const double v = 1.0 + prod;
        ok = std::isfinite(v);
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
      use_ksvd[p] = ok && lo > 1e-3 * hi;
    }
    std::vector<double> Mp(F0), Ap(F1);
    int64_t kept = 0;
    for(int64_t p = 0; p < L.P; ++p)
      if(!use_ksvd[p])
      {
        ++kept;
        std::copy_n(&Msur[(size_t)p * dim * nn], (size_t)dim * nn, &Mp[(size_t)p * dim * nn]);
        std::copy_n(&Asur[(size_t)p * dim * nn], (size_t)dim * nn, &Ap[(size_t)p * dim * nn]);
      }
    auto T = build_tables(L, pen, ras, &Mp, &Ap);
    // per-patch reciprocal eigenvalue combinations: product form for the fitted patches, the
    // Kronecker sum for the surrogate ones
    std::vector<double> r64((size_t)L.P * nloc);
    std::vector<float> r32(r64.size());
    for(int64_t p = 0; p < L.P; ++p)
      for(int i = 0; i < nloc; ++i)
      {
        double prod = 1.0, lsum = 0.0;
        for(int dd = 0, rem = i; dd < dim; ++dd, rem /= n)
        {
          const double l = T->lam_host[((size_t)p * dim + dd) * n + rem % n];
          prod *= l;
          lsum += l;
        }
        const double v = use_ksvd[p] ? 1.0 / (1.0 + prod) : 1.0 / lsum;
        r64[(size_t)p * nloc + i] = v;
        r32[(size_t)p * nloc + i] = float(v);
      }
    T->rcp64.upload(r64.data(), r64.size());
    T->rcp32.upload(r32.data(), r32.size());
    T->rcp_E = -1;  // one table per patch
    T->learned_fallbacks = kept;
    T->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return T;
  }
  default:
    return build_tables(L, pen, ras);
  }
}

void validate_desc(const tpss_precond_desc &d)
{
  TPSS_REQUIRE(d.kernel_variant >= TPSS_KERNEL_AUTO && d.kernel_variant <= TPSS_KERNEL_STREAM,
               "invalid kernel variant");
  TPSS_REQUIRE(d.stream_variant >= 0 && d.stream_variant <= 7, "stream_variant must be in 0..7");
  TPSS_REQUIRE(d.relaxation > 0.0, "Invalid relaxation factor.");
  TPSS_REQUIRE(d.precision == TPSS_FP64 || d.precision == TPSS_FP32, "invalid precision");
  TPSS_REQUIRE(d.penalty_mode == TPSS_PENALTY_REFERENCE || d.penalty_mode == TPSS_PENALTY_2KP1SQ,
               "invalid penalty_mode");
  TPSS_REQUIRE(d.local_solver >= TPSS_LOCAL_FD && d.local_solver <= TPSS_LOCAL_KSVD,
               "invalid local solver");
  if(d.local_solver == TPSS_LOCAL_EXACT && d.use_ras_weights)
    fail(TPSS_ERR_NOT_IMPLEMENTED, "RAS weights are implemented for the FD local solvers");
  if(d.local_solver == TPSS_LOCAL_LEARNED)
    TPSS_REQUIRE(d.model != nullptr, "the learned local solver needs a trained model");
  if(d.use_ras_weights && d.use_ras_boolean_weights)
    fail(TPSS_ERR_INVALID_ARGUMENT, "It isn't possible to use more than one RAS option.");
  if(d.local_solver == TPSS_LOCAL_EXACT && d.use_ras_boolean_weights)
    fail(TPSS_ERR_NOT_IMPLEMENTED, "RAS boolean weights are implemented for the FD local solvers");
}

// RAS boolean weights need additive vertex patches (DoFInfo::compute_restricted_dofs_impl,
// TPSS/dof_info.templates.h:194-216)
void validate_ras_boolean(const tpss_layout &L, const tpss_precond_desc &d)
{
  if(!d.use_ras_boolean_weights) return;
  if(L.patch_variant != TPSS_PATCH_VERTEX)
    fail(TPSS_ERR_NOT_IMPLEMENTED, "RAS boolean weights: only vertex patches are supported (TODO in the reference)");
  TPSS_REQUIRE(L.smoother_variant == TPSS_ADDITIVE, "RAS boolean weights: Additive scheme is only supported.");
}

// Restricted prolongation of the RAS boolean weights. Of the (up to 2^dim) vertex patches that
// hold a DoF, only the one where the DoF has the smallest (distance to the patch centre,
// patch-local index) scatters it; the distance is max_d trunc(|n/2 - 1/2 - m_d|) for the
// patch-local 1-D indices m_d (dof_info.templates.h:233-313). Two patches never give the same
// (distance, index) pair, so the reference's last tie-break (patch id) never applies, and the
// choice depends only on which neighbouring patches exist: per patch the class
// sum_d (lo_d + 2 hi_d) 4^d of its boundary flags (lo_d: no patch below in direction d, hi_d:
// none above).
void build_keep_tables(const tpss_layout &L, FdTables &T)
{
  if(T.keep_mask.n) return;
  const int dim = L.dim, n = L.n, K1 = L.np, nloc = L.nloc, ncls = ipow(4, dim);
  auto dist_of = [&](const int *m) {
    int dist = 0;
    for(int d = 0; d < dim; ++d) dist = std::max(dist, (int)std::fabs(0.5 * n - 0.5 - m[d]));
    return dist;
  };
  std::vector<unsigned char> mask((size_t)ncls * nloc, 0);
  for(int c = 0; c < ncls; ++c)
    for(int i = 0; i < nloc; ++i)
    {
      int m[3] = {0, 0, 0};
      for(int d = 0, rem = i; d < dim; ++d, rem /= n) m[d] = rem % n;
      const int own = dist_of(m);
      bool keep = true;
      for(int f = 1; f < (1 << dim) && keep; ++f)
      {
        int m2[3] = {m[0], m[1], m[2]};
        bool exists = true;
        for(int d = 0; d < dim; ++d)
          if(f >> d & 1)
          {
            const bool lower_cell = m[d] < K1;  // the DoF's cell is this patch's lower cell
            const int flag = (c >> (2 * d + (lower_cell ? 0 : 1))) & 1;
            exists = exists && !flag;
            m2[d] = lower_cell ? m[d] + K1 : m[d] - K1;
          }
        if(!exists) continue;
        int i2 = 0;
        for(int d = dim - 1; d >= 0; --d) i2 = i2 * n + m2[d];
        const int other = dist_of(m2);
        if(other < own || (other == own && i2 < i)) keep = false;
      }
      mask[(size_t)c * nloc + i] = keep;
    }
  std::vector<int32_t> cls(L.P);
  for(int64_t p = 0; p < L.P; ++p)
  {
    int c = 0;
    for(int d = dim - 1; d >= 0; --d)
    {
      const int lo = L.lower[p * 3 + d] == 0, hi = L.lower[p * 3 + d] + 2 == L.nc[d];
      c = c * 4 + lo + 2 * hi;
    }
    cls[p] = c;
  }
  T.keep_class.upload(cls.data(), cls.size());
  T.keep_mask.upload(mask.data(), mask.size());
}

cudaEvent_t get_event(tpss_precond *p)
{
  if(!p->event_pool.empty())
  {
    cudaEvent_t e = p->event_pool.back();
    p->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  TPSS_CUDA(cudaEventCreate(&e));
  return e;
}

// Timers are read lazily: start/stop events are recorded on the stream and resolved when
// the caller asks for the time data (or when too many are pending).
void harvest(tpss_precond *p, bool all)
{
  size_t keep_from = 0;
  for(size_t i = 0; i < p->pending.size(); ++i)
  {
    auto &pe = p->pending[i];
    if(!all && cudaEventQuery(pe.stop) != cudaSuccess)
    {
      keep_from = i;
      break;
    }
    TPSS_CUDA(cudaEventSynchronize(pe.stop));
    float ms = 0.f;
    TPSS_CUDA(cudaEventElapsedTime(&ms, pe.start, pe.stop));
    p->timers[pe.slot].time += ms * 1e-3;
    p->timers[pe.slot].n_calls += 1;
    p->event_pool.push_back(pe.start);
    p->event_pool.push_back(pe.stop);
    keep_from = i + 1;
  }
  p->pending.erase(p->pending.begin(), p->pending.begin() + keep_from);
}

struct ScopedTimer
{
  tpss_precond *p;
  int slot;
  cudaStream_t s;
  cudaEvent_t start = nullptr;
  bool enabled;
  ScopedTimer(tpss_precond *p_, int slot_, cudaStream_t s_) : p(p_), slot(slot_), s(s_)
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    enabled = cs == cudaStreamCaptureStatusNone;  // no event timing inside graph capture
    if(enabled)
    {
      start = get_event(p);
      TPSS_CUDA(cudaEventRecord(start, s));
    }
  }
  ~ScopedTimer()
  {
    if(!enabled) return;
    cudaEvent_t stop = nullptr;
    try
    {
      stop = get_event(p);
    }
    catch(...)
    {
      return;
    }
    cudaEventRecord(stop, s);
    p->pending.push_back({start, stop, slot});
    if(p->pending.size() > 256)
    {
      try
      {
        harvest(p, false);
      }
      catch(...)
      {
      }
    }
  }
};

__global__ void finite_check_kernel(const double *__restrict__ x, int64_t n, int *flag)
{
  int bad = 0;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(x[i]);
  if(__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

void apply_color(tpss_precond *p, int color, double *dst, const double *src, cudaStream_t s)
{
  const tpss_layout &L = *p->tables->layout;
  const int64_t b = L.color_start[color], e = L.color_start[color + 1];
  if(e <= b) return;
  if(p->tables->dense)
  {
    const bool f32 = p->desc.precision == TPSS_FP32;
    dense_apply_color(L, f32 ? (const void *)p->tables->dense32.ptr : (const void *)p->tables->dense64.ptr,
                      f32, color, p->desc.relaxation, dst, src, s);
    return;
  }
  FdLaunch a;
  a.src = src;
  a.dst = dst;
  a.patch_first = L.d_patch_first.ptr + b * L.npc;
  a.patch_fd = (p->tables->own_fd.n ? p->tables->own_fd.ptr : L.d_patch_fd.ptr) + b * L.dim;
  const bool ras = p->desc.use_ras_weights && L.smoother_variant == TPSS_ADDITIVE;
  a.ras_w = ras ? p->tables->ras_w.ptr + b * L.npc : nullptr;
  if(p->desc.use_ras_boolean_weights)
  {
    a.keep_mask = p->tables->keep_mask.ptr;
    a.keep_class = p->tables->keep_class.ptr + b;
  }
  a.n_patches = e - b;
  a.omega = p->desc.relaxation;
  a.variant = p->color_variant;
  bool ok;
  // even/odd forms of the mirror-symmetric entries (shared keyed tables only; per-patch tables
  // of the fitted and learned solvers have none)
  const bool eo = p->tables->has_eo && !p->tables->own_fd.n;
  const int h = L.n / 2;
  a.sym = eo ? p->tables->sym.ptr : nullptr;
  // reciprocal eigenvalue combinations: per combination of keyed entries (rcp_E > 0) or per
  // patch (rcp_E < 0, the first patch of the color at offset b)
  const bool rcp = p->tables->rcp_E != 0;
  const int64_t rcp_off = p->tables->rcp_E < 0 ? b * (int64_t)L.nloc : 0;
  a.rcp_E = p->tables->rcp_E;
  if(p->desc.precision == TPSS_FP32)
  {
    a.rcp = rcp ? (const void *)(p->tables->rcp32.ptr + rcp_off) : nullptr;
    a.fd = p->tables->fd32.ptr;
    a.entry_stride = (2 * L.n + 1) * p->tables->npad32;
    a.fd_eo = eo ? (const void *)p->tables->fd32_eo.ptr : nullptr;
    a.eo_stride = 4 * h * p->tables->hpad32 + p->tables->npad32;
    ok = launch_fd_f32(L.dim, L.k, L.ncp, a, s);
  }
  else
  {
    a.rcp = rcp ? (const void *)(p->tables->rcp64.ptr + rcp_off) : nullptr;
    a.fd = p->tables->fd64.ptr;
    a.entry_stride = (2 * L.n + 1) * p->tables->npad64;
    a.fd_eo = eo ? (const void *)p->tables->fd64_eo.ptr : nullptr;
    a.eo_stride = 4 * h * p->tables->hpad64 + p->tables->npad64;
    ok = launch_fd_f64(L.dim, L.k, L.ncp, a, s);
  }
  if(!ok)
  {
    cudaError_t err = cudaGetLastError();
    fail(TPSS_ERR_CUDA, std::string("Schwarz color kernel launch failed: ") + cudaGetErrorString(err));
  }
}
}  // namespace

bool launch_fd_float_2(int k, int ncp, const FdLaunch &a, cudaStream_t s);
bool launch_fd_float_3(int k, int ncp, const FdLaunch &a, cudaStream_t s);
bool launch_fd_double_2(int k, int ncp, const FdLaunch &a, cudaStream_t s);
bool launch_fd_double_3(int k, int ncp, const FdLaunch &a, cudaStream_t s);

bool launch_fd_f32(int dim, int k, int ncp, const FdLaunch &a, cudaStream_t s)
{
  return dim == 2 ? launch_fd_float_2(k, ncp, a, s) : launch_fd_float_3(k, ncp, a, s);
}

bool launch_fd_f64(int dim, int k, int ncp, const FdLaunch &a, cudaStream_t s)
{
  return dim == 2 ? launch_fd_double_2(k, ncp, a, s) : launch_fd_double_3(k, ncp, a, s);
}

int fd_variants_float_2(int k, int ncp);
int fd_variants_float_3(int k, int ncp);
int fd_variants_double_2(int k, int ncp);
int fd_variants_double_3(int k, int ncp);

int fd_variants(bool fp32, int dim, int k, int ncp)
{
  if(fp32) return dim == 2 ? fd_variants_float_2(k, ncp) : fd_variants_float_3(k, ncp);
  return dim == 2 ? fd_variants_double_2(k, ncp) : fd_variants_double_3(k, ncp);
}

// the column-streamed FP32 smoother applies to this preconditioner: additive 3D vertex patches
// with k <= 5 and FD tables (keyed, or per patch up to k = 3 on distorted levels), not dense
// inverses or the rank-2 Kronecker solver's product-form eigenvalues
bool stream_eligible(const tpss_precond *p)
{
  const tpss_layout &L = *p->tables->layout;
  // per-patch tables (distorted levels) need Kronecker-sum patch inverses: not the product-form
  // eigenvalues of the rank-2 Kronecker solver (rcp_E < 0)
  const bool per_patch = L.per_patch_fd || p->tables->own_fd.n != 0;
  return L.smoother_variant == TPSS_ADDITIVE && p->desc.precision == TPSS_FP32 &&
         stream_supported(L) && !p->tables->dense && (!per_patch || L.k <= 3) && p->tables->rcp_E >= 0 &&
         !p->desc.use_ras_boolean_weights;
}

bool use_stream(const tpss_precond *p)
{
  if(p->desc.kernel_variant == TPSS_KERNEL_COLOR) return false;
  const bool ok = stream_eligible(p);
  if(p->desc.kernel_variant == TPSS_KERNEL_STREAM && !ok)
    fail(TPSS_ERR_INVALID_ARGUMENT,
         "the streamed kernel needs additive 3D vertex patches, FP32, k <= 5 and fast-diagonalization "
         "local solvers (per-patch 1-D problems: k <= 3)");
  return ok;
}

StreamLaunch stream_launch(tpss_precond *p, double *dst, const double *src)
{
  const tpss_layout &L = *p->tables->layout;
  StreamLaunch l;
  l.src = src;
  l.dst = dst;
  l.fd32 = p->tables->fd32.ptr;
  l.fd32_eo = p->tables->fd32_eo.ptr;
  l.sym = p->tables->sym.ptr;
  l.es_eo = 4 * (L.n / 2) * p->tables->hpad32 + p->tables->npad32;
  l.omega = p->desc.relaxation;
  l.ras = p->desc.use_ras_weights != 0;
  l.halo = &p->halo;
  l.variant = p->stream_variant;
  l.fix_rec = &p->fix_rec[p->stream_variant];
  l.fix_n = &p->fix_n[p->stream_variant];
  l.fix_layer = &p->fix_layer[p->stream_variant];
  l.per_patch = L.per_patch_fd || p->tables->own_fd.n != 0;
  if(l.per_patch)
  {
    FdTables &T = *p->tables;
    {
      // vertex -> patch map, built on first use (tables are shared by shallow copies)
      static std::mutex mu;
      std::lock_guard<std::mutex> lock(mu);
      if(T.vpatch.n == 0)
      {
        const int64_t nvx = L.nc[0] + 1, nvy = L.nc[1] + 1, nvz = L.nc[2] + 1;
        std::vector<int32_t> vp((size_t)(nvx * nvy * nvz), -1);
        for(int64_t q = 0; q < L.P; ++q)
        {
          const int64_t v = (L.lower[q * 3] + 1) + nvx * ((L.lower[q * 3 + 1] + 1) + nvy * (L.lower[q * 3 + 2] + 1));
          vp[(size_t)v] = (int32_t)q;
        }
        T.vpatch.upload(vp.data(), vp.size());
      }
    }
    l.vpatch = T.vpatch.ptr;
    l.pfd = T.own_fd.n ? T.own_fd.ptr : L.d_patch_fd.ptr;
  }
  return l;
}

void precond_vmult(tpss_precond *p, double *dst, const double *src, cudaStream_t s)
{
  const tpss_layout &L = *p->tables->layout;
  TPSS_REQUIRE(dst && src, "null vector");
  TPSS_REQUIRE(dst != src, "dst and src must not alias");
  ScopedTimer step(p, 4, s);
  if(!(L.smoother_variant == TPSS_ADDITIVE && use_stream(p)))
    TPSS_CUDA(cudaMemsetAsync(dst, 0, sizeof(double) * L.n_dofs, s));
  if(L.smoother_variant == TPSS_ADDITIVE)
  {
    ScopedTimer t(p, 1, s);
    if(use_stream(p))
    {
      // one pass over all patches; every cell of dst is written, no zeroing needed
      const StreamLaunch l = stream_launch(p, dst, src);
      if(!launch_stream3d(L, l, s)) fail(TPSS_ERR_CUDA, "streamed smoother launch failed");
    }
    else
      for(int c = 0; c < L.n_colors; ++c) apply_color(p, c, dst, src, s);
  }
  else
  {
    TPSS_REQUIRE(p->op, "the multiplicative smoother needs the level operator");
    std::vector<int> seq;
    for(int c = 0; c < L.n_colors; ++c) seq.push_back(p->desc.reverse ? L.n_colors - 1 - c : c);
    if(p->desc.symmetrized)
      for(int i = L.n_colors - 2; i >= 0; --i) seq.push_back(seq[i]);
    if(p->residual.n < (size_t)L.n_dofs) p->residual.resize(L.n_dofs);
    double *res = p->residual.ptr;
    {
      ScopedTimer t(p, 1, s);
      apply_color(p, seq[0], dst, src, s);
    }
    for(size_t i = 1; i < seq.size(); ++i)
    {
      {
        ScopedTimer t(p, 0, s);
        operator_apply(p->op, res, dst, s);
        vec_sub(L.n_dofs, src, res, s);  // res = src - A dst
      }
      ScopedTimer t(p, 1, s);
      apply_color(p, seq[i], dst, res, s);
    }
  }
  if(p->desc.check_finite)
  {
    if(p->flag.n == 0) p->flag.resize(1);
    TPSS_CUDA(cudaMemsetAsync(p->flag.ptr, 0, sizeof(int), s));
    finite_check_kernel<<<num_sms() * 4, 256, 0, s>>>(dst, L.n_dofs, p->flag.ptr);
    TPSS_CUDA(cudaGetLastError());
    int h = 0;
    TPSS_CUDA(cudaMemcpyAsync(&h, p->flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    TPSS_CUDA(cudaStreamSynchronize(s));
    if(h) fail(TPSS_ERR_NOT_FINITE, "vmult produced a non-finite value");
  }
}
}  // namespace tpss

using namespace tpss;

struct tpss_smoother
{
  tpss_operator *op = nullptr;
  tpss_precond *p = nullptr;
  int n_steps = 1;
  double damping = 1.0;
  DeviceBuffer<double> residual, tmp;
};

extern "C" int tpss_precond_create(const tpss_layout *layout, tpss_operator *op,
                                   const tpss_precond_desc *desc, tpss_precond **out)
{
  return guarded([&] {
    TPSS_REQUIRE(layout && desc && out, "null argument");
    *out = nullptr;
    validate_desc(*desc);
    validate_ras_boolean(*layout, *desc);
    if(layout->smoother_variant == TPSS_MULTIPLICATIVE)
    {
      TPSS_REQUIRE(op, "the multiplicative smoother needs the level operator");
      TPSS_REQUIRE(op->layout->n_dofs == layout->n_dofs, "operator does not match the layout");
    }
    layout_to_device(*layout);
    auto p = std::make_unique<tpss_precond>();
    p->desc = *desc;
    p->op = op;
    // a decomposition the level does not offer (the plane passes need k = 4) falls back to 0
    p->stream_variant = desc->stream_variant < stream_variant_count(*layout) ? desc->stream_variant : 0;
    p->color_variant = desc->stream_variant;  // variants the kernel does not offer fall back to 0
    p->tables = build_local_solvers(*layout, op, *desc);
    if(desc->use_ras_boolean_weights) build_keep_tables(*layout, *p->tables);
    p->timers.resize(5);
    for(int i = 0; i < 5; ++i) p->timers[i].name = kTimerNames[i];
    p->timers[2].time = p->tables->setup_seconds;
    p->timers[2].n_calls = 1;
    *out = p.release();
  });
}

extern "C" int tpss_precond_create_shallow(const tpss_precond *other, const tpss_precond_desc *desc,
                                           tpss_precond **out)
{
  return guarded([&] {
    TPSS_REQUIRE(other && desc && out, "null argument");
    *out = nullptr;
    validate_desc(*desc);
    TPSS_REQUIRE(desc->ip_factor == other->desc.ip_factor,
                 "shallow copies share the local solvers: ip_factor must match");
    TPSS_REQUIRE(desc->penalty_mode == other->desc.penalty_mode,
                 "shallow copies share the local solvers: penalty_mode must match");
    TPSS_REQUIRE(desc->local_solver == other->desc.local_solver && desc->model == other->desc.model,
                 "shallow copies share the local solvers: local_solver must match");
    if(other->tables->dense)
      TPSS_REQUIRE(desc->precision == other->desc.precision,
                   "shallow copies of dense local inverses keep the precision");
    auto p = std::make_unique<tpss_precond>();
    p->desc = *desc;
    p->op = other->op;
    p->tables = other->tables;
    if(desc->use_ras_weights && p->tables->ras_w.n == 0)
      fail(TPSS_ERR_INVALID_ARGUMENT, "shallow copy cannot add RAS weights");
    validate_ras_boolean(*p->tables->layout, *desc);
    if(desc->use_ras_boolean_weights) build_keep_tables(*p->tables->layout, *p->tables);
    p->timers = other->timers;
    *out = p.release();
  });
}

extern "C" int tpss_precond_vmult(tpss_precond *p, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(p, "null preconditioner");
    precond_vmult(p, dst, src, as_stream(stream));
  });
}

extern "C" int tpss_precond_vmult_add(tpss_precond *p, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(p, "null preconditioner");
    const int64_t n = p->tables->layout->n_dofs;
    if(p->residual.n < (size_t)n) p->residual.resize(n);
    // vmult into the scratch vector, then dst += scratch (multiplicative also uses the
    // scratch for its residual, so it gets its own temporary)
    if(p->tables->layout->smoother_variant == TPSS_MULTIPLICATIVE)
    {
      DeviceBuffer<double> tmp(n);
      precond_vmult(p, tmp.ptr, src, as_stream(stream));
      vec_axpby(n, 1.0, tmp.ptr, 1.0, dst, as_stream(stream));
      TPSS_CUDA(cudaStreamSynchronize(as_stream(stream)));
    }
    else
    {
      precond_vmult(p, p->residual.ptr, src, as_stream(stream));
      vec_axpby(n, 1.0, p->residual.ptr, 1.0, dst, as_stream(stream));
    }
  });
}

extern "C" int tpss_precond_Tvmult(tpss_precond *p, double *, const double *, void *)
{
  return guarded([&] {
    TPSS_REQUIRE(p, "null preconditioner");
    fail(TPSS_ERR_NOT_IMPLEMENTED, "TODO transpose operation is not implemented.");
  });
}

extern "C" int tpss_precond_time_info(tpss_precond *p, tpss_time_info *out, int *n_inout)
{
  return guarded([&] {
    TPSS_REQUIRE(p && n_inout, "null argument");
    harvest(p, true);
    const int n = (int)p->timers.size();
    if(out)
    {
      const int m = std::min(n, *n_inout);
      for(int i = 0; i < m; ++i)
      {
        out[i].time = p->timers[i].time;
        out[i].n_calls = p->timers[i].n_calls;
        std::snprintf(out[i].description, sizeof(out[i].description), "%s", p->timers[i].name);
      }
    }
    *n_inout = n;
  });
}

extern "C" void tpss_precond_destroy(tpss_precond *p)
{
  if(!p) return;
  for(auto &pe : p->pending)
  {
    cudaEventSynchronize(pe.stop);
    cudaEventDestroy(pe.start);
    cudaEventDestroy(pe.stop);
  }
  for(auto e : p->event_pool) cudaEventDestroy(e);
  delete p;
}

extern "C" int tpss_smoother_create(tpss_operator *op, tpss_precond *p, int n_steps,
                                    double damping, tpss_smoother **out)
{
  return guarded([&] {
    TPSS_REQUIRE(op && p && out, "null argument");
    TPSS_REQUIRE(n_steps >= 1, "n_steps must be positive");
    TPSS_REQUIRE(op->layout->n_dofs == p->tables->layout->n_dofs, "operator/preconditioner mismatch");
    auto s = std::make_unique<tpss_smoother>();
    s->op = op;
    s->p = p;
    s->n_steps = n_steps;
    s->damping = damping;
    *out = s.release();
  });
}

namespace
{
void smoother_steps(tpss_smoother *sm, double *x, const double *b, cudaStream_t s)
{
  const int64_t n = sm->p->tables->layout->n_dofs;
  if(sm->residual.n < (size_t)n) sm->residual.resize(n);
  if(sm->tmp.n < (size_t)n) sm->tmp.resize(n);
  for(int k = 0; k < sm->n_steps; ++k)
  {
    operator_apply(sm->op, sm->residual.ptr, x, s);  // r = A x
    vec_sub(n, b, sm->residual.ptr, s);              // r = b - A x
    precond_vmult(sm->p, sm->tmp.ptr, sm->residual.ptr, s);
    vec_axpby(n, sm->damping, sm->tmp.ptr, 1.0, x, s);  // x += damping P r
  }
}
}  // namespace

extern "C" int tpss_smoother_step(tpss_smoother *sm, double *x, const double *b, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(sm && x && b, "null argument");
    smoother_steps(sm, x, b, as_stream(stream));
  });
}

extern "C" int tpss_smoother_vmult(tpss_smoother *sm, double *x, const double *b, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(sm && x && b, "null argument");
    TPSS_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * sm->p->tables->layout->n_dofs,
                              as_stream(stream)));
    smoother_steps(sm, x, b, as_stream(stream));
  });
}

extern "C" void tpss_smoother_destroy(tpss_smoother *s) { delete s; }

extern "C" int tpss_precond_autotune(tpss_precond *p, double *dst, const double *src, int reps,
                                     int *chosen, double *ms_per_variant, int *n_variants,
                                     void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(p && dst && src && reps >= 1, "invalid argument");
    cudaStream_t s = as_stream(stream);
    const tpss_layout &L = *p->tables->layout;
    // the streamed kernel's work decompositions, or the per-color kernel's patches per CTA
    // (dense local inverses have a single kernel)
    const bool streamed = use_stream(p);
    const int nv = streamed ? stream_variant_count(L)
                   : p->tables->dense ? 1
                                      : fd_variants(p->desc.precision == TPSS_FP32, L.dim, L.k, L.ncp);
    int &variant = streamed ? p->stream_variant : p->color_variant;
    if(n_variants) *n_variants = nv;
    if(nv <= 1)
    {
      if(chosen) *chosen = 0;
      if(ms_per_variant) ms_per_variant[0] = 0.;  // a single variant is not timed
      precond_vmult(p, dst, src, s);
      return;
    }
    struct Events
    {
      cudaEvent_t e[2] = {nullptr, nullptr};
      ~Events()
      {
        for(cudaEvent_t x : e)
          if(x) cudaEventDestroy(x);
      }
    } ev;
    TPSS_CUDA(cudaEventCreate(&ev.e[0]));
    TPSS_CUDA(cudaEventCreate(&ev.e[1]));
    cudaEvent_t e0 = ev.e[0], e1 = ev.e[1];
    int best = 0;
    float best_ms = 0.f;
    for(int v = 0; v < nv; ++v)
    {
      variant = v;
      precond_vmult(p, dst, src, s);  // warm-up (scratch sizing, attributes)
      TPSS_CUDA(cudaEventRecord(e0, s));
      for(int r = 0; r < reps; ++r) precond_vmult(p, dst, src, s);
      TPSS_CUDA(cudaEventRecord(e1, s));
      TPSS_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      TPSS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      ms /= reps;
      if(ms_per_variant) ms_per_variant[v] = ms;
      if(v == 0 || ms < best_ms)
      {
        best = v;
        best_ms = ms;
      }
    }
    variant = best;
    if(chosen) *chosen = best;
    precond_vmult(p, dst, src, s);  // dst holds the chosen variant's result
  });
}

extern "C" int tpss_precond_vmult_host(tpss_precond *p, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(p && dst && src, "null argument");
    TPSS_REQUIRE(dst != src, "dst and src must not alias");
    cudaStream_t s = as_stream(stream);
    const tpss_layout &L = *p->tables->layout;
    const size_t N = (size_t)L.n_dofs;
    if(p->pipe.src.n < N) p->pipe.src.resize(N);
    if(p->pipe.dst.n < N) p->pipe.dst.resize(N);
    ScopedTimer step(p, 4, s);
    if(L.smoother_variant == TPSS_ADDITIVE && use_stream(p) && !p->desc.check_finite)
    {
      // The pipeline is copy-bound (262 MB each way at 64^3 DGQ4 against a 1.3 ms kernel); its
      // fill and drain are one chunk of one z-item, so it runs the 4-layer-deep twin of the
      // chosen decomposition (warp per patch: 4 -> 5, plane passes: 6 -> 7, otherwise 2), which
      // halves both.
      StreamLaunch l = stream_launch(p, p->pipe.dst.ptr, p->pipe.src.ptr);
      const int sv = p->stream_variant;
      const int hv = (sv == 4 || sv == 5) ? 5 : (sv == 6 || sv == 7) ? 7 : 2;
      l.variant = hv;
      l.fix_rec = &p->fix_rec[hv];
      l.fix_n = &p->fix_n[hv];
      l.fix_layer = &p->fix_layer[hv];
      if(launch_stream3d_host(L, l, p->pipe, dst, src, s)) return;
    }
    TPSS_CUDA(cudaMemcpyAsync(p->pipe.src.ptr, src, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    precond_vmult(p, p->pipe.dst.ptr, p->pipe.src.ptr, s);
    TPSS_CUDA(cudaMemcpyAsync(dst, p->pipe.dst.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
  });
}
