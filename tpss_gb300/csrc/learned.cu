// Learned local solver: surrogate 1-D patch problems corrected by a trained network.
//
// On a distorted level the reference's local solver is fast diagonalization of surrogate
// Cartesian patches (mapping_info.templates.h:42-240): per direction d a 1-D problem
// (M_d, A_d). Here a network maps the patch's vertex geometry to a correction of each A_d,
// scaled by the surrogate diagonal D = diag(A_d):
//     T_d = D^-1/2 (A_d' - A_d) D^-1/2,
// whose targets come from the Kronecker sum fitted to the EXACT patch matrix with the same
// masses (local.cu): A_d' = A_d^fit. At inference A_d' = A_d + D^1/2 T_d D^1/2 is
// diagonalized with M_d like any FD entry, so the smoother kernels are unchanged. A patch
// direction whose corrected A_d' is not positive definite, or a patch whose corrected
// Kronecker sum loses more than half of the surrogate's smallest eigenvalue, keeps the
// surrogate problems (the fallback).
//
// Network input per vertex patch (3^d vertices): the displacement of every patch vertex from
// the regular lattice around the patch's centre vertex, coordinate d in units of the patch's
// mean surrogate width in direction d, followed by the 2d boundary flags of the patch's 1-D
// problems. Output: the upper
// triangles (row-major, i <= j) of T_0 ... T_(d-1).
#include "internal.h"

#include <chrono>
#include <cmath>

namespace tpss
{
namespace
{
int n_in_of(const tpss_layout &L) { return ipow(3, L.dim) * L.dim + 2 * L.dim; }
int n_out_of(const tpss_layout &L) { return L.dim * L.n * (L.n + 1) / 2; }

void check_learned_layout(const tpss_layout &L)
{
  TPSS_REQUIRE(L.patch_variant == TPSS_PATCH_VERTEX && L.ncp == 2,
               "the learned local solver is defined for vertex patches");
  TPSS_REQUIRE(!L.coords.empty(), "the learned local solver needs vertex_coords");
}

std::vector<float> features(const tpss_layout &L)
{
  const int dim = L.dim, nin = n_in_of(L), nv = ipow(3, dim);
  std::vector<float> X((size_t)L.P * nin, 0.f);
  for(int64_t p = 0; p < L.P; ++p)
  {
    const int lo[3] = {L.lower[p * 3], L.lower[p * 3 + 1], L.lower[p * 3 + 2]};
    double hbar[3] = {1.0, 1.0, 1.0};
    for(int d = 0; d < dim; ++d)
    {
      const auto &k = L.fd_keys[L.patch_fd_key[p * dim + d]];
      hbar[d] = 0.5 * (k.h0 + k.h1);
    }
    auto vid = [&](int x, int y, int z) {
      return x + (int64_t)(L.nc[0] + 1) * (y + (int64_t)(L.nc[1] + 1) * z);
    };
    const int c[3] = {lo[0] + 1, dim > 1 ? lo[1] + 1 : 0, dim > 2 ? lo[2] + 1 : 0};
    const int64_t cid = vid(c[0], c[1], c[2]);
    for(int v = 0; v < nv; ++v)
    {
      int off[3] = {0, 0, 0}, r = v;
      for(int d = 0; d < dim; ++d)
      {
        off[d] = r % 3 - 1;
        r /= 3;
      }
      const int64_t id = vid(c[0] + off[0], c[1] + off[1], c[2] + off[2]);
      for(int d = 0; d < dim; ++d)
        X[(size_t)p * nin + v * dim + d] =
          float((L.coords[id * dim + d] - L.coords[cid * dim + d]) / hbar[d] - off[d]);
    }
    for(int d = 0; d < dim; ++d)
    {
      const auto &k = L.fd_keys[L.patch_fd_key[p * dim + d]];
      X[(size_t)p * nin + nv * dim + 2 * d] = float(k.lo);
      X[(size_t)p * nin + nv * dim + 2 * d + 1] = float(k.hi);
    }
  }
  return X;
}

// surrogate 1-D problems of every patch direction (entry p * dim + d)
void surrogate_problems(const tpss_layout &L, Penalty ip, std::vector<double> &Mp, std::vector<double> &Ap)
{
  std::vector<double> Mk, Ak;
  key_matrices(L, ip, Mk, Ak);
  Mp = per_patch(L, Mk);
  Ap = per_patch(L, Ak);
}
}  // namespace

std::shared_ptr<FdTables> build_learned_tables(const tpss_layout &L, const tpss_precond_desc &d,
                                               const TableMaker &make)
{
  check_learned_layout(L);
  const tpss_mlp &m = *d.model;
  TPSS_REQUIRE(mlp_n_in(m) == n_in_of(L) && mlp_n_out(m) == n_out_of(L),
               "the model's input/output sizes do not match this layout");
  auto t0 = std::chrono::steady_clock::now();
  const int n = L.n, nn = n * n, dim = L.dim, nout = n_out_of(L);
  const std::vector<float> X = features(L);
  std::vector<float> Y((size_t)L.P * nout);
  {
    DeviceBuffer<float> dx, dy((size_t)L.P * nout);
    dx.upload(X.data(), X.size());
    mlp_infer(m, dx.ptr, L.P, dy.ptr, nullptr);
    TPSS_CUDA(cudaMemcpy(Y.data(), dy.ptr, sizeof(float) * Y.size(), cudaMemcpyDeviceToHost));
  }
  std::vector<double> Mp, Ap;
  surrogate_problems(L, make_penalty(d.ip_factor, d.penalty_mode, L.k), Mp, Ap);
  const std::vector<double> Asur = Ap;
  std::vector<double> H(nn), W(nn);
  int64_t fallbacks = 0;
  for(int64_t p = 0; p < L.P; ++p)
    for(int dd = 0; dd < dim; ++dd)
    {
      const size_t e = (size_t)p * dim + dd;
      double *A = &Ap[e * nn];
      // H = A + D^1/2 T D^1/2 (symmetric, from the upper triangle)
      const float *y = &Y[(size_t)p * nout + (size_t)dd * n * (n + 1) / 2];
      int u = 0;
      bool ok = true;
      for(int i = 0; i < n; ++i)
        for(int j = i; j < n; ++j, ++u)
        {
          const double v = A[i * n + j] + double(y[u]) * std::sqrt(A[i * n + i] * A[j * n + j]);
          H[i * n + j] = H[j * n + i] = v;
          ok = ok && std::isfinite(v);
        }
      // positive definiteness of H by Cholesky on a copy
      W = H;
      for(int j = 0; j < n && ok; ++j)
      {
        double t = W[j * n + j];
        for(int k = 0; k < j; ++k) t -= W[j * n + k] * W[j * n + k];
        if(!(t > 1e-6 * A[j * n + j]))
          ok = false;
        else
        {
          const double g = std::sqrt(t);
          W[j * n + j] = g;
          for(int i = j + 1; i < n; ++i)
          {
            double r = W[i * n + j];
            for(int k = 0; k < j; ++k) r -= W[i * n + k] * W[j * n + k];
            W[i * n + j] = r / g;
          }
        }
      }
      if(ok)
        std::copy(H.begin(), H.end(), A);
      else
        ++fallbacks;
    }
  fallbacks += keep_definite(L, Mp, Ap, Asur);
  auto T = make(&Mp, &Ap);
  T->learned_fallbacks = fallbacks;
  T->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return T;
}
}  // namespace tpss

using namespace tpss;

extern "C" int tpss_learned_sizes(const tpss_layout *L, int *n_in, int *n_out)
{
  return guarded([&] {
    TPSS_REQUIRE(L, "null layout");
    check_learned_layout(*L);
    if(n_in) *n_in = n_in_of(*L);
    if(n_out) *n_out = n_out_of(*L);
  });
}

extern "C" int tpss_learned_features(const tpss_layout *L, float *x_dev)
{
  return guarded([&] {
    TPSS_REQUIRE(L && x_dev, "null argument");
    check_learned_layout(*L);
    const std::vector<float> X = features(*L);
    TPSS_CUDA(cudaMemcpy(x_dev, X.data(), sizeof(float) * X.size(), cudaMemcpyHostToDevice));
  });
}

extern "C" int tpss_learned_targets(const tpss_layout *L, const tpss_operator *op, double ip_factor,
                                    float *y_dev)
{
  return guarded([&] {
    TPSS_REQUIRE(L && op && y_dev, "null argument");
    check_learned_layout(*L);
    check_exact_local(*L, op);
    const int n = L->n, nn = n * n, dim = L->dim, nout = n_out_of(*L);
    std::vector<double> Mp, Ap;
    surrogate_problems(*L, ip_factor, Mp, Ap);
    const std::vector<double> Af = ksum_fit(*L, *op, Mp);
    std::vector<float> Y((size_t)L->P * nout);
    for(int64_t p = 0; p < L->P; ++p)
      for(int dd = 0; dd < dim; ++dd)
      {
        const size_t e = (size_t)p * dim + dd;
        const double *A = &Ap[e * nn], *F = &Af[e * nn];
        float *y = &Y[(size_t)p * nout + (size_t)dd * n * (n + 1) / 2];
        int u = 0;
        for(int i = 0; i < n; ++i)
          for(int j = i; j < n; ++j, ++u)
            y[u] = float((F[i * n + j] - A[i * n + j]) / std::sqrt(A[i * n + i] * A[j * n + j]));
      }
    TPSS_CUDA(cudaMemcpy(y_dev, Y.data(), sizeof(float) * Y.size(), cudaMemcpyHostToDevice));
  });
}
