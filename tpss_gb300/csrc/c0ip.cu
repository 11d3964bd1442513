// C0 interior-penalty biharmonic problem (clamped, FE_Q(k), 2D Cartesian unit square):
// level operator, additive vertex-patch Schwarz smoother, transfer and CG + V-cycle.
//
// The reference builds the level matrix with MeshWorker (apps/biharmonic_integrator.h:69-350)
// and its local solvers from 1-D patch matrices (376-535). On a Cartesian mesh the form
//   sum_K int D^2u:D^2v + sum_F int -{d_nn v}[d_n u] - {d_nn u}[d_n v] + sigma [d_n u][d_n v]
// is separable: A = B (x) M + 2 L (x) L + M (x) B with the 1-D FE_Q mass M, stiffness L and the
// 1-D C0IP bilaplacian B (cell u''v'' plus the point terms), sigma = ip gamma (1/h_0 + 1/h_1)/2
// inside, 2 ip gamma / h on the boundary (Nitsche::compute_penalty_impl, gamma = k(k+1)).
// Nodes: FE_Q Lagrange basis on Gauss-Lobatto points; u = 0 on boundary nodes; vectors hold
// the (n k - 1)^2 interior nodes, x fastest.
//
// GB300 mapping: every 1-D matrix is banded (half bandwidth 2k; also on the host, so set-up
// memory grows linearly with the mesh), and the operator is two FP64 passes over the node grid
// (x then y). A vertex patch holds the (2k-1)^2 nodes
// strictly inside its 2 x 2 cells; patches of one color (vertex parity) are disjoint, so the
// smoother is one kernel per color: a CTA gathers a patch into shared memory, applies the
// local inverse and scatter-adds the damped result. Local solvers (the reference's
// LocalSolverVariant): exact -- dense inverse of the patch matrix (the patch matrix is the
// submatrix of A; basic state + InverseTable); bilaplacian -- fast diagonalization of
// B (x) M + M (x) B, the patch matrix without the mixed-derivative term.
#include <algorithm>
#include <cmath>
#include <map>

#include "internal.h"

namespace tpss
{
namespace
{
// ---- host: 1-D FE_Q data on the Gauss-Lobatto nodes ------------------------------------
struct Poly1D
{
  int k = 0;
  std::vector<double> nodes, qx, qw;
  // values, first and second derivatives of basis i at Gauss point q and at the ends 0 / 1
  std::vector<double> v, d1, d2;           // [i * (k+1) + q]
  std::vector<double> e1[2], e2[2], e0[2];  // [side][i]
};

// Lagrange basis on `nodes`: value, first and second derivative at x
void lagrange_123(const std::vector<double> &z, int i, double x, double &f, double &f1, double &f2)
{
  const int n = (int)z.size();
  f = 1.0;
  f1 = 0.0;
  f2 = 0.0;
  for(int a = 0; a < n; ++a)
  {
    if(a == i) continue;
    const double da = 1.0 / (z[i] - z[a]);
    // product rule on f = prod (x - z_a) da
    f2 = f2 * (x - z[a]) * da + 2.0 * f1 * da;
    f1 = f1 * (x - z[a]) * da + f * da;
    f *= (x - z[a]) * da;
  }
}

Poly1D make_poly(int k)
{
  const Shape1D s = make_shape_1d(k);
  Poly1D p;
  p.k = k;
  p.nodes = s.nodes;
  p.qx = s.qx;
  p.qw = s.qw;
  const int np = k + 1;
  p.v.resize(np * np);
  p.d1.resize(np * np);
  p.d2.resize(np * np);
  for(int side = 0; side < 2; ++side)
  {
    p.e0[side].resize(np);
    p.e1[side].resize(np);
    p.e2[side].resize(np);
  }
  for(int i = 0; i < np; ++i)
  {
    for(int q = 0; q < np; ++q)
      lagrange_123(p.nodes, i, p.qx[q], p.v[i * np + q], p.d1[i * np + q], p.d2[i * np + q]);
    for(int side = 0; side < 2; ++side)
      lagrange_123(p.nodes, i, double(side), p.e0[side][i], p.e1[side][i], p.e2[side][i]);
  }
  return p;
}

// banded 1-D matrix over all nodes: entry (i, j), |i - j| <= bw, at i (2 bw + 1) + j - i + bw
struct Band1D
{
  int n = 0, bw = 0;
  std::vector<double> v;
  void init(int n_, int bw_)
  {
    n = n_;
    bw = bw_;
    v.assign((size_t)n * (2 * bw + 1), 0.0);
  }
  double &at(int i, int j) { return v[(size_t)i * (2 * bw + 1) + (j - i + bw)]; }
  double get(int i, int j) const
  {
    return (j - i > bw || i - j > bw) ? 0.0 : v[(size_t)i * (2 * bw + 1) + (j - i + bw)];
  }
};

// 1-D matrices (M, L, B) on nc uniform cells, all nc k + 1 nodes, half bandwidth 2k
void global_1d(const Poly1D &p, int nc, double ip, Band1D &M, Band1D &L, Band1D &B)
{
  const int k = p.k, np = k + 1, n = nc * k + 1;
  const double h = 1.0 / nc, gamma = k == 0 ? 1.0 : k * (k + 1.0);
  M.init(n, 2 * k);
  L.init(n, 2 * k);
  B.init(n, 2 * k);
  for(int c = 0; c < nc; ++c)
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        double m = 0, l = 0, b = 0;
        for(int q = 0; q < np; ++q)
        {
          const double w = p.qw[q] * h;
          m += w * p.v[i * np + q] * p.v[j * np + q];
          l += w * p.d1[i * np + q] * p.d1[j * np + q] / (h * h);
          b += w * p.d2[i * np + q] * p.d2[j * np + q] / (h * h * h * h);
        }
        M.at(c * k + i, c * k + j) += m;
        L.at(c * k + i, c * k + j) += l;
        B.at(c * k + i, c * k + j) += b;
      }
  // interior nodes: cell c (0, its right end) and c + 1 (1, its left end), normal +1
  for(int c = 0; c + 1 < nc; ++c)
  {
    std::vector<int> idx(2 * np);
    std::vector<double> jump(2 * np), avg(2 * np);
    for(int i = 0; i < np; ++i)
    {
      idx[i] = c * k + i;
      idx[np + i] = (c + 1) * k + i;
      jump[i] = p.e1[1][i] / h;
      jump[np + i] = -p.e1[0][i] / h;
      avg[i] = 0.5 * p.e2[1][i] / (h * h);
      avg[np + i] = 0.5 * p.e2[0][i] / (h * h);
    }
    const double sig = ip * gamma * (2.0 / h) / 2.0;
    for(int a = 0; a < 2 * np; ++a)
      for(int b = 0; b < 2 * np; ++b)
        B.at(idx[a], idx[b]) += -avg[a] * jump[b] - jump[a] * avg[b] + sig * jump[a] * jump[b];
  }
  // boundary nodes, outward normal
  for(int e = 0; e < 2; ++e)
  {
    const int c = e == 0 ? 0 : nc - 1, side = e;
    const double nrm = e == 0 ? -1.0 : 1.0;
    const double sig = ip * 2.0 * gamma / h;
    for(int a = 0; a < np; ++a)
      for(int b = 0; b < np; ++b)
      {
        const double ja = nrm * p.e1[side][a] / h, jb = nrm * p.e1[side][b] / h;
        const double aa = p.e2[side][a] / (h * h), ab = p.e2[side][b] / (h * h);
        B.at(c * k + a, c * k + b) += -aa * jb - ja * ab + sig * ja * jb;
      }
  }
}

// interior-node rows of a 1-D matrix as a band of half width bw: [row][2 bw + 1]
std::vector<double> to_band(const Band1D &A, int n_all, int bw)
{
  const int n = n_all - 2, w = 2 * bw + 1;
  std::vector<double> out((size_t)n * w, 0.0);
  for(int i = 0; i < n; ++i)
    for(int o = -bw; o <= bw; ++o)
    {
      const int j = i + o;
      if(j < 0 || j >= n) continue;
      out[(size_t)i * w + o + bw] = A.get(i + 1, j + 1);
    }
  return out;
}

// interior submatrix [x0, x0 + m) of a 1-D matrix (interior-node numbering), dense
std::vector<double> sub_1d(const Band1D &A, int x0, int m)
{
  std::vector<double> out((size_t)m * m);
  for(int a = 0; a < m; ++a)
    for(int b = 0; b < m; ++b) out[(size_t)a * m + b] = A.get(x0 + a + 1, x0 + b + 1);
  return out;
}
}  // namespace
}  // namespace tpss

namespace tpss
{
namespace
{
// ---- device kernels ------------------------------------------------------------------------
// t_m = M_x u, t_l = L_x u, t_b = B_x u along the rows of the node grid (n x n, x fastest)
__global__ void __launch_bounds__(256) c0ip_x_kernel(const double *__restrict__ u, int n, int bw,
                                                     const double *__restrict__ M, const double *__restrict__ L,
                                                     const double *__restrict__ B, double *__restrict__ tm,
                                                     double *__restrict__ tl, double *__restrict__ tb)
{
  const int64_t total = (int64_t)n * n;
  const int w = 2 * bw + 1;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
  {
    const int x = int(t % n);
    const int64_t row = t - x;
    // M and L couple nodes of one cell (|offset| <= k = bw / 2), B across a node (<= 2k)
    double sm = 0, sl = 0, sb = 0;
    const int bh = bw / 2;
    for(int o = -bw; o <= bw; ++o)
    {
      const int j = x + o;
      if(j < 0 || j >= n) continue;
      const double v = u[row + j];
      const int at = x * w + o + bw;
      sb += B[at] * v;
      if(o >= -bh && o <= bh)
      {
        sm += M[at] * v;
        sl += L[at] * v;
      }
    }
    tm[t] = sm;
    tl[t] = sl;
    tb[t] = sb;
  }
}

// dst = M_y t_b + mixed L_y t_l + B_y t_m along the columns (mixed = 2 for the biharmonic
// form, 0 for the Laplacian, whose "B" is the stiffness matrix)
__global__ void __launch_bounds__(256) c0ip_y_kernel(const double *__restrict__ tm, const double *__restrict__ tl,
                                                     const double *__restrict__ tb, int n, int bw,
                                                     const double *__restrict__ M, const double *__restrict__ L,
                                                     const double *__restrict__ B, double mixed,
                                                     double *__restrict__ dst)
{
  const int64_t total = (int64_t)n * n;
  const int w = 2 * bw + 1;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
  {
    const int x = int(t % n), y = int(t / n);
    double s = 0;
    const int bh = bw / 2;
    for(int o = -bw; o <= bw; ++o)
    {
      const int j = y + o;
      if(j < 0 || j >= n) continue;
      const int64_t src = (int64_t)j * n + x;
      const int at = y * w + o + bw;
      s += B[at] * tm[src];
      if(o >= -bh && o <= bh) s += M[at] * tb[src] + mixed * L[at] * tl[src];
    }
    dst[t] = s;
  }
}

struct PatchArgs
{
  const double *src;
  double *dst;
  const int32_t *vertex;  // per patch of the color: (vx, vy)
  const int32_t *key;     // per patch: (key_x, key_y) for FD, (dense key, 0) for exact
  const void *tab;        // exact: [key][m2 x m2] transposed inverse; FD: [key1d][S m x m][lambda m]
  int n;                  // interior nodes per direction of the level
  int k, m;               // degree, 1-D patch size 2k - 1
  int64_t n_patches;
  double omega;
};

// one patch per warp (4 per CTA): gather (2k-1)^2 nodes into shared memory, apply the local
// inverse, scatter-add omega * result (patches of one color are disjoint)
template<typename T, bool DENSE>
__global__ void __launch_bounds__(128) c0ip_patch_kernel(const PatchArgs a)
{
  extern __shared__ unsigned char smraw[];
  const int m = a.m, m2 = m * m;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  T *r = reinterpret_cast<T *>(smraw) + (size_t)warp * 2 * m2;
  T *w = r + m2;
  const T *tab = reinterpret_cast<const T *>(a.tab);
  for(int64_t p = (int64_t)blockIdx.x * 4 + warp; p < a.n_patches; p += (int64_t)gridDim.x * 4)
  {
    const int x0 = (a.vertex[2 * p] - 1) * a.k, y0 = (a.vertex[2 * p + 1] - 1) * a.k;
    for(int l = lane; l < m2; l += 32) r[l] = T(a.src[(int64_t)(y0 + l / m) * a.n + x0 + l % m]);
    __syncwarp();
    if constexpr(DENSE)
    {
      const T *Ai = tab + (size_t)a.key[2 * p] * m2 * m2;
      for(int i = lane; i < m2; i += 32)
      {
        T acc = 0;
        for(int j = 0; j < m2; ++j) acc += Ai[(size_t)j * m2 + i] * r[j];
        w[i] = acc;
      }
    }
    else
    {
      // u = (Sy x Sx) diag(1 / (lx + ly)) (Sy x Sx)^T r; entry layout [S m x m][lambda m]
      const T *ex = tab + (size_t)a.key[2 * p] * (m * m + m), *ey = tab + (size_t)a.key[2 * p + 1] * (m * m + m);
      for(int l = lane; l < m2; l += 32)  // w = Sx^T along x
      {
        const int i = l % m, row = l - i;
        T s = 0;
        for(int j = 0; j < m; ++j) s += ex[j * m + i] * r[row + j];
        w[l] = s;
      }
      __syncwarp();
      for(int l = lane; l < m2; l += 32)  // r = Sy^T along y, / eigenvalue sums
      {
        const int i = l % m, b = l / m;
        T s = 0;
        for(int j = 0; j < m; ++j) s += ey[j * m + b] * w[j * m + i];
        r[l] = s / (ex[m * m + i] + ey[m * m + b]);
      }
      __syncwarp();
      for(int l = lane; l < m2; l += 32)  // w = Sx along x
      {
        const int i = l % m, row = l - i;
        T s = 0;
        for(int j = 0; j < m; ++j) s += ex[i * m + j] * r[row + j];
        w[l] = s;
      }
      __syncwarp();
      for(int l = lane; l < m2; l += 32)  // r = Sy along y
      {
        const int i = l % m, b = l / m;
        T s = 0;
        for(int j = 0; j < m; ++j) s += ey[b * m + j] * w[j * m + i];
        r[l] = s;
      }
      __syncwarp();
      for(int l = lane; l < m2; l += 32) w[l] = r[l];
    }
    __syncwarp();
    for(int l = lane; l < m2; l += 32) a.dst[(int64_t)(y0 + l / m) * a.n + x0 + l % m] += a.omega * double(w[l]);
    __syncwarp();
  }
}

// one direction of a sparse 1-D map applied to a 2-D grid: out[y][i] (+)= sum_e c_e in[y][col_e]
// (dir 0) or out[i][x] (+)= sum_e c_e in[col_e][x] (dir 1); rows of at most R entries
__global__ void __launch_bounds__(256) c0ip_map_kernel(const double *__restrict__ in, int n_in_x,
                                                       double *__restrict__ out, int n_out_x, int n_out_y,
                                                       const int32_t *__restrict__ col, const double *__restrict__ coef,
                                                       int R, int dir, int accumulate)
{
  const int64_t total = (int64_t)n_out_x * n_out_y;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
  {
    const int x = int(t % n_out_x), y = int(t / n_out_x);
    const int i = dir == 0 ? x : y;
    double s = 0;
    for(int e = 0; e < R; ++e)
    {
      const int c = col[i * R + e];
      if(c < 0) continue;
      s += coef[i * R + e] * (dir == 0 ? in[(int64_t)y * n_in_x + c] : in[(int64_t)c * n_in_x + x]);
    }
    out[t] = accumulate ? out[t] + s : s;
  }
}

unsigned grid_for_c(int64_t n)
{
  const int64_t b = (n + 255) / 256, cap = (int64_t)num_sms() * 8;
  return (unsigned)(b < 1 ? 1 : (b < cap ? b : cap));
}
}  // namespace
}  // namespace tpss

// ---- host objects ----------------------------------------------------------------------------
struct C0ipLevel
{
  int nc = 0, n = 0;  // cells per direction, interior nodes per direction (nc k - 1)
  tpss::DeviceBuffer<double> bandM, bandL, bandB;
  std::vector<int64_t> color_start;  // 5 entries
  tpss::DeviceBuffer<int32_t> vertex, key;
  tpss::DeviceBuffer<double> tab64;
  tpss::DeviceBuffer<float> tab32;
  // prolongation from the next coarser level (interior rows, at most pR entries) and its transpose
  int pR = 0, tR = 0;
  tpss::DeviceBuffer<int32_t> pcol, tcol;
  tpss::DeviceBuffer<double> pcoef, tcoef;
  tpss::DeviceBuffer<double> x, b, r, t, tm, tl, tb, tmp;
};

struct tpss_c0ip
{
  tpss_c0ip_desc desc{};
  int bw = 0, m = 0;
  double mixed = 2.0;  // weight of L (x) L: 2 (biharmonic), 0 (Laplacian)
  std::vector<C0ipLevel> lv;
  tpss::DeviceBuffer<double> coarse_inv, partial, scal, cr, cp, cAp, cz;
  // the CG preconditioner step (z = V-cycle(r)) as one CUDA graph, captured on a private stream
  // at the first solve and launched into the caller's stream order through two events
  cudaStream_t gstream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t g_pre = nullptr;
  tpss_c0ip() = default;
  tpss_c0ip(const tpss_c0ip &) = delete;
  ~tpss_c0ip()
  {
    if(g_pre) cudaGraphExecDestroy(g_pre);
    if(ev_in) cudaEventDestroy(ev_in);
    if(ev_out) cudaEventDestroy(ev_out);
    if(gstream) cudaStreamDestroy(gstream);
  }
};

namespace tpss
{
namespace
{
std::vector<double> cholesky_inv(const std::vector<double> &A, int N)
{
  std::vector<double> G(A);
  for(int j = 0; j < N; ++j)
  {
    double d = G[(size_t)j * N + j];
    for(int p = 0; p < j; ++p) d -= G[(size_t)j * N + p] * G[(size_t)j * N + p];
    if(!(d > 0.0)) fail(TPSS_ERR_INVALID_ARGUMENT, "C0IP matrix is not positive definite");
    const double g = std::sqrt(d);
    G[(size_t)j * N + j] = g;
    for(int i = j + 1; i < N; ++i)
    {
      double t = G[(size_t)i * N + j];
      for(int p = 0; p < j; ++p) t -= G[(size_t)i * N + p] * G[(size_t)j * N + p];
      G[(size_t)i * N + j] = t / g;
    }
  }
  std::vector<double> Gi((size_t)N * N, 0.0), Ai((size_t)N * N, 0.0);
  for(int c = 0; c < N; ++c)
    for(int i = c; i < N; ++i)
    {
      double t = i == c ? 1.0 : 0.0;
      for(int p = c; p < i; ++p) t -= G[(size_t)i * N + p] * Gi[(size_t)p * N + c];
      Gi[(size_t)i * N + c] = t / G[(size_t)i * N + i];
    }
  for(int i = 0; i < N; ++i)
    for(int j = 0; j <= i; ++j)
    {
      double t = 0.0;
      for(int p = i; p < N; ++p) t += Gi[(size_t)p * N + i] * Gi[(size_t)p * N + j];
      Ai[(size_t)i * N + j] = Ai[(size_t)j * N + i] = t;
    }
  return Ai;
}

// 1-D key of a patch position: bit 0 touches the lower boundary, bit 1 the upper one
int key_1d(int v, int nc) { return (v == 1 ? 1 : 0) | (v == nc - 1 ? 2 : 0); }

void build_level(tpss_c0ip &c, C0ipLevel &L, const Poly1D &poly, int nc)
{
  const tpss_c0ip_desc &d = c.desc;
  const int k = d.degree, m = c.m, na = nc * k + 1, bw = c.bw;
  L.nc = nc;
  L.n = nc * k - 1;
  Band1D M, Lm, B;
  global_1d(poly, nc, d.ip_factor, M, Lm, B);
  if(d.problem == TPSS_Q_POISSON) B = Lm;  // A = M (x) L + L (x) M
  L.bandM.upload(to_band(M, na, bw).data(), (size_t)L.n * (2 * bw + 1));
  L.bandL.upload(to_band(Lm, na, bw).data(), (size_t)L.n * (2 * bw + 1));
  L.bandB.upload(to_band(B, na, bw).data(), (size_t)L.n * (2 * bw + 1));
  // patches, colors (vx % 2) + 2 (vy % 2), lexicographic inside a color
  std::vector<int32_t> vert, key;
  L.color_start.assign(1, 0);
  for(int color = 0; color < 4; ++color)
  {
    for(int vy = 1; vy < nc; ++vy)
      for(int vx = 1; vx < nc; ++vx)
        if((vx % 2) + 2 * (vy % 2) == color)
        {
          vert.push_back(vx);
          vert.push_back(vy);
          const int kx = key_1d(vx, nc), ky = key_1d(vy, nc);
          if(d.local_solver == TPSS_LOCAL_EXACT)
          {
            key.push_back(kx + 4 * ky);
            key.push_back(0);
          }
          else
          {
            key.push_back(kx);
            key.push_back(ky);
          }
        }
    L.color_start.push_back((int64_t)vert.size() / 2);
  }
  if(!vert.empty())
  {
    L.vertex.upload(vert.data(), vert.size());
    L.key.upload(key.data(), key.size());
  }
  // local inverse tables for every 1-D key (a representative vertex per key)
  auto rep = [&](int kk) {
    for(int v = 1; v < nc; ++v)
      if(key_1d(v, nc) == kk) return v;
    return -1;
  };
  std::vector<double> tab;
  if(d.local_solver == TPSS_LOCAL_EXACT)
  {
    const int m2 = m * m;
    tab.assign((size_t)16 * m2 * m2, 0.0);
    for(int kx = 0; kx < 4; ++kx)
      for(int ky = 0; ky < 4; ++ky)
      {
        const int vx = rep(kx), vy = rep(ky);
        if(vx < 0 || vy < 0) continue;
        const auto Mx = sub_1d(M, (vx - 1) * k, m), Lx = sub_1d(Lm, (vx - 1) * k, m),
                   Bx = sub_1d(B, (vx - 1) * k, m);
        const auto My = sub_1d(M, (vy - 1) * k, m), Ly = sub_1d(Lm, (vy - 1) * k, m),
                   By = sub_1d(B, (vy - 1) * k, m);
        std::vector<double> K((size_t)m2 * m2);
        for(int b = 0; b < m; ++b)
          for(int a = 0; a < m; ++a)
            for(int b2 = 0; b2 < m; ++b2)
              for(int a2 = 0; a2 < m; ++a2)
                K[(size_t)(b * m + a) * m2 + b2 * m + a2] =
                  My[b * m + b2] * Bx[a * m + a2] + c.mixed * Ly[b * m + b2] * Lx[a * m + a2] +
                  By[b * m + b2] * Mx[a * m + a2];
        const auto Ki = cholesky_inv(K, m2);
        double *dst = &tab[(size_t)(kx + 4 * ky) * m2 * m2];
        for(int i = 0; i < m2; ++i)
          for(int j = 0; j < m2; ++j) dst[(size_t)j * m2 + i] = Ki[(size_t)i * m2 + j];
      }
  }
  else
  {
    std::vector<double> Ms((size_t)4 * m * m), As((size_t)4 * m * m), S, lam;
    for(int kk = 0; kk < 4; ++kk)
    {
      const int v = rep(kk) > 0 ? rep(kk) : 1;
      const auto Mk = sub_1d(M, (v - 1) * k, m), Bk = sub_1d(B, (v - 1) * k, m);
      std::copy(Mk.begin(), Mk.end(), &Ms[(size_t)kk * m * m]);
      std::copy(Bk.begin(), Bk.end(), &As[(size_t)kk * m * m]);
    }
    gen_eig_batched(m, 4, Ms, As, S, lam);
    tab.assign((size_t)4 * (m * m + m), 0.0);
    for(int kk = 0; kk < 4; ++kk)
    {
      std::copy_n(&S[(size_t)kk * m * m], m * m, &tab[(size_t)kk * (m * m + m)]);
      std::copy_n(&lam[(size_t)kk * m], m, &tab[(size_t)kk * (m * m + m) + m * m]);
    }
  }
  if(d.precision == TPSS_FP32)
  {
    std::vector<float> t32(tab.begin(), tab.end());
    L.tab32.upload(t32.data(), t32.size());
  }
  else
    L.tab64.upload(tab.data(), tab.size());
  const size_t N = (size_t)L.n * L.n;
  for(auto *buf : {&L.x, &L.b, &L.r, &L.t, &L.tm, &L.tl, &L.tb}) buf->resize(N);
}

// prolongation from nc to 2 nc cells (interior nodes), CSR rows of R entries, and its transpose
void build_transfer(tpss_c0ip &c, C0ipLevel &F, const Poly1D &poly, int ncc)
{
  const int k = c.desc.degree, nf = 2 * ncc * k - 1, nco = ncc * k - 1;
  const int R = k + 1;
  std::vector<int32_t> col((size_t)nf * R, -1);
  std::vector<double> coef((size_t)nf * R, 0.0);
  std::vector<std::vector<std::pair<int, double>>> tr(nco);
  for(int i = 0; i < nf; ++i)
  {
    const int g = i + 1;  // fine node
    int cf = g / k;
    if(cf > 2 * ncc - 1) cf = 2 * ncc - 1;
    const int cc = cf / 2, s = cf % 2, z = g - cf * k;
    for(int j = 0; j <= k; ++j)
    {
      const int gc = cc * k + j;  // coarse node
      if(gc == 0 || gc == ncc * k) continue;
      double f, f1, f2;
      lagrange_123(poly.nodes, j, (poly.nodes[z] + s) / 2.0, f, f1, f2);
      col[(size_t)i * R + j] = gc - 1;
      coef[(size_t)i * R + j] = f;
      tr[gc - 1].push_back({i, f});
    }
  }
  int tR = 1;
  for(auto &r : tr) tR = std::max<int>(tR, (int)r.size());
  std::vector<int32_t> tcol((size_t)nco * tR, -1);
  std::vector<double> tcoef((size_t)nco * tR, 0.0);
  for(int i = 0; i < nco; ++i)
    for(size_t e = 0; e < tr[i].size(); ++e)
    {
      tcol[(size_t)i * tR + e] = tr[i][e].first;
      tcoef[(size_t)i * tR + e] = tr[i][e].second;
    }
  F.pR = R;
  F.tR = tR;
  F.pcol.upload(col.data(), col.size());
  F.pcoef.upload(coef.data(), coef.size());
  F.tcol.upload(tcol.data(), tcol.size());
  F.tcoef.upload(tcoef.data(), tcoef.size());
  F.tmp.resize((size_t)nf * nf);
}

void op_apply(const tpss_c0ip &c, const C0ipLevel &L, double *dst, const double *src, cudaStream_t s)
{
  const int64_t N = (int64_t)L.n * L.n;
  c0ip_x_kernel<<<grid_for_c(N), 256, 0, s>>>(src, L.n, c.bw, L.bandM.ptr, L.bandL.ptr, L.bandB.ptr,
                                             L.tm.ptr, L.tl.ptr, L.tb.ptr);
  c0ip_y_kernel<<<grid_for_c(N), 256, 0, s>>>(L.tm.ptr, L.tl.ptr, L.tb.ptr, L.n, c.bw, L.bandM.ptr,
                                             L.bandL.ptr, L.bandB.ptr, c.mixed, dst);
  TPSS_CUDA(cudaGetLastError());
}

// dst = omega sum_j R_j^T A_j^-1 R_j src
void smooth(const tpss_c0ip &c, const C0ipLevel &L, double *dst, const double *src, cudaStream_t s)
{
  TPSS_CUDA(cudaMemsetAsync(dst, 0, sizeof(double) * (size_t)L.n * L.n, s));
  const bool dense = c.desc.local_solver == TPSS_LOCAL_EXACT;
  const bool f32 = c.desc.precision == TPSS_FP32;
  const int m2 = c.m * c.m;
  const size_t smem = (f32 ? sizeof(float) : sizeof(double)) * 2 * m2 * 4;  // 4 warps
  for(int color = 0; color < 4; ++color)
  {
    const int64_t b = L.color_start[color], e = L.color_start[color + 1];
    if(e <= b) continue;
    PatchArgs a;
    a.src = src;
    a.dst = dst;
    a.vertex = L.vertex.ptr + 2 * b;
    a.key = L.key.ptr + 2 * b;
    a.tab = f32 ? (const void *)L.tab32.ptr : (const void *)L.tab64.ptr;
    a.n = L.n;
    a.k = c.desc.degree;
    a.m = c.m;
    a.n_patches = e - b;
    a.omega = c.desc.relaxation;
    const unsigned grid = (unsigned)std::min<int64_t>((a.n_patches + 3) / 4, (int64_t)num_sms() * 16);
    if(dense && f32)
      c0ip_patch_kernel<float, true><<<grid, 128, smem, s>>>(a);
    else if(dense)
      c0ip_patch_kernel<double, true><<<grid, 128, smem, s>>>(a);
    else if(f32)
      c0ip_patch_kernel<float, false><<<grid, 128, smem, s>>>(a);
    else
      c0ip_patch_kernel<double, false><<<grid, 128, smem, s>>>(a);
    TPSS_CUDA(cudaGetLastError());
  }
}

// fine += P coarse (F is the fine level)
void prolongate_add(const C0ipLevel &F, const C0ipLevel &Cl, double *fine, const double *coarse, cudaStream_t s)
{
  const int nf = F.n, nco = Cl.n;
  c0ip_map_kernel<<<grid_for_c((int64_t)nf * nco), 256, 0, s>>>(coarse, nco, F.tmp.ptr, nf, nco, F.pcol.ptr,
                                                                F.pcoef.ptr, F.pR, 0, 0);
  c0ip_map_kernel<<<grid_for_c((int64_t)nf * nf), 256, 0, s>>>(F.tmp.ptr, nf, fine, nf, nf, F.pcol.ptr,
                                                               F.pcoef.ptr, F.pR, 1, 1);
  TPSS_CUDA(cudaGetLastError());
}

// coarse = P^T fine
void restrict_to(const C0ipLevel &F, const C0ipLevel &Cl, double *coarse, const double *fine, cudaStream_t s)
{
  const int nf = F.n, nco = Cl.n;
  c0ip_map_kernel<<<grid_for_c((int64_t)nco * nf), 256, 0, s>>>(fine, nf, F.tmp.ptr, nco, nf, F.tcol.ptr,
                                                                F.tcoef.ptr, F.tR, 0, 0);
  c0ip_map_kernel<<<grid_for_c((int64_t)nco * nco), 256, 0, s>>>(F.tmp.ptr, nco, coarse, nco, nco, F.tcol.ptr,
                                                                 F.tcoef.ptr, F.tR, 1, 0);
  TPSS_CUDA(cudaGetLastError());
}

// CG scalars on the device (no host round trip per iteration but the convergence check):
// sc[0] rz, sc[1] pAp, sc[2] rr, sc[3] rz_new, sc[4] alpha, sc[5] -alpha, sc[6] beta, sc[7] 1
__global__ void c0ip_cg_scalars(double *sc, int which)
{
  if(which == 0)
  {
    sc[4] = sc[0] / sc[1];
    sc[5] = -sc[4];
    sc[7] = 1.0;
  }
  else
  {
    sc[6] = sc[3] / sc[0];
    sc[0] = sc[3];
  }
}

// y = a x + b y with a, b in device memory (the arithmetic of vec_axpby)
__global__ void c0ip_axpby_dev(int64_t n, const double *__restrict__ pa, const double *__restrict__ x,
                               const double *__restrict__ pb, double *__restrict__ y)
{
  const double a = *pa, b = *pb;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

double dot(tpss_c0ip &c, int64_t n, const double *x, const double *y, cudaStream_t s)
{
  vec_dot(n, x, y, c.partial.ptr, c.scal.ptr, s);
  double h = 0.0;
  TPSS_CUDA(cudaMemcpyAsync(&h, c.scal.ptr, sizeof(double), cudaMemcpyDeviceToHost, s));
  TPSS_CUDA(cudaStreamSynchronize(s));
  return h;
}

// coarse solve x = A_0^-1 b with the dense inverse, one warp per row
__global__ void c0ip_dense_kernel(int n, const double *__restrict__ Ai, const double *__restrict__ b,
                                  double *__restrict__ x)
{
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
  if(row >= n) return;
  double s = 0.0;
  for(int j = lane; j < n; j += 32) s += Ai[(size_t)row * n + j] * b[j];
  for(int o = 16; o > 0; o /= 2) s += __shfl_down_sync(0xffffffffu, s, o);
  if(lane == 0) x[row] = s;
}

void dense_matvec_c(tpss_c0ip &c, C0ipLevel &L, cudaStream_t s)
{
  const int n = L.n * L.n;
  c0ip_dense_kernel<<<(n * 32 + 255) / 256, 256, 0, s>>>(n, c.coarse_inv.ptr, L.b.ptr, L.x.ptr);
  TPSS_CUDA(cudaGetLastError());
}

// x_l = V-cycle(b_l): pre-smoothing from zero, residual, restriction, recursion,
// prolongation, post-smoothing (the semantics of the DG multigrid)
void vcycle(tpss_c0ip &c, int l, cudaStream_t s)
{
  C0ipLevel &L = c.lv[l];
  const int64_t N = (int64_t)L.n * L.n;
  if(l == 0)
  {
    dense_matvec_c(c, L, s);
    return;
  }
  C0ipLevel &Cl = c.lv[l - 1];
  smooth(c, L, L.x.ptr, L.b.ptr, s);
  op_apply(c, L, L.t.ptr, L.x.ptr, s);
  vec_axpby(N, 1.0, L.b.ptr, -1.0, L.t.ptr, s);  // t = b - A x
  restrict_to(L, Cl, Cl.b.ptr, L.t.ptr, s);
  vcycle(c, l - 1, s);
  prolongate_add(L, Cl, L.x.ptr, Cl.x.ptr, s);
  op_apply(c, L, L.t.ptr, L.x.ptr, s);
  vec_axpby(N, 1.0, L.b.ptr, -1.0, L.t.ptr, s);
  smooth(c, L, L.r.ptr, L.t.ptr, s);
  vec_axpby(N, 1.0, L.r.ptr, 1.0, L.x.ptr, s);  // x += P (b - A x)
}
}  // namespace
}  // namespace tpss

using namespace tpss;

extern "C" int tpss_c0ip_create(const tpss_c0ip_desc *d, tpss_c0ip **out)
{
  return guarded([&] {
    TPSS_REQUIRE(d && out, "null argument");
    *out = nullptr;
    TPSS_REQUIRE(d->degree >= 2 && d->degree <= 7, "C0IP: degree must be in 2..7");
    TPSS_REQUIRE(d->n_rep >= 2 && d->n_cells_fine >= d->n_rep, "C0IP: n_rep >= 2 (interior vertices)");
    TPSS_REQUIRE(d->ip_factor > 0.0 && d->relaxation > 0.0, "C0IP: ip_factor and relaxation must be positive");
    TPSS_REQUIRE(d->local_solver == TPSS_LOCAL_EXACT || d->local_solver == TPSS_LOCAL_FD,
                 "C0IP: local_solver must be TPSS_LOCAL_EXACT or TPSS_LOCAL_FD (no mixed derivatives)");
    TPSS_REQUIRE(d->precision == TPSS_FP64 || d->precision == TPSS_FP32, "invalid precision");
    TPSS_REQUIRE(d->problem == TPSS_C0IP_BIHARMONIC || d->problem == TPSS_Q_POISSON, "invalid problem");
    int nl = 0;
    for(int nc = d->n_rep; nc <= d->n_cells_fine; nc *= 2) ++nl;
    TPSS_REQUIRE((d->n_rep << (nl - 1)) == d->n_cells_fine, "n_cells_fine must be n_rep * 2^L");
    auto c = std::make_unique<tpss_c0ip>();
    c->desc = *d;
    c->mixed = d->problem == TPSS_Q_POISSON ? 0.0 : 2.0;
    c->bw = 2 * d->degree;
    c->m = 2 * d->degree - 1;
    const Poly1D poly = make_poly(d->degree);
    c->lv.resize(nl);
    for(int l = 0; l < nl; ++l)
    {
      build_level(*c, c->lv[l], poly, d->n_rep << l);
      if(l > 0) build_transfer(*c, c->lv[l], poly, d->n_rep << (l - 1));
    }
    // dense coarse inverse
    {
      const int nc0 = d->n_rep, na = nc0 * d->degree + 1, n0 = nc0 * d->degree - 1, N0 = n0 * n0;
      TPSS_REQUIRE(N0 <= 4096, "C0IP: coarse level too large for the dense solve");
      Band1D M, Lm, B;
      global_1d(poly, nc0, d->ip_factor, M, Lm, B);
      if(d->problem == TPSS_Q_POISSON) B = Lm;
      std::vector<double> A((size_t)N0 * N0);
      for(int y = 0; y < n0; ++y)
        for(int x = 0; x < n0; ++x)
          for(int y2 = 0; y2 < n0; ++y2)
            for(int x2 = 0; x2 < n0; ++x2)
            {
              auto at = [&](const Band1D &X, int i, int j) { return X.get(i + 1, j + 1); };
              A[(size_t)(y * n0 + x) * N0 + y2 * n0 + x2] = at(M, y, y2) * at(B, x, x2) +
                                                            c->mixed * at(Lm, y, y2) * at(Lm, x, x2) +
                                                            at(B, y, y2) * at(M, x, x2);
            }
      const auto inv = cholesky_inv(A, N0);
      c->coarse_inv.upload(inv.data(), inv.size());
    }
    const int64_t nt = (int64_t)c->lv.back().n * c->lv.back().n;
    c->partial.resize(dot_partials());
    c->scal.resize(16);
    for(auto *b : {&c->cr, &c->cp, &c->cAp, &c->cz}) b->resize(nt);
    *out = c.release();
  });
}

extern "C" int tpss_c0ip_info(const tpss_c0ip *c, int level, int64_t *n_dofs, int *n_levels)
{
  return guarded([&] {
    TPSS_REQUIRE(c, "null argument");
    const int nl = (int)c->lv.size();
    if(n_levels) *n_levels = nl;
    if(n_dofs)
    {
      const int l = level < 0 ? nl - 1 : level;
      TPSS_REQUIRE(l < nl, "invalid level");
      *n_dofs = (int64_t)c->lv[l].n * c->lv[l].n;
    }
  });
}

extern "C" int tpss_c0ip_operator_vmult(tpss_c0ip *c, int level, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(c && dst && src && dst != src, "invalid argument");
    const int nl = (int)c->lv.size(), l = level < 0 ? nl - 1 : level;
    TPSS_REQUIRE(l < nl, "invalid level");
    op_apply(*c, c->lv[l], dst, src, as_stream(stream));
  });
}

extern "C" int tpss_c0ip_smoother_vmult(tpss_c0ip *c, int level, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(c && dst && src && dst != src, "invalid argument");
    const int nl = (int)c->lv.size(), l = level < 0 ? nl - 1 : level;
    TPSS_REQUIRE(l >= 1 && l < nl, "smoothers live on levels 1..L");
    smooth(*c, c->lv[l], dst, src, as_stream(stream));
  });
}

extern "C" int tpss_c0ip_cg_solve(tpss_c0ip *c, double *u, const double *f, double rel_tol, double abs_tol,
                                  int max_iter, int *iterations, double *res_history, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(c && u && f && max_iter >= 0, "invalid argument");
    cudaStream_t s = as_stream(stream);
    C0ipLevel &T = c->lv.back();
    const int top = (int)c->lv.size() - 1;
    const int64_t N = (int64_t)T.n * T.n;
    TPSS_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * N, s));
    TPSS_CUDA(cudaMemcpyAsync(c->cr.ptr, f, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
    double res = std::sqrt(dot(*c, N, c->cr.ptr, c->cr.ptr, s));
    if(res_history) res_history[0] = res;
    const double tol = std::max(abs_tol, rel_tol * res);
    int it = 0;
    bool converged = res <= tol;
    if(!converged)
    {
      auto precondition_on = [&](cudaStream_t st) {
        TPSS_CUDA(cudaMemcpyAsync(T.b.ptr, c->cr.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        vcycle(*c, top, st);
        TPSS_CUDA(cudaMemcpyAsync(c->cz.ptr, T.x.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
      };
      auto precondition = [&]() {
        if(!c->g_pre)
        {
          precondition_on(s);  // eager first application (lazy scratch allocations happen here)
          TPSS_CUDA(cudaStreamSynchronize(s));
          if(!c->gstream)
          {
            TPSS_CUDA(cudaStreamCreateWithFlags(&c->gstream, cudaStreamNonBlocking));
            TPSS_CUDA(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming));
            TPSS_CUDA(cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming));
          }
          cudaGraph_t g = nullptr;
          TPSS_CUDA(cudaStreamBeginCapture(c->gstream, cudaStreamCaptureModeThreadLocal));
          try
          {
            precondition_on(c->gstream);
          }
          catch(...)
          {
            cudaStreamEndCapture(c->gstream, &g);
            if(g) cudaGraphDestroy(g);
            throw;
          }
          TPSS_CUDA(cudaStreamEndCapture(c->gstream, &g));
          const cudaError_t e = cudaGraphInstantiate(&c->g_pre, g, 0);
          cudaGraphDestroy(g);
          TPSS_CUDA(e);
          return;
        }
        TPSS_CUDA(cudaEventRecord(c->ev_in, s));
        TPSS_CUDA(cudaStreamWaitEvent(c->gstream, c->ev_in, 0));
        TPSS_CUDA(cudaGraphLaunch(c->g_pre, c->gstream));
        TPSS_CUDA(cudaEventRecord(c->ev_out, c->gstream));
        TPSS_CUDA(cudaStreamWaitEvent(s, c->ev_out, 0));
      };
      precondition();
      TPSS_CUDA(cudaMemcpyAsync(c->cp.ptr, c->cz.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
      double *sc = c->scal.ptr + 8;
      vec_dot(N, c->cr.ptr, c->cz.ptr, c->partial.ptr, sc + 0, s);  // rz
      const unsigned vg = (unsigned)std::min<int64_t>((N + 255) / 256, (int64_t)num_sms() * 8);
      for(it = 1; it <= max_iter; ++it)
      {
        op_apply(*c, T, c->cAp.ptr, c->cp.ptr, s);
        vec_dot(N, c->cp.ptr, c->cAp.ptr, c->partial.ptr, sc + 1, s);  // pAp
        c0ip_cg_scalars<<<1, 1, 0, s>>>(sc, 0);                          // alpha = rz / pAp
        c0ip_axpby_dev<<<vg, 256, 0, s>>>(N, sc + 4, c->cp.ptr, sc + 7, u);
        c0ip_axpby_dev<<<vg, 256, 0, s>>>(N, sc + 5, c->cAp.ptr, sc + 7, c->cr.ptr);
        TPSS_CUDA(cudaGetLastError());
        res = std::sqrt(dot(*c, N, c->cr.ptr, c->cr.ptr, s));  // the one host round trip
        if(res_history) res_history[it] = res;
        if(res <= tol)
        {
          converged = true;
          break;
        }
        precondition();
        vec_dot(N, c->cr.ptr, c->cz.ptr, c->partial.ptr, sc + 3, s);  // rz_new
        c0ip_cg_scalars<<<1, 1, 0, s>>>(sc, 1);                         // beta, rz = rz_new
        c0ip_axpby_dev<<<vg, 256, 0, s>>>(N, sc + 7, c->cz.ptr, sc + 6, c->cp.ptr);  // p = z + beta p
        TPSS_CUDA(cudaGetLastError());
      }
    }
    if(iterations) *iterations = converged ? it : max_iter;
    if(!converged) fail(TPSS_ERR_NOT_CONVERGED, "C0IP CG did not converge");
  });
}

extern "C" void tpss_c0ip_destroy(tpss_c0ip *c) { delete c; }
