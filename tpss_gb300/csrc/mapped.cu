// SIPG level operator on multilinear (bi-/trilinear) meshes, as a block-sparse matrix.
//
// The reference applies its DG Laplace operator matrix-free with deal.II's MatrixFree on
// the mapped mesh (apps/laplace_integrator.h:578-743). On a distorted level the operator
// has no tensor-product structure, so here it is assembled once per level into a
// block-sparse matrix: for every cell one (k+1)^d x (k+1)^d block for itself and one for
// each face neighbour (2d+1 blocks per block row), FP64, assembled on the GPU by quadrature.
// With 280 GB of HBM a 32^3 DGQ3 level takes 7.5 GB, and the same blocks are the exact
// local matrices of the vertex patches (patch blocks are cell blocks of the level matrix).
//
// Bilinear form (laplace_integrator.h:613-743):
//   cell:      int grad u . grad v, Gauss rule with k+1 points per direction;
//   interior:  int sigma [u][v] - {d_n u}[v] - [u]{d_n v}, one normal n for both sides,
//              sigma = ip * gamma * (1/h_in + 1/h_out) / 2 (laplace_integrator.h:649-654);
//   Dirichlet: int sigma u v - d_n u v - u d_n v, sigma = 2 ip gamma / h (691-693, 707-726);
//   gamma = k(k+1) (common_integrator.h:30-37); h of a side = 1/|n . grad xi_normal| at the
//   face's first quadrature point, which is what `normal * inverse_jacobian(0)` evaluates.
// Block storage: block (row cell c, slot s) holds A(i, j) (i test, j trial) at j * nd + i,
// so that the threads of a block row read consecutive addresses in the product.
// Slots: 0 = the cell, 1 + 2d + side = face neighbour in direction d (side 0 lower, 1 upper).
#include "internal.h"
#include "mapped_tab.cuh"

namespace tpss
{
namespace
{
constexpr int kMaxNp = kMapMaxNp;

struct AsmArgs
{
  const double *coords;  // lexicographic vertices, dim coordinates each
  int nc[3];
  int np, nd, nb;
  double ip, ip_bd, gamma;  // interior / boundary ip factors
  double *vals;
  int32_t *col;
  double *fgeo;  // face geometry records (mapped_tab.cuh), n_cells * 2 dim of fg doubles, or null
  int fg;
};

template<int DIM>
__device__ void jacobian(const double *X, const double *xi, double J[DIM][DIM])
{
  for(int a = 0; a < DIM; ++a)
    for(int b = 0; b < DIM; ++b) J[a][b] = 0.0;
  for(int v = 0; v < (1 << DIM); ++v)
    for(int b = 0; b < DIM; ++b)
    {
      double t = 1.0;
      for(int e = 0; e < DIM; ++e)
      {
        const bool up = (v >> e) & 1;
        t *= e == b ? (up ? 1.0 : -1.0) : (up ? xi[e] : 1.0 - xi[e]);
      }
      for(int a = 0; a < DIM; ++a) J[a][b] += t * X[v * DIM + a];
    }
}

template<int DIM>
__device__ double invert(const double J[DIM][DIM], double Ji[DIM][DIM])
{
  if constexpr(DIM == 2)
  {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det;
    Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det;
    Ji[1][1] = J[0][0] / det;
    return det;
  }
  else
  {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    Ji[0][0] = c00 / det;
    Ji[1][0] = c01 / det;
    Ji[2][0] = c02 / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    return det;
  }
}

__device__ __forceinline__ int64_t vertex_id(const int *nc, int x, int y, int z)
{
  return x + (int64_t)(nc[0] + 1) * (y + (int64_t)(nc[1] + 1) * z);
}

template<int DIM>
__device__ void load_cell(const AsmArgs &a, const int *c, double *X)
{
  for(int v = threadIdx.x; v < (1 << DIM); v += blockDim.x)
  {
    int p[3] = {c[0], c[1], c[2]};
    for(int e = 0; e < DIM; ++e) p[e] += (v >> e) & 1;
    const int64_t id = vertex_id(a.nc, p[0], p[1], p[2]);
    for(int e = 0; e < DIM; ++e) X[v * DIM + e] = a.coords[id * DIM + e];
  }
}

// value and reference gradient of basis function i at a point given per direction by
// (kind, index): kind 0 = Gauss point index, 1 = face side
template<int DIM>
__device__ double basis(const MapTab &t, int np, int i, const int *kind, const int *pos,
                        double *g)
{
  double v1[DIM], d1[DIM];
  for(int d = 0; d < DIM; ++d)
  {
    const int id = i % np;
    i /= np;
    if(kind[d] == 0)
    {
      v1[d] = t.V[id * np + pos[d]];
      d1[d] = t.D[id * np + pos[d]];
    }
    else
    {
      v1[d] = t.F[pos[d] * np + id];
      d1[d] = t.G[pos[d] * np + id];
    }
  }
  double val = 1.0;
  for(int d = 0; d < DIM; ++d) val *= v1[d];
  for(int gd = 0; gd < DIM; ++gd)
  {
    double p = 1.0;
    for(int d = 0; d < DIM; ++d) p *= d == gd ? d1[d] : v1[d];
    g[gd] = p;
  }
  return val;
}

template<int DIM>
__global__ void __launch_bounds__(256) assemble_kernel(const AsmArgs a, const MapTab t)
{
  extern __shared__ double sm[];
  const int np = a.np, nd = a.nd, nb = a.nb;
  int nq = 1, nfq = 1;
  for(int d = 0; d < DIM; ++d) nq *= np;
  for(int d = 0; d < DIM - 1; ++d) nfq *= np;
  constexpr int NS = DIM * (DIM + 1) / 2;
  double *Xc = sm;                 // 8 * 3
  double *Xn = Xc + 24;            // 8 * 3
  double *Gm = Xn + 24;            // nq * NS metric
  double *wq = Gm + nq * NS;       // nfq
  double *cnc = wq + nfq;          // nfq * DIM: J_c^-1 n
  double *cnn = cnc + nfq * DIM;   // nfq * DIM: J_nb^-1 n
  double *hh = cnn + nfq * DIM;    // 2: h of the cell and of the neighbour
  double *phi = hh + 2;            // nfq * nd each
  double *dphi = phi + nfq * nd;
  double *psi = dphi + nfq * nd;
  double *dpsi = psi + nfq * nd;

  const int64_t cell = blockIdx.x;
  int c[3] = {0, 0, 0};
  {
    int64_t r = cell;
    for(int d = 0; d < DIM; ++d)
    {
      c[d] = int(r % a.nc[d]);
      r /= a.nc[d];
    }
  }
  load_cell<DIM>(a, c, Xc);
  __syncthreads();
  // metric w det(J) J^-1 J^-T at the cell quadrature points
  for(int q = threadIdx.x; q < nq; q += blockDim.x)
  {
    double xi[DIM], w = 1.0;
    int r = q;
    for(int d = 0; d < DIM; ++d)
    {
      xi[d] = t.qx[r % np];
      w *= t.qw[r % np];
      r /= np;
    }
    double J[DIM][DIM], Ji[DIM][DIM];
    jacobian<DIM>(Xc, xi, J);
    const double det = invert<DIM>(J, Ji);
    int s = 0;
    for(int a0 = 0; a0 < DIM; ++a0)
      for(int b0 = a0; b0 < DIM; ++b0)
      {
        double g = 0.0;
        for(int e = 0; e < DIM; ++e) g += Ji[a0][e] * Ji[b0][e];
        Gm[q * NS + s++] = w * fabs(det) * g;
      }
  }
  __syncthreads();
  const size_t bsz = (size_t)nd * nd;
  double *self = a.vals + (cell * nb) * bsz;
  for(int e = threadIdx.x; e < nd * nd; e += blockDim.x)
  {
    const int i = e % nd, j = e / nd;
    double acc = 0.0;
    for(int q = 0; q < nq; ++q)
    {
      int kind[DIM], pos[DIM], r = q;
      for(int d = 0; d < DIM; ++d)
      {
        kind[d] = 0;
        pos[d] = r % np;
        r /= np;
      }
      double gi[DIM], gj[DIM];
      basis<DIM>(t, np, i, kind, pos, gi);
      basis<DIM>(t, np, j, kind, pos, gj);
      const double *G = Gm + q * NS;
      double Gg[DIM];
      if constexpr(DIM == 2)
      {
        Gg[0] = G[0] * gj[0] + G[1] * gj[1];
        Gg[1] = G[1] * gj[0] + G[2] * gj[1];
      }
      else
      {
        Gg[0] = G[0] * gj[0] + G[1] * gj[1] + G[2] * gj[2];
        Gg[1] = G[1] * gj[0] + G[3] * gj[1] + G[4] * gj[2];
        Gg[2] = G[2] * gj[0] + G[4] * gj[1] + G[5] * gj[2];
      }
      for(int d = 0; d < DIM; ++d) acc += gi[d] * Gg[d];
    }
    self[e] = acc;
  }
  if(threadIdx.x == 0) a.col[cell * nb] = (int32_t)cell;
  __syncthreads();

  for(int d = 0; d < DIM; ++d)
    for(int side = 0; side < 2; ++side)
    {
      const int slot = 1 + 2 * d + side;
      int cn[3] = {c[0], c[1], c[2]};
      cn[d] += side ? 1 : -1;
      const bool boundary = cn[d] < 0 || cn[d] >= a.nc[d];
      const int64_t ncell = boundary ? -1 : cn[0] + (int64_t)a.nc[0] * (cn[1] + (int64_t)a.nc[1] * cn[2]);
      double *blk = a.vals + (cell * nb + slot) * bsz;
      if(!boundary) load_cell<DIM>(a, cn, Xn);
      __syncthreads();
      const double sgn = side ? 1.0 : -1.0;
      for(int q = threadIdx.x; q < nfq; q += blockDim.x)
      {
        double xi[DIM], w = 1.0;
        int r = q;
        for(int e = 0; e < DIM; ++e)
        {
          if(e == d)
            xi[e] = side;
          else
          {
            xi[e] = t.qx[r % np];
            w *= t.qw[r % np];
            r /= np;
          }
        }
        double J[DIM][DIM], Ji[DIM][DIM];
        jacobian<DIM>(Xc, xi, J);
        const double det = invert<DIM>(J, Ji);
        double ng = 0.0;
        for(int e = 0; e < DIM; ++e) ng += Ji[d][e] * Ji[d][e];
        ng = sqrt(ng);
        double n[DIM];
        for(int e = 0; e < DIM; ++e) n[e] = sgn * Ji[d][e] / ng;
        wq[q] = w * fabs(det) * ng;
        for(int e = 0; e < DIM; ++e)
        {
          double s = 0.0;
          for(int f = 0; f < DIM; ++f) s += Ji[e][f] * n[f];
          cnc[q * DIM + e] = s;
        }
        if(q == 0) hh[0] = 1.0 / ng;
        if(!boundary)
        {
          xi[d] = 1 - side;
          jacobian<DIM>(Xn, xi, J);
          invert<DIM>(J, Ji);
          double nn = 0.0;
          for(int e = 0; e < DIM; ++e)
          {
            double s = 0.0;
            for(int f = 0; f < DIM; ++f) s += Ji[e][f] * n[f];
            cnn[q * DIM + e] = s;
            nn += n[e] * Ji[d][e];
          }
          if(q == 0) hh[1] = 1.0 / fabs(nn);
        }
      }
      __syncthreads();
      for(int idx = threadIdx.x; idx < nfq * nd; idx += blockDim.x)
      {
        const int q = idx / nd, i = idx % nd;
        int kind[DIM], pos[DIM], r = q;
        for(int e = 0; e < DIM; ++e)
        {
          if(e == d)
          {
            kind[e] = 1;
            pos[e] = side;
          }
          else
          {
            kind[e] = 0;
            pos[e] = r % np;
            r /= np;
          }
        }
        double g[DIM];
        phi[idx] = basis<DIM>(t, np, i, kind, pos, g);
        double s = 0.0;
        for(int e = 0; e < DIM; ++e) s += g[e] * cnc[q * DIM + e];
        dphi[idx] = s;
        if(!boundary)
        {
          pos[d] = 1 - side;
          psi[idx] = basis<DIM>(t, np, i, kind, pos, g);
          s = 0.0;
          for(int e = 0; e < DIM; ++e) s += g[e] * cnn[q * DIM + e];
          dpsi[idx] = s;
        }
      }
      __syncthreads();
      const double sigma = boundary ? a.ip_bd * 2.0 * a.gamma / hh[0]
                                    : a.ip * a.gamma * (1.0 / hh[0] + 1.0 / hh[1]) * 0.5;
      const double beta = boundary ? 1.0 : 0.5;
      if(a.fgeo && !boundary)
      {
        double *rec = a.fgeo + ((size_t)cell * 2 * DIM + (2 * d + side)) * a.fg;
        for(int q = threadIdx.x; q < nfq; q += blockDim.x)
        {
          rec[q] = wq[q];
          for(int e = 0; e < DIM; ++e)
          {
            rec[nfq + q * DIM + e] = cnc[q * DIM + e];
            rec[nfq + nfq * DIM + q * DIM + e] = cnn[q * DIM + e];
          }
        }
        if(threadIdx.x == 0) rec[nfq * (1 + 2 * DIM)] = sigma;
      }
      for(int e = threadIdx.x; e < nd * nd; e += blockDim.x)
      {
        const int i = e % nd, j = e / nd;
        double s = 0.0, o = 0.0;
        for(int q = 0; q < nfq; ++q)
        {
          const double pi = phi[q * nd + i], dpi = dphi[q * nd + i];
          const double pj = phi[q * nd + j], dpj = dphi[q * nd + j];
          s += wq[q] * (sigma * pi * pj - beta * (pi * dpj + dpi * pj));
          if(!boundary)
          {
            const double qj = psi[q * nd + j], dqj = dpsi[q * nd + j];
            o += wq[q] * (-sigma * pi * qj - 0.5 * pi * dqj + 0.5 * dpi * qj);
          }
        }
        self[e] += s;
        blk[e] = o;
      }
      if(threadIdx.x == 0) a.col[cell * nb + slot] = (int32_t)ncell;
      __syncthreads();
    }
}

// T: value, source and accumulation type (float: the level operator of a single-precision
// V-cycle, on an FP32 copy of the blocks and of the source); the result is stored in FP64
template<typename T>
struct MvArgs
{
  const T *vals;
  const int32_t *col;
  const int64_t *cell_start;  // null: lexicographic blocks of nd
  const T *src;
  double *dst;
  const double *rhs;          // non-null: dst = rhs - A src
  int64_t n_rows;
  int nd, nb;
};

template<typename T>
__global__ void __launch_bounds__(256) bsr_vmult_kernel(const MvArgs<T> a)
{
  for(int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n_rows;
      r += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t cell = r / a.nd;
    const int i = int(r % a.nd);
    const size_t bsz = (size_t)a.nd * a.nd;
    T acc = T(0);
    for(int s = 0; s < a.nb; ++s)
    {
      const int32_t cc = a.col[cell * a.nb + s];
      if(cc < 0) continue;
      const T *x = a.src + (a.cell_start ? a.cell_start[cc] : (int64_t)cc * a.nd);
      const T *blk = a.vals + (cell * a.nb + s) * bsz + i;
      for(int j = 0; j < a.nd; ++j) acc += blk[(size_t)j * a.nd] * __ldg(x + j);
    }
    const int64_t g = (a.cell_start ? a.cell_start[cell] : cell * a.nd) + i;
    a.dst[g] = a.rhs ? a.rhs[g] - double(acc) : double(acc);
  }
}

__global__ void d2f_copy_kernel(int64_t n, const double *__restrict__ x, float *__restrict__ y)
{
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = float(x[i]);
}

}  // namespace

MapTab make_tab(int k)
{
  const Shape1D s = make_shape_1d(k);
  const int np = k + 1;
  MapTab t{};
  for(int q = 0; q < np; ++q)
  {
    t.qx[q] = s.qx[q];
    t.qw[q] = s.qw[q];
  }
  for(int i = 0; i < np; ++i)
  {
    for(int q = 0; q < np; ++q)
    {
      t.V[i * np + q] = s.val[i * np + q];
      t.D[i * np + q] = s.grad[i * np + q];
    }
    for(int side = 0; side < 2; ++side)
    {
      t.F[side * np + i] = s.fval[side][i];
      t.G[side * np + i] = s.fgrad[side][i];
    }
  }
  return t;
}

size_t mapped_smem_bytes(int dim, int np)
{
  const int nd = ipow(np, dim), nq = nd, nfq = ipow(np, dim - 1);
  const int ns = dim * (dim + 1) / 2;
  return sizeof(double) * (48 + (size_t)nq * ns + nfq + 2 * (size_t)nfq * dim + 2 + 4 * (size_t)nfq * nd);
}

void mapped_build(tpss_operator &op, const tpss_layout &L, Penalty ip)
{
  TPSS_REQUIRE(L.k + 1 <= kMaxNp, "mapped operator: degree must be at most 7");
  const size_t smem = mapped_smem_bytes(L.dim, L.np);
  TPSS_REQUIRE(smem <= 220 * 1024, "mapped operator: degree too high for this dimension");
  auto M = std::make_unique<MappedOperator>();
  M->nd = L.cell_dofs;
  M->nb = 2 * L.dim + 1;
  M->n_cells = L.n_cells;
  M->coords.upload(L.coords.data(), L.coords.size());
  M->vals.resize((size_t)L.n_cells * M->nb * M->nd * M->nd);
  M->col.resize((size_t)L.n_cells * M->nb);
  AsmArgs a;
  a.coords = M->coords.ptr;
  for(int d = 0; d < 3; ++d) a.nc[d] = L.nc[d];
  a.np = L.np;
  a.nd = M->nd;
  a.nb = M->nb;
  a.ip = ip.in;
  a.ip_bd = ip.bd;
  a.gamma = L.k == 0 ? 1.0 : L.k * (L.k + 1.0);
  a.vals = M->vals.ptr;
  a.col = M->col.ptr;
  // face geometry of the matrix-free face couplings (mapped_mf.cu)
  M->fg = face_geo_size(L.dim, ipow(L.np, L.dim - 1));
  M->fgeo.resize((size_t)L.n_cells * 2 * L.dim * M->fg);
  TPSS_CUDA(cudaMemset(M->fgeo.ptr, 0, sizeof(double) * M->fgeo.n));
  a.fgeo = M->fgeo.ptr;
  a.fg = M->fg;
  const MapTab t = make_tab(L.k);
  if(L.dim == 2)
  {
    TPSS_CUDA(cudaFuncSetAttribute(assemble_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    assemble_kernel<2><<<(unsigned)L.n_cells, 256, smem>>>(a, t);
  }
  else if(L.dim == 3)
  {
    TPSS_CUDA(cudaFuncSetAttribute(assemble_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    assemble_kernel<3><<<(unsigned)L.n_cells, 256, smem>>>(a, t);
  }
  else
    fail(TPSS_ERR_NOT_IMPLEMENTED, "mapped operator: dim must be 2 or 3");
  TPSS_CUDA(cudaGetLastError());
  TPSS_CUDA(cudaDeviceSynchronize());
  op.mapped = std::move(M);
}

namespace
{
template<typename T>
void launch_bsr(const tpss_operator &op, const T *vals, const T *src, double *dst, const double *rhs,
                cudaStream_t s)
{
  const tpss_layout &L = *op.layout;
  const MappedOperator &M = *op.mapped;
  MvArgs<T> a;
  a.vals = vals;
  a.col = M.col.ptr;
  a.cell_start = L.lexicographic ? nullptr : L.d_cell_start.ptr;
  a.src = src;
  a.dst = dst;
  a.rhs = rhs;
  a.n_rows = M.n_cells * M.nd;
  a.nd = M.nd;
  a.nb = M.nb;
  const int64_t blocks = (a.n_rows + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 16;
  bsr_vmult_kernel<T><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
}

int d2f_grid(int64_t n)
{
  const int64_t b = (n + 255) / 256, cap = (int64_t)num_sms() * 8;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}
}  // namespace

void mapped_apply(const tpss_operator &op, double *dst, const double *src, cudaStream_t s, const double *rhs)
{
  // the cell blocks plus matrix-free face couplings (2.4x fewer FP64 FLOPs than the seven
  // blocks); the block-sparse product where that path has no kernel
  if(mapped_apply_mf(op, dst, src, s, rhs)) return;
  launch_bsr<double>(op, op.mapped->vals.ptr, src, dst, rhs, s);
}

void mapped_apply_f32(tpss_operator &op, double *dst, const double *src, cudaStream_t s, const double *rhs)
{
  if(mapped_apply_mf_f32(op, dst, src, s, rhs)) return;
  MappedOperator &M = *op.mapped;
  if(M.vals32.n != M.vals.n)
  {
    // FP32 copy of the blocks, made on first use (half the bytes the FP64 blocks stream)
    M.vals32.resize(M.vals.n);
    d2f_copy_kernel<<<d2f_grid((int64_t)M.vals.n), 256, 0, s>>>((int64_t)M.vals.n, M.vals.ptr, M.vals32.ptr);
    TPSS_CUDA(cudaGetLastError());
  }
  const int64_t n = op.layout->n_dofs;
  if(op.x32.n < (size_t)n) op.x32.resize(n);
  d2f_copy_kernel<<<d2f_grid(n), 256, 0, s>>>(n, src, op.x32.ptr);
  TPSS_CUDA(cudaGetLastError());
  launch_bsr<float>(op, M.vals32.ptr, op.x32.ptr, dst, rhs, s);
}

std::vector<double> mapped_dense(const tpss_operator &op)
{
  const tpss_layout &L = *op.layout;
  const MappedOperator &M = *op.mapped;
  const int64_t N = L.n_dofs;
  const int nd = M.nd, nb = M.nb;
  std::vector<double> vals(M.vals.n);
  std::vector<int32_t> col(M.col.n);
  TPSS_CUDA(cudaMemcpy(vals.data(), M.vals.ptr, vals.size() * sizeof(double), cudaMemcpyDeviceToHost));
  TPSS_CUDA(cudaMemcpy(col.data(), M.col.ptr, col.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
  std::vector<double> A((size_t)N * N, 0.0);
  for(int64_t c = 0; c < M.n_cells; ++c)
    for(int s = 0; s < nb; ++s)
    {
      const int32_t cc = col[c * nb + s];
      if(cc < 0) continue;
      const int64_t r0 = L.cell_start[c], c0 = L.cell_start[cc];
      const double *blk = &vals[((size_t)c * nb + s) * nd * nd];
      for(int j = 0; j < nd; ++j)
        for(int i = 0; i < nd; ++i) A[(size_t)(r0 + i) * N + c0 + j] += blk[(size_t)j * nd + i];
    }
  return A;
}
}  // namespace tpss
