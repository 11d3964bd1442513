// setup.cu -- host-side 1-D finite element data of the smoother and the operator (FP64).
//
// FE_DGQ(k): Lagrange polynomials on the k+1 Gauss-Lobatto points, integrated with the
// (k+1)-point Gauss rule, as deal.II's ShapeInfo provides them to FDEvaluation
// (TPSS/fd_evaluation.h:33-446).  The 1-D patch matrices follow
// FDEvaluation::patch_action (TPSS/fd_evaluation.templates.h:168-281) with the SIPG terms of
// apps/common_integrator.h:159-293 and the average factor of TPSS/fd_evaluation.h:651-688.
#include <cmath>
#include <cstring>

#include "internal.h"

namespace tpss
{
namespace
{
// Legendre P_m(x) and P_m'(x) on [-1,1] by the three-term recurrence.
void legendre(int m, double x, double &p, double &dp)
{
  double pm1 = 1.0, pcur = x;
  if(m == 0)
  {
    p = 1.0;
    dp = 0.0;
    return;
  }
  for(int j = 2; j <= m; ++j)
  {
    const double pn = ((2 * j - 1) * x * pcur - (j - 1) * pm1) / j;
    pm1 = pcur;
    pcur = pn;
  }
  p = pcur;
  dp = m * (x * pcur - pm1) / (x * x - 1.0);
}

void gauss_rule(int n, std::vector<double> &x, std::vector<double> &w)
{
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for(int i = 0; i < n; ++i)
  {
    // i-th root counted from the left end
    double z = -std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double p = 0, dp = 1;
    for(int it = 0; it < 100; ++it)
    {
      legendre(n, z, p, dp);
      const double step = p / dp;
      z -= step;
      if(std::fabs(step) < 1e-17) break;
    }
    legendre(n, z, p, dp);
    x[i] = 0.5 * (1.0 + z);
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

std::vector<double> lobatto_nodes(int n)
{
  std::vector<double> x(n);
  if(n == 1)
  {
    x[0] = 0.5;
    return x;
  }
  const int m = n - 1;
  x[0] = 0.0;
  x[m] = 1.0;
  for(int i = 1; i < m; ++i)
  {
    double z = -std::cos(M_PI * i / m);
    for(int it = 0; it < 200; ++it)
    {
      double p, dp;
      legendre(m, z, p, dp);
      const double ddp = (2.0 * z * dp - m * (m + 1.0) * p) / (1.0 - z * z);
      const double step = dp / ddp;
      z -= step;
      if(std::fabs(step) < 1e-17) break;
    }
    x[i] = 0.5 * (1.0 + z);
  }
  return x;
}

// values and first derivatives of the Lagrange basis on `z` at `x`
void lagrange_eval(const std::vector<double> &z, double x, double *v, double *d)
{
  const int n = (int)z.size();
  for(int i = 0; i < n; ++i)
  {
    double prod = 1.0, deriv = 0.0;
    for(int j = 0; j < n; ++j)
    {
      if(j == i) continue;
      const double f = (x - z[j]) / (z[i] - z[j]);
      deriv = deriv * f + prod / (z[i] - z[j]);  // product rule, accumulated left to right
      prod *= f;
    }
    v[i] = prod;
    d[i] = n == 1 ? 0.0 : deriv;
  }
}
}  // namespace

Shape1D make_shape_1d(int k)
{
  Shape1D s;
  s.k = k;
  s.np = k + 1;
  gauss_rule(k + 1, s.qx, s.qw);
  s.nodes = lobatto_nodes(k + 1);
  s.val.assign(s.np * s.np, 0.0);
  s.grad.assign(s.np * s.np, 0.0);
  std::vector<double> v(s.np), d(s.np);
  for(int q = 0; q < s.np; ++q)
  {
    lagrange_eval(s.nodes, s.qx[q], v.data(), d.data());
    for(int i = 0; i < s.np; ++i)
    {
      s.val[i * s.np + q] = v[i];
      s.grad[i * s.np + q] = d[i];
    }
  }
  for(int f = 0; f < 2; ++f)
  {
    s.fval[f].assign(s.np, 0.0);
    s.fgrad[f].assign(s.np, 0.0);
    lagrange_eval(s.nodes, double(f), s.fval[f].data(), s.fgrad[f].data());
  }
  return s;
}

Penalty make_penalty(double ip, int mode, int k)
{
  if(mode == TPSS_PENALTY_REFERENCE) return Penalty(ip);
  TPSS_REQUIRE(mode == TPSS_PENALTY_2KP1SQ, "unknown penalty_mode");
  // interior: in * gamma = 2 (k+1)^2; boundary: 2 bd gamma = 2 (k+1)^2
  const double gamma = k == 0 ? 1.0 : double(k) * (k + 1), kp = k + 1.0;
  return Penalty(ip * 2.0 * kp * kp / gamma, ip * kp * kp / gamma);
}

void patch_matrices_1d(const Shape1D &s, int ncp, const double *h, bool bdry_lo, bool bdry_hi,
                       Penalty ip, double *M, double *A)
{
  const int np = s.np, n = ncp * np;
  const double gamma = s.k == 0 ? 1.0 : double(s.k) * (s.k + 1);
  std::memset(M, 0, sizeof(double) * n * n);
  std::memset(A, 0, sizeof(double) * n * n);
  auto at = [n](double *X, int r, int c) -> double & { return X[r * n + c]; };
  for(int c = 0; c < ncp; ++c)
  {
    const double hc = h[c];
    const int off = c * np;
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        double m = 0.0, l = 0.0;
        for(int q = 0; q < np; ++q)
        {
          m += s.val[i * np + q] * s.val[j * np + q] * s.qw[q];
          l += s.grad[i * np + q] * s.grad[j * np + q] * s.qw[q];
        }
        at(M, off + i, off + j) += m * hc;
        at(A, off + i, off + j) += l / hc;
      }
    // the two faces of cell c (the patch interface gets average factor 1/2)
    for(int f = 0; f < 2; ++f)
    {
      const double nu = f == 0 ? -1.0 : 1.0;
      const bool interface = ncp == 2 && ((c == 0 && f == 1) || (c == 1 && f == 0));
      const bool physical = !interface && (f == 0 ? bdry_lo : bdry_hi);
      const double avg = physical ? 1.0 : 0.5;
      const double penalty = (physical ? ip.bd : ip.in) * avg * 2.0 * gamma / hc;
      for(int i = 0; i < np; ++i)
        for(int j = 0; j < np; ++j)
        {
          const double v = s.fval[f][i], dv = s.fgrad[f][i] / hc;
          const double u = s.fval[f][j], du = s.fgrad[f][j] / hc;
          at(A, off + i, off + j) += -avg * nu * (v * du + dv * u) + penalty * v * u;
        }
    }
  }
  if(ncp == 2)
  {
    const double h0 = h[0], h1 = h[1];
    const double penalty = ip.in * gamma * (0.5 / h0 + 0.5 / h1);  // ip * 0.5 * 2 gamma (...)
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        // cell 0 sees the interface as face 1 (normal +1), cell 1 as face 0 (normal -1)
        const double v0 = s.fval[1][i], dv0 = s.fgrad[1][i] / h0;
        const double u1 = s.fval[0][j], du1 = s.fgrad[0][j] / h1;
        const double v1 = s.fval[0][i], dv1 = s.fgrad[0][i] / h1;
        const double u0 = s.fval[1][j], du0 = s.fgrad[1][j] / h0;
        at(A, i, np + j) += -0.5 * (v0 * du1 - dv0 * u1) - penalty * v0 * u1;
        at(A, np + i, j) += -0.5 * (-v1 * du0 + dv1 * u0) - penalty * v1 * u0;
      }
  }
}

void operator_blocks_1d(const Shape1D &s, int nc, const double *h, Penalty ip,
                        std::vector<double> &mass, std::vector<double> &blk)
{
  const int np = s.np, q2 = np * np;
  const double gamma = s.k == 0 ? 1.0 : double(s.k) * (s.k + 1);
  mass.assign((size_t)nc * q2, 0.0);
  blk.assign((size_t)nc * 3 * q2, 0.0);
  for(int c = 0; c < nc; ++c)
  {
    const double hc = h[c];
    double *C = &blk[((size_t)c * 3 + 1) * q2];
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        double m = 0.0, l = 0.0;
        for(int q = 0; q < np; ++q)
        {
          m += s.val[i * np + q] * s.val[j * np + q] * s.qw[q];
          l += s.grad[i * np + q] * s.grad[j * np + q] * s.qw[q];
        }
        mass[(size_t)c * q2 + i * np + j] = m * hc;
        C[i * np + j] += l / hc;
      }
    // Dirichlet boundary faces: sigma = 2 ip gamma / h, outward normal derivative
    for(int f = 0; f < 2; ++f)
    {
      if((f == 0 && c != 0) || (f == 1 && c != nc - 1)) continue;
      const double nu = f == 0 ? -1.0 : 1.0, sigma = ip.bd * 2.0 * gamma / hc;
      for(int i = 0; i < np; ++i)
        for(int j = 0; j < np; ++j)
        {
          const double v = s.fval[f][i], dv = nu * s.fgrad[f][i] / hc;
          const double u = s.fval[f][j], du = nu * s.fgrad[f][j] / hc;
          C[i * np + j] += sigma * u * v - du * v - u * dv;
        }
    }
  }
  for(int c = 0; c + 1 < nc; ++c)
  {
    const double hl = h[c], hr = h[c + 1];
    const double sigma = ip.in * 0.5 * gamma * (1.0 / hl + 1.0 / hr);
    double *LL = &blk[((size_t)c * 3 + 1) * q2], *LR = &blk[((size_t)c * 3 + 2) * q2];
    double *RL = &blk[((size_t)(c + 1) * 3 + 0) * q2], *RR = &blk[((size_t)(c + 1) * 3 + 1) * q2];
    for(int i = 0; i < np; ++i)
      for(int j = 0; j < np; ++j)
      {
        // trial j, test i: sigma [u][v] - {u'}[v] - [u]{v'}, [w] = w_l(1) - w_r(0)
        const double ul = s.fval[1][j], dul = s.fgrad[1][j] / hl;
        const double ur = s.fval[0][j], dur = s.fgrad[0][j] / hr;
        const double vl = s.fval[1][i], dvl = s.fgrad[1][i] / hl;
        const double vr = s.fval[0][i], dvr = s.fgrad[0][i] / hr;
        LL[i * np + j] += sigma * ul * vl - 0.5 * dul * vl - 0.5 * ul * dvl;
        LR[i * np + j] += -sigma * ur * vl - 0.5 * dur * vl + 0.5 * ur * dvl;
        RL[i * np + j] += -sigma * ul * vr + 0.5 * dul * vr - 0.5 * ul * dvr;
        RR[i * np + j] += sigma * ur * vr + 0.5 * dur * vr + 0.5 * ur * dvr;
      }
  }
}

std::vector<double> embedding_1d(const Shape1D &s)
{
  const int np = s.np;
  std::vector<double> E(2 * np * np), v(np), d(np);
  for(int ch = 0; ch < 2; ++ch)
    for(int i = 0; i < np; ++i)
    {
      lagrange_eval(s.nodes, 0.5 * (s.nodes[i] + ch), v.data(), d.data());
      for(int j = 0; j < np; ++j) E[ch * np * np + i * np + j] = v[j];
    }
  return E;
}

}  // namespace tpss

namespace tpss
{
// Per cell of one direction: [M np*np][C np*np][aL 2*np][bL 2*np][aR 2*np][bR 2*np].
// C is the cell's own block of the global 1-D SIPG matrix; the couplings to the neighbours are
// rank two (only face values and normal derivatives meet):
//   block(c, c+1) = aR_0 bR_0^T + aR_1 bR_1^T,  block(c, c-1) = aL_0 bL_0^T + aL_1 bL_1^T
// (zero at the physical boundary), from the interior-face terms
// sigma [u][v] - {u'}[v] - [u]{v'} with sigma = ip gamma (1/h_l + 1/h_r)/2.
std::vector<double> operator_factors_1d(const Shape1D &s, int nc, const double *h, Penalty ip)
{
  const int np = s.np, q2 = np * np, stride = 2 * q2 + 8 * np;
  const double gamma = s.k == 0 ? 1.0 : double(s.k) * (s.k + 1);
  std::vector<double> mass, blk;
  operator_blocks_1d(s, nc, h, ip, mass, blk);
  std::vector<double> out((size_t)nc * stride, 0.0);
  for(int c = 0; c < nc; ++c)
  {
    double *o = &out[(size_t)c * stride];
    for(int i = 0; i < q2; ++i)
    {
      o[i] = mass[(size_t)c * q2 + i];
      o[q2 + i] = blk[((size_t)c * 3 + 1) * q2 + i];
    }
    double *aL = o + 2 * q2, *bL = aL + 2 * np, *aR = bL + 2 * np, *bR = aR + 2 * np;
    if(c > 0)
    {
      const double hl = h[c - 1], hc = h[c];
      const double sigma = ip.in * 0.5 * gamma * (1.0 / hl + 1.0 / hc);
      for(int i = 0; i < np; ++i)
      {
        aL[i] = s.fval[0][i];                // test value at the cell's left face
        aL[np + i] = s.fgrad[0][i] / hc;     // test derivative there
        bL[i] = -sigma * s.fval[1][i] + 0.5 * s.fgrad[1][i] / hl;  // trial side of cell c-1
        bL[np + i] = -0.5 * s.fval[1][i];
      }
    }
    if(c + 1 < nc)
    {
      const double hc = h[c], hr = h[c + 1];
      const double sigma = ip.in * 0.5 * gamma * (1.0 / hc + 1.0 / hr);
      for(int i = 0; i < np; ++i)
      {
        aR[i] = s.fval[1][i];
        aR[np + i] = s.fgrad[1][i] / hc;
        bR[i] = -sigma * s.fval[0][i] - 0.5 * s.fgrad[0][i] / hr;
        bR[np + i] = 0.5 * s.fval[0][i];
      }
    }
  }
  return out;
}
}  // namespace tpss
