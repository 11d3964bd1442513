// layout.cu -- patch layout of a structured level (the SubdomainHandler of this library).
//
// Vertex patches are the 2^dim cells around every interior vertex, cells in lexicographic
// order (TPSS/patch_info.templates.h:176-409, collection[2^dim-1-v] at 389-402); cell patches
// are single cells (patch_info.templates.h:59-173).  Colors: the tiled coloring of
// apps/coloring.h:347-401 for vertex patches (color bit d set when the patch's vertex index
// in direction d is even), one color for additive cell patches (patch_info.templates.h:96-102)
// and red-black for multiplicative cell patches; within a color interior patches come before
// boundary patches (patch_info.templates.h:605-680).  A user coloring may replace the default;
// it is checked to be conflict-free (no cell twice within a color), the contract the reference
// leaves to the user for additive TBB loops (patch_info.templates.h:461-470).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "internal.h"

namespace tpss
{
namespace
{
thread_local std::string g_last_error;
}

void set_last_error(const std::string &msg) { g_last_error = msg; }
const char *last_error_cstr() { return g_last_error.c_str(); }

// SM count of the current device (queried once per device)
int num_sms()
{
  static std::mutex mu;
  static int sms[64] = {0};
  int dev = 0;
  if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if(sms[dev] == 0)
  {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms[dev] = n > 0 ? n : 1;
  }
  return sms[dev];
}

namespace
{
struct PatchRec
{
  int32_t lo[3];
  int32_t color;
  bool boundary;
  int64_t lex;  // default lexicographic anchor order
};

// ---- surrogate widths of vertex patches on distorted meshes
// Gauss-Lobatto points and weights on [0,1] (endpoints plus roots of P'_{n-1}).
void lobatto_rule(int n, std::vector<double> &z, std::vector<double> &w)
{
  z.assign(n, 0.0);
  w.assign(n, 0.0);
  const int m = n - 1;
  for(int i = 0; i < n; ++i)
  {
    double x = -std::cos(M_PI * i / m);
    auto leg = [m](double t, double &p, double &dp) {
      double p0 = 1.0, p1 = t;
      for(int j = 2; j <= m; ++j)
      {
        const double p2 = ((2 * j - 1) * t * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      p = m == 0 ? 1.0 : p1;
      dp = m * (t * p1 - p0) / (t * t - 1.0);
    };
    double p = 0, dp = 0;
    if(i > 0 && i < m)
      for(int it = 0; it < 200; ++it)
      {
        leg(x, p, dp);
        const double ddp = (2.0 * x * dp - m * (m + 1.0) * p) / (1.0 - x * x);
        const double step = dp / ddp;
        x -= step;
        if(std::fabs(step) < 1e-17) break;
      }
    if(i == 0 || i == m)
      p = (i == 0 && (m % 2)) ? -1.0 : 1.0;
    else
      leg(x, p, dp);
    z[i] = 0.5 * (x + 1.0);
    w[i] = 1.0 / (n * (n - 1.0) * p * p);
  }
}

// arc length in each direction of the trilinear cell with corner coordinates X[2^dim][dim]
void cell_arc_lengths(int dim, const double *X, const std::vector<double> &z,
                      const std::vector<double> &w, double *h)
{
  const int nq = (int)z.size();
  auto map = [&](const double *xi, double *x) {
    for(int c = 0; c < dim; ++c) x[c] = 0.0;
    for(int v = 0; v < (1 << dim); ++v)
    {
      double wt = 1.0;
      for(int e = 0; e < dim; ++e) wt *= ((v >> e) & 1) ? xi[e] : 1.0 - xi[e];
      for(int c = 0; c < dim; ++c) x[c] += wt * X[v * dim + c];
    }
  };
  for(int d = 0; d < dim; ++d)
  {
    double acc = 0.0;
    const int nf = dim == 2 ? nq : nq * nq;
    for(int f = 0; f < nf; ++f)
    {
      const int fi[2] = {f % nq, f / nq};
      double wf = 1.0;
      for(int t = 0; t < dim - 1; ++t) wf *= w[fi[t]];
      double len = 0.0, prev[3] = {0, 0, 0};
      for(int i = 0; i < nq; ++i)
      {
        double xi[3] = {0, 0, 0}, x[3];
        int t = 0;
        for(int e = 0; e < dim; ++e) xi[e] = e == d ? z[i] : z[fi[t++]];
        map(xi, x);
        if(i > 0)
        {
          double s2 = 0.0;
          for(int c = 0; c < dim; ++c) s2 += (x[c] - prev[c]) * (x[c] - prev[c]);
          len += std::sqrt(s2);
        }
        for(int c = 0; c < dim; ++c) prev[c] = x[c];
      }
      acc += wf * len;
    }
    h[d] = acc;
  }
}

void build_layout(tpss_layout &L, const tpss_layout_desc &d)
{
  TPSS_REQUIRE(d.dim == 2 || d.dim == 3, "dim must be 2 or 3");
  TPSS_REQUIRE(d.degree >= 1 && d.degree <= 7, "degree must be in 1..7");
  TPSS_REQUIRE(d.dof_layout == TPSS_DOF_DGQ, "only the DGQ DoF layout is implemented");
  TPSS_REQUIRE(d.patch_variant == TPSS_PATCH_VERTEX || d.patch_variant == TPSS_PATCH_CELL,
               "invalid patch variant");
  TPSS_REQUIRE(d.smoother_variant == TPSS_ADDITIVE || d.smoother_variant == TPSS_MULTIPLICATIVE,
               "invalid smoother variant");
  L.dim = d.dim;
  L.k = d.degree;
  L.np = d.degree + 1;
  L.patch_variant = d.patch_variant;
  L.smoother_variant = d.smoother_variant;
  L.ncp = d.patch_variant == TPSS_PATCH_VERTEX ? 2 : 1;
  L.n = L.ncp * L.np;
  L.nloc = ipow(L.n, L.dim);
  L.npc = ipow(L.ncp, L.dim);
  L.cell_dofs = ipow(L.np, L.dim);
  L.n_cells = 1;
  for(int dd = 0; dd < 3; ++dd)
  {
    L.nc[dd] = dd < d.dim ? d.n_cells[dd] : 1;
    TPSS_REQUIRE(L.nc[dd] >= 1, "n_cells must be positive");
    L.n_cells *= L.nc[dd];
    L.h[dd].resize(L.nc[dd]);
    for(int c = 0; c < L.nc[dd]; ++c)
    {
      const double hv = (dd < d.dim && d.cell_h[dd]) ? d.cell_h[dd][c] : 1.0 / L.nc[dd];
      TPSS_REQUIRE(hv > 0.0, "cell widths must be positive");
      L.h[dd][c] = hv;
    }
  }
  TPSS_REQUIRE(L.n_cells < (int64_t(1) << 31), "too many cells");
  L.n_dofs = L.n_cells * L.cell_dofs;
  L.lexicographic = d.cell_dof_start == nullptr;
  L.cell_start.resize(L.n_cells);
  for(int64_t c = 0; c < L.n_cells; ++c)
  {
    const int64_t s = L.lexicographic ? c * L.cell_dofs : d.cell_dof_start[c];
    TPSS_REQUIRE(s >= 0 && s + L.cell_dofs <= L.n_dofs, "cell_dof_start out of range");
    L.cell_start[c] = s;
  }
  if(!L.lexicographic)
  {
    // the blocks must tile [0, n_dofs) without overlap
    std::vector<int64_t> sorted(L.cell_start);
    std::sort(sorted.begin(), sorted.end());
    for(int64_t c = 0; c < L.n_cells; ++c)
      TPSS_REQUIRE(sorted[c] == c * L.cell_dofs, "cell_dof_start must be a permutation of cell blocks");
  }

  // ---- patches and default colors
  const int dim = L.dim;
  const bool vertex = L.patch_variant == TPSS_PATCH_VERTEX;
  int na[3] = {1, 1, 1};
  for(int dd = 0; dd < dim; ++dd) na[dd] = vertex ? L.nc[dd] - 1 : L.nc[dd];
  std::vector<PatchRec> recs;
  if(na[0] > 0 && na[1] > 0 && na[2] > 0)
  {
    recs.reserve((size_t)na[0] * na[1] * na[2]);
    int64_t lex = 0;
    for(int a2 = 0; a2 < na[2]; ++a2)
      for(int a1 = 0; a1 < na[1]; ++a1)
        for(int a0 = 0; a0 < na[0]; ++a0, ++lex)
        {
          const int a[3] = {a0, a1, a2};
          PatchRec r{{0, 0, 0}, 0, false, lex};
          int parity = 0;
          for(int dd = 0; dd < dim; ++dd)
          {
            r.lo[dd] = a[dd];
            const int hi = a[dd] + L.ncp - 1;
            r.boundary = r.boundary || a[dd] == 0 || hi == L.nc[dd] - 1;
            if(vertex)
              r.color |= (((a[dd] + 1) % 2) == 0 ? 1 : 0) << dd;  // vertex index a+1 even
            else
              parity ^= a[dd] & 1;
          }
          if(!vertex && L.smoother_variant == TPSS_MULTIPLICATIVE) r.color = parity;
          recs.push_back(r);
        }
  }
  L.n_colors = vertex ? (1 << dim) : (L.smoother_variant == TPSS_MULTIPLICATIVE ? 2 : 1);
  if(d.patch_color)
  {
    // user coloring, indexed in the default storage order computed below
    std::stable_sort(recs.begin(), recs.end(), [](const PatchRec &x, const PatchRec &y) {
      return std::make_tuple(x.color, (int)x.boundary, x.lex) <
             std::make_tuple(y.color, (int)y.boundary, y.lex);
    });
    int maxc = -1;
    for(size_t i = 0; i < recs.size(); ++i)
    {
      TPSS_REQUIRE(d.patch_color[i] >= 0, "patch colors must be non-negative");
      recs[i].color = d.patch_color[i];
      maxc = std::max(maxc, (int)recs[i].color);
    }
    L.n_colors = maxc + 1;
  }
  std::stable_sort(recs.begin(), recs.end(), [](const PatchRec &x, const PatchRec &y) {
    return std::make_tuple(x.color, (int)x.boundary, x.lex) <
           std::make_tuple(y.color, (int)y.boundary, y.lex);
  });
  L.P = (int64_t)recs.size();
  L.color_start.assign(L.n_colors + 1, 0);
  for(const auto &r : recs) L.color_start[r.color + 1]++;
  for(int c = 0; c < L.n_colors; ++c) L.color_start[c + 1] += L.color_start[c];

  // ---- per patch: cells, FD keys; per cell: multiplicity and color conflict check
  L.lower.resize((size_t)L.P * 3);
  L.color.resize(L.P);
  L.patch_fd_key.resize((size_t)L.P * dim);
  std::vector<int64_t> first((size_t)L.P * L.npc);
  L.cell_multiplicity.assign(L.n_cells, 0);
  std::vector<int32_t> last_color(L.n_cells, -1);
  std::map<std::tuple<double, double, int, int>, int32_t> keymap;
  if(d.vertex_coords)
  {
    TPSS_REQUIRE(vertex, "surrogate widths are defined for vertex patches");
    TPSS_REQUIRE(d.surrogate_n_q == 0 || (d.surrogate_n_q >= 2 && d.surrogate_n_q <= 16),
                 "surrogate_n_q must be in 2..16");
    L.per_patch_fd = true;
    const size_t nv = (size_t)(L.nc[0] + 1) * (dim > 1 ? L.nc[1] + 1 : 1) * (dim > 2 ? L.nc[2] + 1 : 1);
    L.coords.assign(d.vertex_coords, d.vertex_coords + nv * dim);
    for(double x : L.coords) TPSS_REQUIRE(std::isfinite(x), "vertex_coords must be finite");
  }
  std::vector<double> gl_z, gl_w;
  if(d.vertex_coords) lobatto_rule(d.surrogate_n_q ? d.surrogate_n_q : 5, gl_z, gl_w);
  for(int64_t p = 0; p < L.P; ++p)
  {
    const auto &r = recs[p];
    for(int dd = 0; dd < 3; ++dd) L.lower[p * 3 + dd] = r.lo[dd];
    L.color[p] = r.color;
    for(int cn = 0; cn < L.npc; ++cn)
    {
      int c[3] = {r.lo[0], r.lo[1], r.lo[2]}, rem = cn;
      for(int dd = 0; dd < dim; ++dd)
      {
        c[dd] += rem % L.ncp;
        rem /= L.ncp;
      }
      const int64_t cell = c[0] + (int64_t)L.nc[0] * (c[1] + (int64_t)L.nc[1] * c[2]);
      first[(size_t)p * L.npc + cn] = L.cell_start[cell];
      L.cell_multiplicity[cell]++;
      // patches are sorted by color, so an earlier patch of the same color is a conflict
      if(last_color[cell] == r.color)
        fail(TPSS_ERR_INVALID_ARGUMENT,
             "coloring conflict: a cell belongs to two patches of color " + std::to_string(r.color));
      last_color[cell] = r.color;
    }
    double hs[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    if(d.vertex_coords)
    {
      // surrogate widths: average over the 2^(dim-1) patch cells sharing a 1-D cell index
      for(int cn = 0; cn < L.npc; ++cn)
      {
        int c[3] = {r.lo[0], r.lo[1], r.lo[2]};
        for(int e = 0; e < dim; ++e) c[e] += (cn >> e) & 1;
        double X[8 * 3], hc[3];
        for(int v = 0; v < (1 << dim); ++v)
        {
          int vi[3] = {c[0], c[1], c[2]};
          for(int e = 0; e < dim; ++e) vi[e] += (v >> e) & 1;
          const int64_t vid = vi[0] + (int64_t)(L.nc[0] + 1) * (vi[1] + (int64_t)(L.nc[1] + 1) * vi[2]);
          for(int e = 0; e < dim; ++e) X[v * dim + e] = d.vertex_coords[vid * dim + e];
        }
        cell_arc_lengths(dim, X, gl_z, gl_w, hc);
        for(int e = 0; e < dim; ++e) hs[e][(cn >> e) & 1] += hc[e] / (1 << (dim - 1));
      }
    }
    for(int dd = 0; dd < dim; ++dd)
    {
      const int c0 = r.lo[dd], c1 = r.lo[dd] + L.ncp - 1;
      double h0 = L.h[dd][c0], h1 = L.ncp == 2 ? L.h[dd][c1] : 0.0;
      if(d.vertex_coords)
      {
        h0 = hs[dd][0];
        h1 = hs[dd][1];
      }
      const int lo = c0 == 0, hi = c1 == L.nc[dd] - 1;
      auto key = std::make_tuple(h0, h1, lo, hi);
      auto it = keymap.find(key);
      int32_t idx;
      if(it == keymap.end())
      {
        idx = (int32_t)L.fd_keys.size();
        keymap.emplace(key, idx);
        L.fd_keys.push_back({h0, h1, lo, hi});
      }
      else
        idx = it->second;
      L.patch_fd_key[(size_t)p * dim + dd] = idx;
    }
  }
  L.patch_first = std::move(first);
  // vertex patches on the structured level: the FD key of direction d depends only on the
  // vertex index v_d, which the streaming kernel uses instead of per-patch indices
  if(vertex && !L.per_patch_fd)
    for(int dd = 0; dd < dim; ++dd)
    {
      L.vertex_fd[dd].assign(L.nc[dd] + 1, -1);
      for(int v = 1; v < L.nc[dd]; ++v)
      {
        auto key = std::make_tuple(L.h[dd][v - 1], L.h[dd][v], (int)(v - 1 == 0), (int)(v == L.nc[dd] - 1));
        auto it = keymap.find(key);
        L.vertex_fd[dd][v] = it == keymap.end() ? -1 : it->second;
      }
    }
}
}  // namespace

// Device copies are made on first use, so the host-side layout (patches, colors, keys) can
// be built and inspected without a GPU.
void layout_to_device(const tpss_layout &Lc)
{
  auto &L = const_cast<tpss_layout &>(Lc);
  std::lock_guard<std::mutex> lock(L.device_mutex);
  if(L.on_device) return;
  L.d_patch_first.upload(L.patch_first.data(), L.patch_first.size());
  L.d_patch_fd.upload(L.patch_fd_key.data(), L.patch_fd_key.size());
  if(!L.lexicographic) L.d_cell_start.upload(L.cell_start.data(), L.cell_start.size());
  for(int dd = 0; dd < 3; ++dd)
    if(!L.vertex_fd[dd].empty()) L.d_vertex_fd[dd].upload(L.vertex_fd[dd].data(), L.vertex_fd[dd].size());
  L.on_device = true;
}
}  // namespace tpss

using namespace tpss;

extern "C" const char *tpss_last_error(void) { return tpss::last_error_cstr(); }

extern "C" const char *tpss_version(void) { return "tpss_gb300 0.1 (sm_103a)"; }

extern "C" int tpss_layout_create(const tpss_layout_desc *desc, tpss_layout **out)
{
  return guarded([&] {
    TPSS_REQUIRE(desc && out, "null argument");
    *out = nullptr;
    auto L = std::make_unique<tpss_layout>();
    build_layout(*L, *desc);
    *out = L.release();
  });
}

extern "C" int tpss_layout_info(const tpss_layout *L, int64_t *n_dofs, int64_t *n_patches,
                                int *n_colors)
{
  return guarded([&] {
    TPSS_REQUIRE(L, "null layout");
    if(n_dofs) *n_dofs = L->n_dofs;
    if(n_patches) *n_patches = L->P;
    if(n_colors) *n_colors = L->n_colors;
  });
}

extern "C" int tpss_layout_patches(const tpss_layout *L, int32_t *lower_cells, int32_t *colors)
{
  return guarded([&] {
    TPSS_REQUIRE(L, "null layout");
    if(lower_cells && L->P) std::memcpy(lower_cells, L->lower.data(), sizeof(int32_t) * 3 * L->P);
    if(colors && L->P) std::memcpy(colors, L->color.data(), sizeof(int32_t) * L->P);
  });
}

extern "C" void tpss_layout_destroy(tpss_layout *L) { delete L; }
