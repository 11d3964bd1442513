"""The C++ host interface (include/tpss_gpu.hpp) driven on the GPU.

A C++ program is compiled against the header, linked with libtpss_gpu.so and the CUDA runtime,
and used the way a reference caller uses the smoother path:
  - SchwarzPreconditioner::initialize(subdomain_handler, operator, additional_data) and
    vmult(dst, src) on every golden case of tests/golden/vmult.npz (additive and
    multiplicative, vertex and cell patches): relative max-norm error <= 1e-12 against the
    fixture (PreconditionerBase::vmult, preconditioner/preconditioner_base.h:21-31);
  - Tvmult throws the not-implemented error, as the reference's does;
  - SchwarzSmoother::vmult with one step and damping 1 equals the preconditioner's vmult, and
    step(x, b) from x = 0 twice equals x = P b + P (b - A P b) (smoother_richardson.h:118-156),
    both to 1e-12;
  - MultigridSolver::solve on a golden CG + GMG case gives the stored iteration count.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

PROGRAM = r'''
#include "tpss_gpu.hpp"
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

using namespace tpss_gpu;

static std::vector<double> read_bin(const std::string &path, size_t n)
{
  std::vector<double> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char *>(v.data()), n * sizeof(double));
  return v;
}

static void write_bin(const std::string &path, const std::vector<double> &v)
{
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

struct Dev
{
  double *p = nullptr;
  explicit Dev(size_t n) { cudaMalloc(&p, n * sizeof(double)); }
  ~Dev() { cudaFree(p); }
  void put(const std::vector<double> &h) { cudaMemcpy(p, h.data(), h.size() * 8, cudaMemcpyHostToDevice); }
  std::vector<double> get(size_t n) const
  {
    std::vector<double> h(n);
    cudaMemcpy(h.data(), p, n * 8, cudaMemcpyDeviceToHost);
    return h;
  }
};

static double rel(const std::vector<double> &a, const std::vector<double> &b)
{
  double m = 0, r = 0;
  for(size_t i = 0; i < a.size(); ++i)
  {
    m = std::fmax(m, std::fabs(a[i] - b[i]));
    r = std::fmax(r, std::fabs(b[i]));
  }
  return m / r;
}

int main(int argc, char **argv)
{
  std::ifstream cases(argv[1]);
  std::string line;
  while(std::getline(cases, line))
  {
    std::istringstream in(line);
    std::string kind;
    in >> kind;
    if(kind == "vmult")
    {
      int dim, k, pv, sv;
      std::vector<int> nc(3);
      double omega, ip;
      size_t N;
      std::string src_path, dst_path;
      in >> dim >> k >> nc[0] >> nc[1] >> nc[2] >> pv >> sv >> omega >> ip >> N >> src_path >> dst_path;
      SubdomainHandler::AdditionalData ad;
      ad.dim = dim;
      ad.degree = k;
      ad.n_cells = std::vector<int>(nc.begin(), nc.begin() + dim);
      ad.patch_variant = pv ? PatchVariant::vertex : PatchVariant::cell;
      ad.smoother_variant = sv ? SmootherVariant::multiplicative : SmootherVariant::additive;
      auto sh = std::make_shared<SubdomainHandler>(ad);
      LaplaceOperator op(sh, ip);
      auto P = std::make_shared<SchwarzPreconditioner>();
      SchwarzPreconditioner::AdditionalData pd;
      pd.relaxation = omega;
      pd.ip_factor = ip;
      P->initialize(sh, &op, pd);
      Dev src(N), dst(N);
      src.put(read_bin(src_path, N));
      P->vmult(dst.p, src.p);
      const std::vector<double> Pb = dst.get(N);
      write_bin(dst_path, Pb);
      bool threw = false;
      try
      {
        P->Tvmult(dst.p, src.p);
      }
      catch(const Error &e)
      {
        threw = e.code == TPSS_ERR_NOT_IMPLEMENTED;
      }
      if(!threw) return 10;
      if(sv == 0)
      {
        // SchwarzSmoother / SmootherRichardson semantics
        SchwarzSmoother S;
        SchwarzSmoother::AdditionalData sd;
        S.initialize(op, P, sd);
        Dev x(N);
        S.vmult(x.p, src.p);
        const double e1 = rel(x.get(N), Pb);
        // two steps from zero: x1 = P b, x2 = x1 + P (b - A x1)
        cudaMemset(x.p, 0, N * 8);
        S.step(x.p, src.p);
        S.step(x.p, src.p);
        const std::vector<double> x2 = x.get(N);
        Dev t(N), r(N);
        op.vmult(t.p, dst.p);  // A P b
        std::vector<double> b = read_bin(src_path, N), Ax1 = t.get(N), res(N);
        for(size_t i = 0; i < N; ++i) res[i] = b[i] - Ax1[i];
        r.put(res);
        P->vmult(t.p, r.p);
        std::vector<double> expect = t.get(N);
        for(size_t i = 0; i < N; ++i) expect[i] += Pb[i];
        const double e2 = rel(x2, expect);
        std::printf("smoother %.3e %.3e\n", e1, e2);
      }
    }
    else if(kind == "mg")
    {
      tpss_mg_desc d{};
      size_t N;
      std::string rhs;
      in >> d.dim >> d.degree >> d.n_rep >> d.n_cells_fine >> d.patch_variant >> d.smoother_variant >>
        d.relaxation >> N >> rhs;
      d.ip_factor = 1.0;
      d.precision = TPSS_FP64;
      d.coarse_tol = 1e-12;
      d.use_graph = 1;
      MultigridSolver mg(d);
      Dev u(N), f(N);
      f.put(read_bin(rhs, N));
      cudaMemset(u.p, 0, N * 8);
      std::vector<double> hist;
      const int it = mg.solve(u.p, f.p, 1e-8, 1e-14, 100, &hist);
      std::printf("mg %d %.6e\n", it, hist.back());
    }
  }
  cudaDeviceSynchronize();
  return 0;
}
'''


def test_cpp_header_drives_the_gpu(tpss, oracle, xcheck, tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    from tpss_gb300 import build as b
    lib = b.build()
    libdir = os.path.dirname(lib)
    src = tmp_path / "drive.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "drive"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(CUDA, "include"), str(src), "-o", str(exe), "-L", libdir, "-ltpss_gpu",
                    f"-Wl,-rpath,{libdir}", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
                    f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"], check=True)
    g = np.load(os.path.join(GOLDEN, "vmult.npz"))
    cases = json.load(open(os.path.join(GOLDEN, "vmult_cases.json")))
    lines = []
    for i, c in enumerate(cases):
        s = g[f"c{i}_src"]
        s.astype(np.float64).tofile(tmp_path / f"c{i}.src")
        nc = list(c["n_cells"]) + [1] * (3 - len(c["n_cells"]))
        lines.append(f"vmult {c['dim']} {c['k']} {nc[0]} {nc[1]} {nc[2]} {c['patch_variant']} "
                     f"{c['smoother_variant']} {c['omega']!r} {c['ip']!r} {s.size} {tmp_path / f'c{i}.src'} "
                     f"{tmp_path / f'c{i}.dst'}")
    mgc = [c for c in json.load(open(os.path.join(GOLDEN, "mg_iterations.json"))) if c["rhs"] == "random"][0]
    N = mgc["n_cells_fine"] ** mgc["dim"] * (mgc["k"] + 1) ** mgc["dim"]
    f = np.random.Generator(np.random.Philox(mgc["rhs_seed"])).uniform(-1, 1, N)
    f.tofile(tmp_path / "mg.rhs")
    omega = oracle.lookup_damping_factor(mgc["patch_variant"], mgc["smoother_variant"], mgc["dim"])
    lines.append(f"mg {mgc['dim']} {mgc['k']} {mgc['n_rep']} {mgc['n_cells_fine']} {mgc['patch_variant']} "
                 f"{mgc['smoother_variant']} {omega!r} {N} {tmp_path / 'mg.rhs'}")
    (tmp_path / "cases.txt").write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), str(tmp_path / "cases.txt")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    for i, c in enumerate(cases):
        got = np.fromfile(tmp_path / f"c{i}.dst", dtype=np.float64)
        ref = g[f"c{i}_dst"]
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), i
    sm = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("smoother")]
    assert len(sm) == sum(1 for c in cases if c["smoother_variant"] == 0)
    for _, e1, e2 in sm:
        assert float(e1) <= 1e-12 and float(e2) <= 1e-12, (e1, e2)
    mg = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("mg")]
    assert len(mg) == 1 and int(mg[0][1]) == mgc["iterations"], (mg, mgc["iterations"])
