"""The C++ host interface (include/tpss_gpu.hpp) compiles against the C ABI and links with
libtpss_gpu.so (no GPU needed: the program is built and only its error path is run)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include "tpss_gpu.hpp"
#include <cstdio>
int main()
{
  using namespace tpss_gpu;
  SubdomainHandler::AdditionalData ad;
  ad.dim = 3; ad.degree = 2; ad.n_cells = {3, 3, 3};
  auto sh = std::make_shared<SubdomainHandler>(ad);   // host-side layout, no device memory
  if(sh->n_subdomains() != 8 || sh->n_colors() != 8) return 1;
  try
  {
    ad.dim = 5;
    SubdomainHandler bad(ad);
    return 2;
  }
  catch(const Error &e)
  {
    if(e.code != TPSS_ERR_INVALID_ARGUMENT) return 3;
  }
  std::printf("%s\n", tpss_version());
  return 0;
}
'''


def test_cpp_wrapper_compiles_and_runs(tpss, tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    from tpss_gb300 import build as b
    lib = b.build()
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-ltpss_gpu", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "sm_103a" in r.stdout
