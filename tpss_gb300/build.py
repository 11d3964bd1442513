"""Build recipe of the CUDA library libtpss_gpu.so (sm_103a), in-tree under tpss_gb300/_build.

Each translation unit is compiled by nvcc in parallel; the fused Schwarz kernel source
fd_inst.cu is compiled four times (float/double x 2D/3D).  Objects are rebuilt only when a
source or header is newer.  No torch dependency: the library exposes the C ABI of
include/tpss_gpu.h only.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtpss_gpu.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr", "-I", CSRC, "-I", os.path.join(ROOT, "include")]

UNITS = [
    ("setup.cu", []), ("eigen.cu", []), ("layout.cu", []), ("precond.cu", []),
    ("operator.cu", []), ("mg.cu", []), ("diag.cu", []), ("stream3d.cu", []), ("mapped.cu", []), ("mapped_mf.cu", []), ("local.cu", []), ("mlp.cu", []), ("learned.cu", []), ("c0ip.cu", []),
    ("plane_inst.cu", ["-DPLANE_BZ=8"]), ("plane_inst.cu", ["-DPLANE_BZ=4"]),
    ("stream_k5.cu", ["-DK5_PART=0"]), ("stream_k5.cu", ["-DK5_PART=1"]),
    ("fd_inst.cu", ["-DFD_T=float", "-DFD_DIM=2"]),
    ("fd_inst.cu", ["-DFD_T=float", "-DFD_DIM=3"]),
    ("fd_inst.cu", ["-DFD_T=double", "-DFD_DIM=2"]),
    ("fd_inst.cu", ["-DFD_T=double", "-DFD_DIM=3"]),
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _obj_name(src, defs):
    tag = "".join(d.split("=")[-1] for d in defs)
    return os.path.join(OUT, os.path.splitext(src)[0] + ("_" + tag if tag else "") + ".o")


def _newest_dep():
    deps = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    deps.append(os.path.join(ROOT, "include", "tpss_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return max(os.path.getmtime(d) for d in deps if os.path.exists(d))


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    dep_time = _newest_dep()
    todo = []
    objs = []
    for src, defs in UNITS:
        obj = _obj_name(src, defs)
        objs.append(obj)
        spath = os.path.join(CSRC, src)
        if (not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(spath)
                or os.path.getmtime(obj) < dep_time):
            todo.append([cc, *ARCH, *FLAGS, *defs, "-c", spath, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for msg in ex.map(run, todo):
                if verbose and msg:
                    print(msg)
    if todo or not os.path.exists(LIB):
        cmd = [cc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        run(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
