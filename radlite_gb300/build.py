"""In-tree build of the CUDA library (sm_103a) and the RADlite_gpu executable."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction, so that host arithmetic rounds alike on x86 and Arm
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-lineinfo"]
SOURCES = ["rl_kernels.cu", "rl_adjoint.cu", "rl_host.cpp", "rl_capi.cpp", "rl_batch.cpp", "rl_diff.cpp",
           "rl_noalloc.cu", "rl_posvel.cu", "rl_genspec.cu", "rl_walk_tau.cu", "rl_walk_chk.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build radlite_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every translation unit in parallel, link librlgpu.so and RADlite_gpu."""
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    objs = []
    cmds = []
    for src in SOURCES + ["rl_main.cpp"]:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        extra = ["-Xptxas", "-v"] if (ptxas_info and src.endswith(".cu")) else []
        cmds.append([cc, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        logs = list(ex.map(_run, cmds))
    lib = os.path.join(OUT, "librlgpu.so")
    _run([cc, *ARCH, "-shared", "-o", lib, *objs[:-1]])
    exe = os.path.join(OUT, "RADlite_gpu")
    _run([cc, *ARCH, "-o", exe, objs[-1], "-L" + OUT, "-lrlgpu", "-Xlinker", "-rpath=$ORIGIN"])
    if verbose:
        sys.stdout.write("".join(logs))
    return lib


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
