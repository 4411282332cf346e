"""Build the native parts in-tree.

* ``motex_gb300/lib/libmotex_gpu.so`` -- CUDA kernels + C ABI
  (include/motex_gpu.h), compiled for sm_103a only.
* ``motex_gb300/lib/motexGPU`` -- the drop-in CLI (same switches and output
  file as motexCPU / motexOMP), linked against the library.

Translation units compile in parallel; objects are cached by source mtime
under ``motex_gb300/_build``.  ``python -m motex_gb300.build`` runs it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + INC, "-I" + CSRC]
CU_SOURCES = ["kernels.cu", "dp.cu", "dp_hclr.cu", "dp_persist.cu", "dp_struct.cu", "dp_structn.cu", "mini.cu", "motex_gpu.cu", "probe.cu", "no_alloc.cu", "server.cu"]
HEADERS = ["common.cuh", "kernels.cuh", "dp_body.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def build(verbose: bool = False, extra_flags=()) -> str:
    """Compile everything that is out of date; return the library path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INC, "motex_gpu.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(LIB, "libmotex_gpu.so")
    if _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lcuda"])
    cli_src = os.path.join(HOST, "motexGPU.cc")
    cli = os.path.join(LIB, "motexGPU")
    if os.path.exists(cli_src) and _stale(cli, [cli_src, lib, os.path.join(INC, "motex_gpu.h")]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-I" + INC, cli_src,
              "-o", cli, "-L" + LIB, "-lmotex_gpu", "-Wl,-rpath,$ORIGIN"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
