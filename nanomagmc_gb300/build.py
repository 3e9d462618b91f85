"""Build recipe of libnmmc (CUDA for sm_103a + host C++), in-tree.

Produces ``nanomagmc_gb300/_build/libnmmc.so`` and the ``nmmc_run`` program. The CUDA
translation units are compiled with ``nvcc -gencode arch=compute_103a,code=sm_103a``;
the host C++ parts with g++ (``-ffp-contract=off``: the Weibull shape test must give the
same masks on x86_64 and aarch64 hosts). Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libnmmc.so")
RUN = os.path.join(OUT, "nmmc_run")

CUDA_SOURCES = ["nmmc_kernels.cu", "nmmc_wave.cu", "nmmc_pf.cu", "nmmc_stencil.cu", "nmmc_resident.cu", "nmmc_general.cu", "nmmc_api.cu",
                "nmmc_noalloc.cu", "nmmc_gen.cu"]
HOST_SOURCES = ["nmmc_host.cpp", "nmmc_driver.cpp", "nmmc_warmstart.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "nmmc.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT, src + ".o")
    if not _stale(obj, [path] + _headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xptxas", "-v" if verbose else "-O3", "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
               "-I/usr/local/cuda/include", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT, f))
    srcs = CUDA_SOURCES + HOST_SOURCES
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, LIB)
    main_src = os.path.join(CSRC, "nmmc_run_main.cpp")
    if force or _stale(RUN, [LIB, main_src]):
        cmd = ["g++", "-std=c++17", "-O2", main_src, "-o", RUN, "-L" + OUT, "-lnmmc",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nmmc_run link failed: %s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
