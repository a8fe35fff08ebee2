"""Builds the native parts of the package in-tree, without cmake.

Products (all git-ignored, rebuilt on every machine):
  boidssimulatormpi_gb300/libboids_gb300.so   the C-ABI library (include/boids.h)
  boidssimulatormpi_gb300/bin/boidsim          all-pairs CLI (reference target boidsim)
  boidssimulatormpi_gb300/bin/boidsim_grid     grid CLI (reference target boidsim_grid)

Device code is compiled for sm_103a only.  Host code is compiled with
-ffp-contract=off so that the initial-state draws round the same way on x86
and aarch64 hosts.
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
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libboids_gb300.so")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found; set CUDA_HOME")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _sources(*names):
    return [os.path.join(CSRC, n) for n in names]


HEADERS = _sources("boids_engine.h") + [os.path.join(INCLUDE, "boids.h")]


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    inc = ["-I" + INCLUDE, "-I" + CSRC]
    jobs = []

    def obj(name):
        return os.path.join(BUILD, name + ".o")

    cu = [("boids_kernels.cu", ["boids_engine.h", "boids_softfp.h"]),
          ("boids_noalloc.cu", ["boids_engine.h"]),
          ("boids_mlp.cu", [])]
    for src, deps in cu:
        o = obj(os.path.splitext(src)[0])
        srcs = _sources(src, *deps) + HEADERS
        if force or not _newer(o, srcs):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "--fmad=false", "-std=c++17",
                   "-Xcompiler", "-fPIC", *inc, "-c", os.path.join(CSRC, src), "-o", o]
            cmd[1:1] = os.environ.get("BOIDS_NVCC_EXTRA", "").split()  # tuning experiments
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    cpp = ["boids_capi.cpp", "boids_ensemble.cpp"]
    for src in cpp:
        o = obj(os.path.splitext(src)[0])
        if force or not _newer(o, _sources(src) + HEADERS):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-Wextra", "-Wno-unused-parameter", *inc,
                         "-I" + os.path.join(cuda, "include"), "-c", os.path.join(CSRC, src), "-o", o])
    out = []
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            out.append(r)
    objs = [obj("boids_kernels"), obj("boids_noalloc"), obj("boids_mlp"), obj("boids_capi"), obj("boids_ensemble")]
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run(["g++", "-shared", "-o", tmp, *objs, "-L" + os.path.join(cuda, "lib64"),
              "-Wl,-Bstatic", "-lcudart_static", "-Wl,-Bdynamic", "-ldl", "-lrt", "-lpthread",
              "-Wl,--no-undefined", "-Wl,-soname,libboids_gb300.so"])
        os.replace(tmp, LIB)
    # CLI binaries
    cli_src = _sources("boidsim_main.cpp", "boids_cli.cpp", "boids_cli.h")
    if os.path.exists(cli_src[0]):
        for name, engine in (("boidsim", "BOIDS_ENGINE_ALLPAIRS"), ("boidsim_grid", "BOIDS_ENGINE_GRID")):
            exe = os.path.join(BIN, name)
            if force or not _newer(exe, cli_src + HEADERS + [LIB]):
                _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", *inc,
                      "-DBOIDSIM_ENGINE=" + engine, cli_src[0], cli_src[1], "-o", exe, "-pthread",
                      "-L" + PKG, "-lboids_gb300", "-Wl,-rpath,$ORIGIN/.."])
    if verbose:
        sys.stdout.write("".join(out))
    return LIB


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    a = ap.parse_args()
    print(build(verbose=True, force=a.force, ptxas_info=a.ptxas_info))
