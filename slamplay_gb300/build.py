"""Build recipe of libgba.so (the GB300 bundle-adjustment library) and the
C++ demo, in-tree under slamplay_gb300/_build/.

CUDA sources are compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host sources with g++.  No
fast-math anywhere; host code is built with ``-ffp-contract=off`` so x86-64
and aarch64 hosts round alike.  Compilation runs in parallel and is
incremental (object newer than its source and every header).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgba.so")

CUDA_SOURCES = ["k_eval.cu", "k_solve.cu", "k_pcg.cu", "k_schur.cu", "k_pcg_cluster.cu", "k_pcg_grid.cu", "k_noalloc.cu"]
CXX_SOURCES = ["engine.cpp", "prep.cpp", "api.cpp", "server.cpp", "bal_io.cpp", "synth.cpp", "tune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith((".h", ".hpp"))]
    return hs


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles libgba.so (and the demo app) if stale; returns the library path."""
    ch = cuda_home()
    nvcc = os.path.join(ch, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    cmds: list[tuple[str, list[str]]] = []
    objs = []
    for f in CUDA_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            cmds.append((obj, [nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                               "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj + ".tmp"]))
    for f in CXX_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            cmds.append((obj, ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread",
                               "-Wall", "-Wno-unused-function", "-I", INCLUDE, "-I", CSRC,
                               "-I", os.path.join(ch, "include"), "-c", src, "-o", obj + ".tmp"]))
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
            futs = {ex.submit(_run, c): o for o, c in cmds}
            for fu in cf.as_completed(futs):
                fu.result()
                os.replace(futs[fu] + ".tmp", futs[fu])
                if verbose:
                    print("built", os.path.basename(futs[fu]), file=sys.stderr)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-cudart", "static",
              "-Xcompiler", "-pthread", "-lrt", "-ldl"])
        os.replace(LIB + ".tmp", LIB)
    app_src = os.path.join(HERE, "apps", "bundle_adjustment_gb300.cpp")
    app = os.path.join(BUILD, "bundle_adjustment_gb300")
    if os.path.exists(app_src) and _stale(app, [app_src, LIB] + hdrs):
        _run(["g++", "-std=c++17", "-O2", "-I", INCLUDE, app_src, "-o", app + ".tmp",
              "-L", BUILD, "-lgba", "-Wl,-rpath,$ORIGIN"])
        os.replace(app + ".tmp", app)
    return LIB


def build_oracle(reference: bool = True) -> None:
    """Builds the CPU checkers (oracle/_build, and oracle/_ref when the
    reference tree is present).  Test infrastructure, not part of libgba."""
    script = os.path.join(ROOT, "oracle", "build_ref.sh")
    _run(["bash", script, "all" if reference else "oracle"])


if __name__ == "__main__":
    print(build(verbose=True))
    build_oracle()
