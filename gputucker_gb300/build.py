"""In-tree build of the gputucker_gb300 native library and CLI.

    python -m gputucker_gb300.build          # or: import gputucker_gb300.build as b; b.build()

Compiles csrc/*.cu and csrc/*.cpp with nvcc for sm_103a only (one -gencode),
in parallel, into gputucker_gb300/lib/libgputucker_gb300.so, and the CLI
csrc/cli.cpp into gputucker_gb300/bin/gputucker_gb300.  Object files go to
gputucker_gb300/_build/ and are rebuilt only when a source or header changed.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libgputucker_gb300.so")
CLI = os.path.join(BINDIR, "gputucker_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without FP contraction: the serial value_t sums that restate the
# reference's (its norm) must round every product and sum separately
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]
LIB_SOURCES = ["api.cpp", "parse.cpp", "gen.cpp", "partition.cu", "sweep.cu", "tc_sweep.cu", "noalloc.cu", "batch.cu", "plan.cpp", "warmstart.cu", "tc_stream.cu", "core_update.cu", "validate.cu", "hostpart.cpp"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile the library and the CLI; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _stale(obj, [path] + headers) or ptxas_verbose:
            cmd = [nvcc, "-c", path, "-o", obj] + COMMON + ARCH
            if src.endswith(".cu") and ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            list(ex.map(_run_logged(verbose), jobs))
    if _stale(LIB, objs):
        _run([nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-lpthread"])
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + headers):
        _run([nvcc, cli_src, "-o", CLI, "-O2", "-std=c++17", "-I" + INCLUDE, "-L" + LIBDIR,
              "-lgputucker_gb300", "-Xlinker", "-rpath=$ORIGIN/../lib"])
    return LIB


SANITIZE = ["-fsanitize=address", "-fsanitize=undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=undefined"]


def build_host_sanitized(out_dir: str) -> str:
    """The library with its host-only C++ sources (parser, generator, planner and
    checkpoint, API layer) compiled under AddressSanitizer + UndefinedBehavior-
    Sanitizer, linked with the regular objects of the CUDA sources, into
    out_dir/libgputucker_gb300.so (for the host sanitizer test; a program that
    loads it must be built with the same -fsanitize flags)."""
    build()
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    jobs, objs = [], []
    for src in LIB_SOURCES:
        if src.endswith(".cpp"):
            obj = os.path.join(out_dir, src + ".o")
            jobs.append([nvcc, "-c", os.path.join(CSRC, src), "-o", obj, "-O1", "-g", "-std=c++17", "-Xcompiler",
                         "-fPIC,-ffp-contract=off," + ",".join(SANITIZE), "-I" + INCLUDE, "-I" + CSRC] + ARCH)
            objs.append(obj)
        else:
            objs.append(os.path.join(BUILD, src + ".o"))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(_run_logged(False), jobs))
    lib = os.path.join(out_dir, "libgputucker_gb300.so")
    _run([nvcc, "-shared", "-o", lib] + objs + ARCH + ["-lpthread", "-Xcompiler", ",".join(SANITIZE)])
    return lib


def _run_logged(verbose: bool):
    def f(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
    return f


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
