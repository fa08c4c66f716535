"""Builds the in-tree CUDA library ``libakua_pbf.so`` for sm_103a.

The library is compiled in place (next to this file) with nvcc: its translation units in
parallel, one ``-gencode``, then one link.  Host code is compiled with ``-ffp-contract=off`` and
device code with ``--fmad=false``: every fused multiply-add of the step is written out in the
source, so results do not depend on the compiler's contraction choices on x86 or Arm hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
LIB_NAME = "libakua_pbf.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libakua_pbf.so")


def sources() -> list[str]:
    return [os.path.join(CSRC, "pbf_solver.cu"), os.path.join(CSRC, "sort_noalloc.cu"),
            os.path.join(CSRC, "mlp.cu"), os.path.join(CSRC, "state_io.cpp"),
            os.path.join(CSRC, "splat.cu")]


def headers() -> list[str]:
    out = [os.path.join(INCLUDE, "akua_pbf.h")]
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cuh", ".h")):
            out.append(os.path.join(CSRC, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def nvcc_command(output: str, extra: list[str] | None = None) -> list[str]:
    return [
        nvcc_path(), *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-O3", "-shared",
        "-I", INCLUDE, "-I", CSRC,
        *(extra or []),
        "-o", output, *sources(),
    ]


def compile_command(src: str, obj: str) -> list[str]:
    """One translation unit of the library, compiled to an object with nvcc_command's flags."""
    cmd = nvcc_command(obj)
    cmd = [c for c in cmd[:cmd.index("-o")] if c != "-shared"]
    return cmd + ["-c", "-o", obj, src]


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile libakua_pbf.so if any source is newer than it; returns its path.  The translation
    units compile in parallel (one nvcc each), then one nvcc links them."""
    deps = sources() + headers() + [os.path.abspath(__file__)]
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp.%d" % os.getpid()
    with tempfile.TemporaryDirectory(prefix="akua_build_") as work:
        jobs = []
        for src in sources():
            obj = os.path.join(work, os.path.basename(src) + ".o")
            cmd = compile_command(src, obj)
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            jobs.append((src, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                                    stderr=subprocess.PIPE, text=True)))
        failed = []
        for src, _, proc in jobs:
            out, err = proc.communicate()
            if proc.returncode != 0:
                failed.append("%s (%d):\n%s\n%s" % (src, proc.returncode, out, err))
        if failed:
            raise RuntimeError("nvcc failed: " + "\n".join(failed))
        link = [nvcc_path(), *ARCH_FLAGS, "-shared", "-o", tmp] + [obj for _, obj, _ in jobs]
        if verbose:
            print(" ".join(link), file=sys.stderr)
        res = subprocess.run(link, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc link failed (%d):\n%s\n%s"
                               % (res.returncode, res.stdout, res.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
