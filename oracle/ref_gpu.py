"""TEST INFRASTRUCTURE ONLY.  Builds the reference's own CUDA kernels for sm_103a and drives them.

build_cubins(): compiles src/CUDA/NeighbourSearchCUDA.cu, ConstraintSolverCUDA.cu and
IntegrationCUDA.cu of the reference tree, unchanged and read in place, into device-code cubins
under oracle/_ref/ (git-ignored; they travel with the working tree to the GPU machine).  Only an
empty GL/gl.h stand-in is added to the include path (cuda_gl_interop.h includes it).

build_harness(): compiles oracle/ref_harness.cu (this project's code) on the GPU machine; it loads
the cubins with the CUDA driver API and re-sequences PBFSolver::step (src/Simulation/
PBFSolver.cpp:22-78) over a device array of particle records, with the reference's thrust::sort.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
UNITS = ["NeighbourSearchCUDA", "ConstraintSolverCUDA", "IntegrationCUDA"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def cubin_paths() -> list[str]:
    return [os.path.join(REF_DIR, u + ".cubin") for u in UNITS]


def have_cubins() -> bool:
    return all(os.path.exists(p) for p in cubin_paths())


def build_cubins(ref_root: str | None = None) -> list[str]:
    """Reference flags (CMakeLists.txt:66-70: --extended-lambda -diag-suppress=20012), sm_103a.
    `ref_root` defaults to oracle/ref_root.py's lookup."""
    from oracle.ref_root import require_reference_root

    ref_root = require_reference_root(ref_root)
    os.makedirs(REF_DIR, exist_ok=True)
    out = []
    for u in UNITS:
        dst = os.path.join(REF_DIR, u + ".cubin")
        cmd = [nvcc(), "-cubin", *ARCH, "-std=c++17", "--extended-lambda", "-diag-suppress=20012",
               "-I", os.path.join(ref_root, "include"), "-I", os.path.join(HERE, "ref_shim_gl"),
               "-o", dst, os.path.join(ref_root, "src", "CUDA", u + ".cu")]
        subprocess.run(cmd, check=True)
        out.append(dst)
    return out


def harness_path() -> str:
    return os.path.join(REF_DIR, "ref_harness")


def build_harness() -> str:
    os.makedirs(REF_DIR, exist_ok=True)
    exe = harness_path()
    src = os.path.join(HERE, "ref_harness.cu")
    if os.path.exists(exe) and os.path.getmtime(exe) > os.path.getmtime(src):
        return exe
    cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", "-o", exe, src, "-lcuda"]
    subprocess.run(cmd, check=True)
    return exe


def run(particles, params: dict, steps: int, mode: str = "resident", dump_lists: bool = False,
        timing: bool = False, workdir: str | None = None):
    """Steps `particles` (PARTICLE_DTYPE array, modified in place) `steps` times with the
    reference kernels.  Returns a dict with the last step's neighbour lists (if asked) and the
    measured milliseconds per step (if `timing`)."""
    import numpy as np
    import tempfile

    exe = build_harness()
    wd = workdir or tempfile.mkdtemp(prefix="refgpu_")
    inp = os.path.join(wd, "in.bin")
    outp = os.path.join(wd, "out.bin")
    particles.tofile(inp)
    args = [exe, "--cubins", REF_DIR, "--in", inp, "--out", outp, "--n", str(len(particles)),
            "--steps", str(steps), "--mode", mode]
    for k, v in params.items():
        args += ["--" + k, ",".join(str(x) for x in v) if isinstance(v, (list, tuple)) else str(v)]
    if dump_lists:
        args += ["--lists", os.path.join(wd, "lists")]
    res = subprocess.run(args, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("ref_harness failed: %s\n%s" % (res.stdout, res.stderr))
    out = np.fromfile(outp, dtype=particles.dtype)
    particles[:] = out
    info = {"stdout": res.stdout}
    for line in res.stdout.splitlines():
        if line.startswith("ms_per_step"):
            info["ms_per_step"] = float(line.split()[1])
    if dump_lists:
        cap = int(params.get("cap", 128))
        n = len(particles)
        info["nbr"] = np.fromfile(os.path.join(wd, "lists") + ".nbr", dtype=np.uint32).reshape(n, cap)
        info["cnt"] = np.fromfile(os.path.join(wd, "lists") + ".cnt", dtype=np.uint32)
    return info
