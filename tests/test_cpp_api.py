"""The C++ host interface (include/akua/PBFSolver.hpp): compiles against the C ABI here; on a GPU it
steps the reference dam-break scene through PBFSolver::step / stepHost and must produce the same
records, byte for byte, as the Python binding of the same library."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from akuaengine_gb300 import PARTICLE_DTYPE, PBFConfig, LambdaCorrParams, PBFSolver, scene
from akuaengine_gb300 import build as _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "pbf_cpp_steps.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def compile_demo(out_dir):
    lib_dir = os.path.dirname(_build.LIB_PATH)
    exe = os.path.join(out_dir, "pbf_cpp_steps")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"), SRC,
           "-L", lib_dir, "-lakua_pbf", "-Wl,-rpath," + lib_dir,
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.fixture(scope="module")
def demo(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    _build.build_library()
    return compile_demo(str(tmp_path_factory.mktemp("cpp")))


def test_cpp_header_compiles_and_links(demo):
    assert os.path.exists(demo)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["host", "device"])
def test_cpp_steps_match_python(demo, tmp_path, mode, cuda_lib):
    sc = scene.reference_dam_break()
    steps = 3
    hdr = np.array([sc.dt, *sc.box_min, *sc.box_max], dtype=np.float32)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(hdr.tobytes())
        f.write(sc.particles.tobytes())
    r = subprocess.run([demo, str(fin), str(fout), str(steps), mode], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert ("steps %d particles %d" % (steps, sc.n)) in r.stdout
    got = np.fromfile(fout, dtype=PARTICLE_DTYPE)

    want = sc.particles.copy()
    s = PBFSolver(sc.n, PBFConfig(), LambdaCorrParams())
    for _ in range(steps):
        s.step_host(want, sc.dt, sc.box_min, sc.box_max)
    s.close()
    assert got.shape == want.shape
    assert got.tobytes() == want.tobytes()
