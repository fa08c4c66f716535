"""CPU tests of the C ABI: the library builds and loads, exports every symbol the header declares,
and the ctypes mirror matches the header's structs.  No call here reaches the GPU."""
import ctypes
import os
import re

import pytest

import akuaengine_gb300 as ak
from akuaengine_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "akua_pbf.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(akua_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(cuda_lib):
    names = header_functions()
    assert len(names) >= 17
    for name in names:
        assert hasattr(cuda_lib, name), name
    assert sorted(_abi.exported_symbols()) == names


def test_abi_version_and_status_strings(cuda_lib):
    assert cuda_lib.akua_pbf_abi_version() == 1
    assert _abi.status_string(0) == "ok"
    assert "argument" in _abi.status_string(ak.AKUA_ERR_INVALID_ARGUMENT)
    assert _abi.status_string(12345) == "unknown status"


def test_struct_layouts_match_header(cuda_lib):
    assert ctypes.sizeof(_abi.CConfig) == 48
    assert ctypes.sizeof(_abi.CCorr) == 16
    assert ak.PARTICLE_DTYPE.itemsize == 108
    offs = {name: ak.PARTICLE_DTYPE.fields[name][1] for name in ak.PARTICLE_DTYPE.names}
    # Particle.h:8-31 offsets, measured on the reference's layout with glm vec3/vec4 of floats
    assert offs == {"position": 0, "velocity": 12, "new_position": 24, "new_velocity": 36,
                    "position_delta": 48, "vorticity": 60, "mass": 72, "density": 76,
                    "lambda": 80, "hash": 84, "color": 88, "size": 104}


def test_default_config_matches_reference(cuda_lib):
    c, k = _abi.CConfig(), _abi.CCorr()
    cuda_lib.akua_pbf_default_config(ctypes.byref(c), ctypes.byref(k))
    py = ak.PBFConfig()
    assert c.restDensity == py.restDensity == 7600.0
    assert c.maxNeighbours == 128 and c.solverIterations == 4
    assert abs(c.smoothRadius - 0.1) < 1e-7 and abs(c.relaxation - 600.0) < 1e-6
    assert list(c.gravity) == pytest.approx([0.0, -9.8, 0.0])
    assert k.enabled == 1 and k.n == 4.0
    assert abs(k.k - 1e-4) < 1e-9 and abs(k.delta_q - 0.03) < 1e-8


def test_invalid_arguments_rejected_before_any_device_call(cuda_lib):
    c, k = _abi.CConfig(), _abi.CCorr()
    cuda_lib.akua_pbf_default_config(ctypes.byref(c), ctypes.byref(k))
    h = ctypes.c_void_p()
    assert cuda_lib.akua_pbf_create(0, ctypes.byref(c), ctypes.byref(k), ctypes.byref(h)) == -1
    assert cuda_lib.akua_pbf_create(-5, ctypes.byref(c), ctypes.byref(k), ctypes.byref(h)) == -1
    assert cuda_lib.akua_pbf_create(10, None, ctypes.byref(k), ctypes.byref(h)) == -1
    c.maxNeighbours = 0
    assert cuda_lib.akua_pbf_create(10, ctypes.byref(c), ctypes.byref(k), ctypes.byref(h)) == -1
    c.maxNeighbours = 128
    # PBFSolver.cpp:15 keeps the table size in an int: maxNeighbours * N must fit
    assert cuda_lib.akua_pbf_create(2**25, ctypes.byref(c), ctypes.byref(k),
                                    ctypes.byref(h)) == ak.AKUA_ERR_TOO_LARGE
    assert cuda_lib.akua_pbf_step(None, 0.01, _abi.vec3((0, 0, 0)), _abi.vec3((1, 1, 1))) == -1
    assert cuda_lib.akua_pbf_destroy(None) == -1


def test_product_path_does_not_import_the_oracle():
    """The package must not reach the test oracle (no CPU fallback)."""
    pkg = os.path.join(ROOT, "akuaengine_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
                assert "liboracle" not in src, f


def test_missing_library_fails_loudly(tmp_path):
    import importlib

    mod = importlib.import_module("akuaengine_gb300._abi")
    saved = mod._lib
    try:
        mod._lib = None
        with pytest.raises(RuntimeError, match="not built"):
            mod.load_library(str(tmp_path / "nope.so"))
    finally:
        mod._lib = saved
