"""State files (akua_state_*): round trip, checksum, and (GPU) resuming a run bit for bit."""
import numpy as np
import pytest

import akuaengine_gb300 as ak
from akuaengine_gb300 import scene
from akuaengine_gb300.state import load_state, save_state, save_solver_state


@pytest.fixture(scope="module")
def lib():
    from akuaengine_gb300 import build as _build

    _build.build_library()
    return ak.load_library()


def test_header_layout(lib):
    import ctypes

    assert ctypes.sizeof(ak._abi.CStateHeader) == 256


def test_round_trip_with_sections(lib, tmp_path):
    sc = scene.workload("dam_break_27k", seed=3)
    cfg, corr = scene.benchmark_params()
    cfg.solverIterations = 3
    sums = np.random.default_rng(0).normal(0, 1e-4, sc.n).astype(np.float32)
    scenes = [{"numParticles": 10000, "gravity": (0, -7, 0), "box_min": (0, 0, 0),
               "box_max": (1, 2, 3)},
              {"numParticles": sc.n - 10000, "gravity": (0, -12, 0), "box_min": (0, 0, 0),
               "box_max": (4, 5, 6)}]
    path = tmp_path / "s.akua"
    save_state(path, sc.particles, cfg, corr, sc.box_min, sc.box_max, sc.dt, step=17,
               options=ak.OPT_EXACT_MATH, lambda_sums=sums, scenes=scenes)
    st = load_state(path)
    assert st.particles.tobytes() == sc.particles.tobytes()
    assert np.array_equal(st.lambda_sums, sums)
    for name in cfg.__dataclass_fields__:  # float fields are stored as float32
        assert np.array_equal(np.float32(getattr(st.config, name)), np.float32(getattr(cfg, name)))
    assert st.corr.k == np.float32(corr.k)
    assert st.step == 17 and st.options == ak.OPT_EXACT_MATH
    assert st.table_size == cfg.maxNeighbours * sc.n
    assert np.allclose(st.box_max, sc.box_max) and st.dt == np.float32(sc.dt)
    assert [d["numParticles"] for d in st.scenes] == [10000, sc.n - 10000]
    assert st.scenes[1]["gravity"] == (0.0, -12.0, 0.0)


def test_corruption_and_truncation_are_detected(lib, tmp_path):
    sc = scene.workload("dam_break_27k", seed=1)
    cfg, corr = scene.benchmark_params()
    path = tmp_path / "s.akua"
    save_state(path, sc.particles, cfg, corr, sc.box_min, sc.box_max, sc.dt)
    raw = bytearray(path.read_bytes())
    raw[256 + 1000] ^= 0x10
    bad = tmp_path / "bad.akua"
    bad.write_bytes(bytes(raw))
    with pytest.raises(ak.AkuaError) as e:
        load_state(bad)
    assert e.value.status == ak._abi.AKUA_ERR_CORRUPT
    short = tmp_path / "short.akua"
    short.write_bytes(bytes(raw[:256 + 500]))
    with pytest.raises(ak.AkuaError):
        load_state(short)
    notastate = tmp_path / "x.akua"
    notastate.write_bytes(b"\0" * 512)
    with pytest.raises(ak.AkuaError):
        load_state(notastate)


@pytest.mark.gpu
def test_resume_continues_bit_for_bit(cuda_lib, tmp_path):
    sc = scene.workload("dam_break_27k", seed=5)
    cfg, corr = scene.benchmark_params()
    straight = sc.particles.copy()
    with ak.PBFSolver(sc.n, cfg, corr) as s:
        for _ in range(6):
            s.step_host(straight, sc.dt, sc.box_min, sc.box_max)
    part = sc.particles.copy()
    with ak.PBFSolver(sc.n, cfg, corr) as s:
        for _ in range(3):
            s.step_host(part, sc.dt, sc.box_min, sc.box_max)
        save_solver_state(tmp_path / "mid.akua", s, sc.box_min, sc.box_max, sc.dt)
    st = load_state(tmp_path / "mid.akua")
    assert st.step == 3 and st.particles.tobytes() == part.tobytes()
    resumed = st.particles.copy()
    with ak.PBFSolver(st.particles.shape[0], st.config, st.corr) as s:
        for _ in range(3):
            s.step_host(resumed, st.dt, st.box_min, st.box_max)
    assert resumed.tobytes() == straight.tobytes()


@pytest.mark.gpu
def test_resume_with_lambda_sums(cuda_lib, tmp_path):
    """With lambda tracking on, the sums saved with the records make the resumed run's features
    (and so a warm start) identical."""
    import torch

    sc = scene.workload("dam_break_27k", seed=6)
    cfg, corr = scene.benchmark_params()

    def run(s, p, steps):
        for _ in range(steps):
            s.step_host(p, sc.dt, sc.box_min, sc.box_max)

    p1 = sc.particles.copy()
    with ak.PBFSolver(sc.n, cfg, corr) as s:
        s.set_lambda_tracking(True)
        run(s, p1, 3)
        f1 = torch.empty((sc.n, 8), device="cuda")
        t1 = torch.empty(sc.n, device="cuda")
        s.capture_training(f1, t1)
        run(s, p1, 1)
        s.synchronize()
    p2 = sc.particles.copy()
    with ak.PBFSolver(sc.n, cfg, corr) as s:
        s.set_lambda_tracking(True)
        run(s, p2, 3)
        save_solver_state(tmp_path / "m.akua", s, sc.box_min, sc.box_max, sc.dt,
                          with_lambda_sums=True)
    st = load_state(tmp_path / "m.akua")
    p3 = st.particles.copy()
    with ak.PBFSolver(sc.n, st.config, st.corr) as s:
        s.set_lambda_tracking(True)
        s.set_lambda_sums(st.lambda_sums)
        f2 = torch.empty((sc.n, 8), device="cuda")
        t2 = torch.empty(sc.n, device="cuda")
        s.capture_training(f2, t2)
        run(s, p3, 1)
        s.synchronize()
    assert p3.tobytes() == p1.tobytes()
    assert torch.equal(f1, f2) and torch.equal(t1, t2)
