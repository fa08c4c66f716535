"""Headless point-splat renderer (akua_splat_*) against its host restatement
(oracle/splat_oracle.py), and the camera matrices against lookAt/perspective written out here."""
import numpy as np
import pytest

import akuaengine_gb300 as ak
from akuaengine_gb300 import scene
from akuaengine_gb300.render import Camera, SplatRenderer, write_ppm


@pytest.fixture(scope="module")
def lib():
    from akuaengine_gb300 import build as _build

    _build.build_library()
    return ak.load_library()


def _look_at(eye, centre, up):
    f = centre - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = [-s @ eye, -u @ eye, f @ eye]
    return m


def _perspective(fovy_deg, aspect, zn, zf):
    t = np.tan(np.radians(fovy_deg) / 2)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = 1 / (aspect * t), 1 / t
    m[2, 2], m[2, 3], m[3, 2] = -(zf + zn) / (zf - zn), -2 * zf * zn / (zf - zn), -1
    return m


def test_camera_matrices(lib):
    cam = Camera(position=(1.0, 2.5, 7.0), gaze=(0.3, -0.4, -1.0), fovDegrees=50.0)
    v, p, vp = cam.matrices(16 / 9)
    eye = np.array(cam.position)
    v_ref = _look_at(eye, eye + np.array(cam.gaze), np.array(cam.up))
    p_ref = _perspective(50.0, 16 / 9, 0.1, 160.0)
    assert np.allclose(v, v_ref, atol=1e-6)
    assert np.allclose(p, p_ref, rtol=1e-6, atol=1e-6)
    assert np.allclose(vp, p_ref @ v_ref, rtol=1e-5, atol=1e-5)


def test_write_ppm(tmp_path):
    img = np.zeros((3, 5, 4), np.uint8)
    img[1, 2] = (10, 20, 30, 255)
    write_ppm(tmp_path / "a.ppm", img)
    data = (tmp_path / "a.ppm").read_bytes()
    assert data.startswith(b"P6\n5 3\n255\n")
    body = np.frombuffer(data[len(b"P6\n5 3\n255\n"):], np.uint8).reshape(3, 5, 3)
    assert tuple(body[1, 2]) == (10, 20, 30)


@pytest.mark.gpu
@pytest.mark.parametrize("cam", [Camera(), Camera(position=(5.5, 3.5, 5.0), gaze=(-0.6, -0.4, -0.7),
                                                  fovDegrees=60.0)])
def test_render_matches_restatement(cuda_lib, tmp_path, cam):
    import torch

    from oracle import splat_oracle

    sc = scene.reference_dam_break()
    p = sc.particles.copy()
    rng = np.random.default_rng(0)
    p["color"] = rng.uniform(0.2, 1.0, (sc.n, 4)).astype(np.float32)  # tell particles apart
    p["size"][::7] = 120.0                                            # some large splats
    w, h = 320, 180
    r = SplatRenderer(w, h)
    buf = torch.from_numpy(p.view(np.uint8).copy()).cuda()
    got = r.render(buf, cam).cpu().numpy()
    r.close()
    _, _, vp = cam.matrices(w / h)
    want = splat_oracle.render(p, vp, cam.position, w, h)
    diff = np.abs(got.astype(int) - want.astype(int)).max(-1)
    covered = (want != splat_oracle._u8(splat_oracle.CLEAR)).any(-1).mean()
    print("covered %.3f, pixels off by >1: %d, max diff %d" % (covered, (diff > 1).sum(), diff.max()))
    write_ppm(tmp_path / "frame.ppm", got)
    assert covered > 0.05
    assert (diff > 1).sum() <= 3
