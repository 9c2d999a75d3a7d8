"""The reference's preset (params_init), the animation driver's camera path
(scale.pl) and the front-ends' output files, on the host: bit-exact against
the fixtures the reference's own host build produced (tests/golden)."""
import os

import numpy as np
import pytest

capi = pytest.importorskip("lyapunov3d_gb300.capi", reason="library not built")
from lyapunov3d_gb300.types import (LyapCam, LyapCamD, LyapLight, LyapLightD, LyapParams,  # noqa: E402
                                    LyapParamsD, struct_to_bytes, POINT_DTYPE)


@pytest.mark.parametrize("double", [False, True])
def test_params_init_bit_exact(golden, double):
    meta, g = golden
    prm, cam, lights, seq, (w, h) = capi.params_init(double)
    sfx = "_d" if double else ""
    assert struct_to_bytes(prm) == g["preset_prm" + sfx].tobytes()
    assert struct_to_bytes(cam) == g["preset_cam" + sfx].tobytes()
    assert b"".join(struct_to_bytes(l) for l in lights) == g["preset_lights" + sfx].tobytes()
    p = meta["preset"]
    assert seq == p["seq"] and len(lights) == p["n_lights"] and (w, h) == (p["width"], p["height"])


@pytest.mark.parametrize("double", [False, True])
def test_anim_camera_at_one_is_the_preset(double):
    """params.cu is scale.pl's template with the eased value 1."""
    _, cam, _, _, _ = capi.params_init(double)
    c = capi.anim_camera(1.0, cam, double)
    assert struct_to_bytes(c) == struct_to_bytes(cam)


def test_anim_camera_path():
    """The path moves the camera on the unit sphere around (4-0.9i, 4-0.9i, 4-0.9i), i the
    eased value, while its direction swings 40 degrees about a fixed axis."""
    _, cam, _, _, _ = capi.params_init()
    ts, t = [], 0.0
    while t <= 1.00001:          # scale.pl:15
        ts.append(t)
        t += 0.01
    assert len(ts) == 101
    eased = [capi.ease_in_out_quart(t, 0.0, 1.0, 1.0) for t in ts]
    cams = [capi.anim_camera(i, cam) for i in eased]
    C = np.array([[c.C.x, c.C.y, c.C.z] for c in cams], dtype=np.float64)
    Q = np.array([[c.Q.x, c.Q.y, c.Q.z, c.Q.w] for c in cams])
    centre = 4.0 - 0.9 * np.array(eased)
    assert np.all(np.isfinite(C)) and np.all(np.isfinite(Q))
    assert np.allclose(np.linalg.norm(C - centre[:, None], axis=1), 1.0, atol=1e-5)
    off = C - centre[:, None]
    cosang = float(off[0] @ off[-1])
    assert abs(np.degrees(np.arccos(cosang)) - 40.0) < 1e-3
    assert np.all(np.diff(eased) >= 0)


def test_ease_in_out_quart_values():
    e = capi.ease_in_out_quart
    assert e(0.0, 0, 1, 1) == 0.0 and e(1.0, 0, 1, 1) == 1.0 and e(0.5, 0, 1, 1) == 0.5
    assert e(0.25, 0, 1, 1) == 0.125 and e(0.75, 0, 1, 1) == 0.875     # quadratic in and out
    assert e(0.5, 2.0, 4.0, 2.0) == 2.5


def test_write_ppm_p3_format(tmp_path):
    rgba = np.zeros((2, 3, 4), np.uint8)
    rgba[0, 0] = (1, 2, 3, 4)
    rgba[1, 2] = (255, 128, 7, 0)
    p = tmp_path / "a.ppm"
    capi.write_ppm(str(p), rgba)
    txt = p.read_bytes().decode()
    px = ["  1   2   3 ", "  0   0   0 ", "  0   0   0 ", "  0   0   0 ", "  0   0   0 ", "255 128   7 "]
    assert txt == "P3\n3 2\n255\n" + "".join(px) + "\n"
    capi.write_ppm(str(p), rgba, binary=True)
    raw = p.read_bytes()
    assert raw.startswith(b"P6\n3 2\n255\n")
    assert np.array_equal(np.frombuffer(raw[len(b"P6\n3 2\n255\n"):], np.uint8).reshape(2, 3, 3), rgba[..., :3])


def test_write_points_and_exps_raw(tmp_path):
    pts = np.zeros(5, POINT_DTYPE)
    pts["l"] = np.arange(5)
    pts["P"][3] = (1.5, -2.0, 3.25)
    capi.write_points(str(tmp_path / "p.raw"), pts)
    back = np.fromfile(tmp_path / "p.raw", dtype=POINT_DTYPE)
    assert back.tobytes() == pts.tobytes() and os.path.getsize(tmp_path / "p.raw") == 5 * 36
    v = np.linspace(-1, 1, 64 ** 3).astype(np.float32).reshape(64, 64, 64)
    capi.write_exps(str(tmp_path / "exps.raw"), v)
    assert np.array_equal(np.fromfile(tmp_path / "exps.raw", np.float32), v.ravel())
    with pytest.raises(capi.LyapError):
        capi.write_exps(str(tmp_path / "no" / "such" / "dir.raw"), v)


def test_output_name_convention():
    prm, cam, _, seq, (w, h) = capi.params_init()
    name = capi.output_name("Render", 1526604923, 8192, 8192, seq, cam, prm, 44 * 3600 + 54 * 60 + 12, "ppm")
    assert name.startswith("Render_1526604923_8192x8192_BCABA_cx=")
    assert name.endswith("_step=2_D=2.1_i=18,1008_d=4096_j=0.5_r=32_ot=-0.75_time=44h54m12s.ppm")
    cx = float(name.split("_cx=")[1].split("_")[0])
    assert cx == pytest.approx(cam.C.x, rel=1e-7)
    long_seq = "AB" * 200
    n2 = capi.output_name("Points", 1, 1, 1, long_seq, cam, prm, 5, "raw")
    assert len(n2) == 254
