"""Pin the oracle: the C restatement (oracle/lyap_oracle.c) against fixtures
recorded from the reference's own code built as host C++
(tests/golden/make_golden.py).  CPU only."""
import ctypes

import numpy as np
import pytest

from lyapunov3d_gb300.types import (LyapCam, LyapCamD, LyapLight, LyapLightD, LyapParams, LyapParamsD,
                                    LyapPoint, LyapPointD, RGBA, POINT_DTYPE, struct_from_bytes)
from oracle import ORC_F64, ORC_REF, params_to_double

CAM_FIELDS = ["C", "Q", "M", "V", "S0", "SDX", "SDY", "textureWidth", "textureHeight", "renderWidth",
              "renderHeight", "renderDenominator", "lightInnerCone", "lightOuterCone", "lightRange",
              "ambient", "diffuseColor", "diffusePower", "specularColor", "specularPower",
              "specularHardness", "chaosColor"]
PRM_FIELDS = ["d", "settle", "accum", "stepMethod", "nearThreshold", "nearMultiplier", "opaqueThreshold",
              "chaosThreshold", "depth", "jitter", "refine", "gradient", "lMin", "lMax"]
PT_FIELDS = ["P", "N", "a", "c", "l"]


def _layout(cam, prm, pt):
    v = [ctypes.sizeof(cam), 16] + [getattr(cam, f).offset for f in CAM_FIELDS]
    v += [ctypes.sizeof(prm)] + [getattr(prm, f).offset for f in PRM_FIELDS]
    v += [ctypes.sizeof(pt)] + [getattr(pt, f).offset for f in PT_FIELDS]
    v += [ctypes.sizeof(RGBA)]
    return v


def test_struct_layouts_match_reference(golden):
    meta, _ = golden
    assert _layout(LyapCam, LyapParams, LyapPoint) == meta["layout_f32"]
    assert _layout(LyapCamD, LyapParamsD, LyapPointD) == meta["layout_f64"]


def test_sequence_parse(oracle, golden):
    meta, _ = golden
    for s, expect in meta["seq"].items():
        rc, got = oracle.seq_parse(s)
        assert rc == 0 and got.tolist() == expect, s
    # the reference exit(1)s on these (scene.cu:98-100); the oracle reports -2
    for bad in ["", "0", "AX", "A0", " A", "E"]:
        assert oracle.seq_parse(bad)[0] == -2, bad
    assert oracle.seq_parse("A9", cap=5)[0] == -6


def _eq_nan(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.array_equal(a, b) or bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def test_cam_and_lights_recalculate(oracle, golden):
    _, g = golden
    for i in range(g["cams_in"].shape[0]):
        cam = struct_from_bytes(LyapCam, g["cams_in"][i].tobytes())
        tw, th, td = (int(x) for x in g["cams_dims"][i])
        assert bytes(oracle.cam_recalculate(cam, tw, th, td)) == g["cams_out"][i].tobytes(), i
        camd = LyapCamD()
        for f in CAM_FIELDS:
            v = getattr(cam, f)
            if hasattr(v, "_fields_"):
                for k, _ in v._fields_:
                    setattr(getattr(camd, f), k, getattr(v, k))
            else:
                setattr(camd, f, v)
        assert bytes(oracle.cam_recalculate_d(camd, tw, th, td)) == g["cams_out_d"][i].tobytes(), i
    lights = [struct_from_bytes(LyapLight, r.tobytes()) for r in g["lights_in"]]
    out = oracle.lights_recalculate(lights)
    assert [bytes(l) for l in out] == [r.tobytes() for r in g["lights_out"]]


def test_lambda_bit_exact(oracle, golden):
    meta, g = golden
    for i, (s, settle, accum, _lo, _hi) in enumerate(meta["lam_cases"]):
        _, seq = oracle.seq_parse(s)
        pts = g[f"lam{i}_pts"]
        assert _eq_nan(oracle.lyap4d(ORC_REF, pts, settle, accum, seq), g[f"lam{i}_f32"]), s
        assert _eq_nan(oracle.lyap4d(ORC_F64, pts, settle, accum, seq), g[f"lam{i}_f64"]), s


def test_volume_bit_exact(oracle, golden):
    _, g = golden
    prm = struct_from_bytes(LyapParams, g["vol32_prm"].tobytes())
    _, seq = oracle.seq_parse("ABC")
    v32 = oracle.volume(ORC_REF, 32, 32, 32, prm, seq)
    assert _eq_nan(v32, g["vol32_f32"])
    v64 = oracle.volume(ORC_F64, 32, 32, 32, params_to_double(prm), seq)
    assert _eq_nan(v64.astype(np.float32), g["vol32_f64"])


@pytest.mark.parametrize("case", ["preset64", "abc64", "inside48x32", "away32"])
def test_render_bit_exact(oracle, golden, case):
    meta, g = golden
    info = next(c for c in meta["render_cases"] if c["name"] == case)
    W, H = info["w"], info["h"]
    cam = struct_from_bytes(LyapCam, g[f"render_{case}_cam"].tobytes())
    prm = struct_from_bytes(LyapParams, g[f"render_{case}_prm"].tobytes())
    lights = [struct_from_bytes(LyapLight, r.tobytes()) for r in g[f"render_{case}_lights"]]
    _, seq = oracle.seq_parse(info["seq"])
    rgba, pts, cnt = oracle.render(ORC_REF, W, H, cam, prm, seq, lights)
    # points: identical bytes (a miss is all 0xFF in both: H3)
    assert np.array_equal(pts.view(np.uint8).reshape(H, W, 36), g[f"render_{case}_points"])
    # hit / miss as raymarch returns it
    rc = g[f"render_{case}_rc"]
    assert np.array_equal(np.isnan(pts["a"]), rc == 1)
    assert np.all(cnt[..., 2][rc == 0] == 6) and np.all(cnt[..., 2][rc == 1] == 0)
    # colours: identical bytes wherever the reference's conversion is in range (H6)
    col = g[f"render_{case}_color"].astype(np.float64) * 255.0
    in_range = np.all((col >= 0.0) & (col < 256.0), axis=-1)
    ref_rgba = g[f"render_{case}_rgba"]
    assert np.array_equal(rgba[in_range], ref_rgba[in_range])
    # out of range the oracle saturates
    sat = np.clip(np.floor(np.nan_to_num(col, nan=0.0)), 0, 255).astype(np.uint8)
    assert np.array_equal(rgba[~in_range], sat[~in_range])


def test_oracle_bounded_loops(oracle):
    """A negative near multiplier would make the reference march backwards
    forever; the oracle stops at its global bound and reports a miss."""
    from lyapunov3d_gb300 import scenes
    q = scenes.uniform_quaternion(scenes.SplitMix64(3))
    cam = oracle.cam_recalculate(scenes.orbit_camera(q, (2, 2, 2), 1.0), 8, 8, 1)
    prm = scenes.make_params(2, 3, step_method=1, depth=4.0, opaque=-50.0, near=100.0, near_mul=-1.0)
    _, seq = oracle.seq_parse("AB")
    rc, _, cnt = oracle.raymarch(ORC_REF, 4, 4, cam, prm, seq)
    assert rc == 1 and cnt[0] <= 4194304
