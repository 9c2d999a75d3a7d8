"""The DOUBLE_REALS render mode: host camera/light preparation bit-exact
against the reference's own DOUBLE_REALS host build (tests/golden), and the
GPU render against the FP64 oracle (orc_raymarch_d)."""
import ctypes

import numpy as np
import pytest

capi = pytest.importorskip("lyapunov3d_gb300.capi", reason="library not built")
from lyapunov3d_gb300 import scenes  # noqa: E402
from lyapunov3d_gb300.types import (LyapCamD, LyapLightD, LyapParamsD, LyapPointD, struct_from_bytes,  # noqa: E402
                                    struct_to_bytes)


def test_cam_and_lights_recalculate_d_bit_exact(golden):
    _, g = golden
    for i in range(g["cams_in"].shape[0]):
        # the fixtures' input cameras are float structs; the DOUBLE_REALS build read the same values
        from lyapunov3d_gb300.types import LyapCam
        c32 = struct_from_bytes(LyapCam, g["cams_in"][i].tobytes())
        cd = LyapCamD()
        for f in ("C", "Q", "V", "S0", "SDX", "SDY"):
            src, dst = getattr(c32, f), getattr(cd, f)
            for k, _ in src._fields_:
                setattr(dst, k, getattr(src, k))
        for f in ("M", "textureWidth", "textureHeight", "renderWidth", "renderHeight", "renderDenominator"):
            setattr(cd, f, getattr(c32, f))
        tw, th, td = (int(x) for x in g["cams_dims"][i])
        out = capi.cam_recalculate_d(cd, tw, th, td)
        assert struct_to_bytes(out) == g["cams_out_d"][i].tobytes(), i


def test_params_init_d_camera_recalculates_like_the_reference(golden):
    _, g = golden
    prm, cam, lights, seq, (w, h) = capi.params_init(double=True)
    c = capi.cam_recalculate_d(cam, 64, 64, 1)
    assert np.isfinite([c.S0.x, c.SDX.x, c.SDY.y]).all()
    L = capi.lights_recalculate_d(lights)
    assert abs(L[0].V.x ** 2 + L[0].V.y ** 2 + L[0].V.z ** 2 - 1.0) < 1e-12


def _dparams(p32):
    d = LyapParamsD()
    for name, _ in p32._fields_:
        setattr(d, name, getattr(p32, name))
    return d


def _dcam(c32, w, h):
    cd = LyapCamD()
    for f in ("C", "Q"):
        src, dst = getattr(c32, f), getattr(cd, f)
        for k, _ in src._fields_:
            setattr(dst, k, getattr(src, k))
    cd.M = c32.M
    cd.renderDenominator = 1
    return capi.cam_recalculate_d(cd, w, h, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["abc", "preset", "preset_jitter"])
def test_render_d_matches_fp64_oracle(oracle, case):
    """Without jitter every pixel matches the FP64 oracle (positions and
    lambda within 1e-9, sample counts equal) but for decisions within ~1e-13
    of a threshold.  With jitter (the preset's 0.5) each step length depends
    on frac(lambda), so the 1e-13 difference between the GPU's renormalised
    log sum and the oracle's per-step log moves the next sample, and the
    chaotic orbit turns that into a different lambda a few samples on: there
    the check is statistical (hits agree, most points close)."""
    torch = pytest.importorskip("torch")
    w, h = 40, 24
    if case == "abc":
        wl = scenes.small_render(w)
        prm, seq, light_model = _dparams(wl.params), capi.seq_parse(wl.seq), wl.light_model
        cam = _dcam(wl.cam, w, h)
        lights = capi.lights_recalculate_d([_light_d(l) for l in wl.lights])
    else:
        prm, cam0, lights0, s, _ = capi.params_init(double=True)
        prm.accum, prm.depth = 200, 192.0     # lighter than the preset's 1008 / 4096
        if case == "preset":
            prm.jitter = 0.0
        seq, light_model = capi.seq_parse(s), capi.LIGHT_SPOT
        cam = capi.cam_recalculate_d(cam0, w, h, 1)
        lights = capi.lights_recalculate_d(lights0)
    n = w * h
    d_seq = torch.from_numpy(seq).cuda()
    la = (LyapLightD * len(lights))(*lights)
    d_l = torch.from_numpy(np.frombuffer(bytes(la), np.uint8).copy()).cuda()
    d_rgba = torch.empty(n * 4, dtype=torch.uint8, device="cuda")
    d_pts = torch.empty(n * 9, dtype=torch.float64, device="cuda")
    d_cnt = torch.empty(n * 3, dtype=torch.int32, device="cuda")
    capi.render_d(cam, prm, d_seq, seq.size, d_l, len(lights), d_rgba, d_pts, w, h, light_model, d_cnt)
    torch.cuda.synchronize()
    pts = d_pts.cpu().numpy().reshape(h, w, 9)
    cnt = d_cnt.cpu().numpy().reshape(h, w, 3)
    agree = same = close = 0
    for y in range(h):
        for x in range(w):
            rc, pt, c = oracle.raymarch_d(x, y, cam, prm, seq)
            ghit = not np.isnan(pts[y, x, 0])
            if ghit == (rc == 0):
                agree += 1
            if rc == 0 and ghit:
                ref = np.array([pt.P.x, pt.P.y, pt.P.z, pt.l])
                if np.allclose(pts[y, x, [0, 1, 2, 8]], ref, rtol=0, atol=1e-9) and tuple(cnt[y, x]) == c:
                    same += 1
                if np.abs(pts[y, x, :3] - ref[:3]).max() < 0.05:
                    close += 1
            elif rc != 0 and not ghit:
                same += 1
                close += 1
    if case == "preset_jitter":
        assert agree / n >= 0.98 and close / n >= 0.9, (agree / n, close / n)
    else:
        assert agree / n >= 0.995 and same / n >= 0.99, (agree / n, same / n)
    assert (d_rgba.cpu().numpy().reshape(h, w, 4)[np.isnan(pts[..., 0])] == 0).all()


def _light_d(l32):
    d = LyapLightD()
    for f, _ in type(l32)._fields_:
        v = getattr(l32, f)
        if hasattr(v, "_fields_"):
            dv = getattr(d, f)
            for k, _ in v._fields_:
                setattr(dv, k, getattr(v, k))
        elif not f.startswith("_"):
            setattr(d, f, v)
    return d


def test_lights_recalculate_d_bit_exact(golden):
    _, g = golden
    from lyapunov3d_gb300.types import LyapLight
    lights = [_light_d(struct_from_bytes(LyapLight, r.tobytes())) for r in g["lights_in"]]
    out = capi.lights_recalculate_d(lights)
    assert [struct_to_bytes(l) for l in out] == [r.tobytes() for r in g["lights_out_d"]]
