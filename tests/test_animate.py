"""The animation driver (scale.pl's camera sweep) on the batched renderer."""
import numpy as np
import pytest

capi = pytest.importorskip("lyapunov3d_gb300.capi", reason="library not built")
from lyapunov3d_gb300 import animate  # noqa: E402


def test_path_matches_scale_pl_loop():
    v = animate.path_values()
    assert len(v) == 101
    assert v[0] == (0.0, 0.0)
    t100, i100 = v[-1]
    assert abs(t100 - 1.0) < 1e-9 and abs(i100 - 1.0) < 1e-9
    assert all(b[1] >= a[1] for a, b in zip(v, v[1:]))


def test_dry_run_prints_t_and_i(capsys):
    assert animate.main(["-n", "--first", "2", "--last", "4"]) == 0
    lines = capsys.readouterr().out.strip().splitlines()
    assert len(lines) == 3 and lines[0].startswith("0.02\t")


def test_frame_cameras_follow_the_path():
    vals = animate.path_values()[::25]
    wls = animate.frame_workloads(32, 18, vals)
    for (t, i), wl in zip(vals, wls):
        c = capi.anim_camera(i)
        assert (wl.cam.C.x, wl.cam.C.y, wl.cam.C.z) == (c.C.x, c.C.y, c.C.z)
        assert wl.seq == "BCABA" and wl.params.accum == 1008


@pytest.mark.gpu
def test_batched_frames_equal_single_renders():
    pytest.importorskip("torch")
    vals = animate.path_values()[::40]
    wls, frames, _ = animate.render_path(64, 36, vals)
    for wl, f in zip(wls, frames):
        cam = capi.cam_recalculate(wl.cam, 64, 36, 1)
        rgba, pts = capi.render_host(cam, wl.params, capi.seq_parse(wl.seq), capi.lights_recalculate(wl.lights),
                                     64, 36)
        assert np.array_equal(f.rgba(), rgba)
        assert f.points().tobytes() == pts.tobytes()
