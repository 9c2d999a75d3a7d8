"""The reference front-ends' command-line equivalents (lyapunov3d_gb300/cli):
they link and start on the host; on the GPU they write the reference's files
(exps.raw, the PPM image, the points dump) with the same contents as the C
ABI calls they wrap."""
import glob
import os
import subprocess

import numpy as np
import pytest

capi = pytest.importorskip("lyapunov3d_gb300.capi", reason="library not built")
from lyapunov3d_gb300.types import POINT_DTYPE  # noqa: E402

LIBDIR = os.path.dirname(capi.LIB_PATH)


def _bin(name):
    p = os.path.join(LIBDIR, name)
    if not os.path.exists(p):
        pytest.skip(f"{name} not built")
    return p


@pytest.mark.parametrize("name", ["lyap_calculate", "lyap_frame"])
def test_cli_links_and_prints_usage(name):
    r = subprocess.run([_bin(name), "--no-such-option"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage:" in r.stderr


@pytest.mark.gpu
def test_lyap_calculate_writes_the_volume(tmp_path):
    torch = pytest.importorskip("torch")
    out = tmp_path / "exps.raw"
    r = subprocess.run([_bin("lyap_calculate"), "--n", "48", "--out", str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Points size = %d" % (48 ** 3 * 4) in r.stdout
    got = np.fromfile(out, np.float32).reshape(48, 48, 48)
    prm, _, _, seq, _ = capi.params_init()
    want = capi.volume_host(48, 48, 48, prm, capi.seq_parse(seq))
    assert got.tobytes() == want.tobytes()


@pytest.mark.gpu
def test_lyap_frame_writes_image_and_points(tmp_path):
    pytest.importorskip("torch")
    r = subprocess.run([_bin("lyap_frame"), "--width", "96", "--height", "54", "--out-dir", str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ppm = glob.glob(str(tmp_path / "Render_*_96x54_BCABA_*_step=2_D=2.1_i=18,1008_d=4096_j=0.5_r=32_ot=-0.75_time=*.ppm"))
    raw = glob.glob(str(tmp_path / "Points_*_96x54_BCABA_*.raw"))
    assert len(ppm) == 1 and len(raw) == 1
    # the same frame through the C ABI
    prm, cam, lights, seq, _ = capi.params_init()
    cam = capi.cam_recalculate(cam, 96, 54, 1)
    lights = capi.lights_recalculate(lights)
    rgba, pts = capi.render_host(cam, prm, capi.seq_parse(seq), lights, 96, 54)
    txt = open(ppm[0]).read().split()
    assert txt[:4] == ["P3", "96", "54", "255"]
    img = np.array(txt[4:], dtype=np.uint8).reshape(54, 96, 3)
    assert np.array_equal(img, rgba[..., :3])
    assert np.fromfile(raw[0], POINT_DTYPE).reshape(54, 96).tobytes() == pts.tobytes()
