"""lyap_render_noalloc, the raymarch entry point that allocates nothing.

Some callers cannot allocate device memory on every call: devices or drivers
without stream-ordered memory pools (lyap_render's stream-ordered allocation
of its queue counter and ray list fails there), applications that own all
device memory, loops that must not risk an allocation failing mid-frame.  lyap_render_noalloc
takes its scratch from a static device array instead.  This test calls it
through the C ABI twice in a row (the second call must find the shared
counter reset, not left at the first call's final count) and compares every
output byte with lyap_render's: both launch the same kernel on the same
inputs, so the tolerance is exact equality, as for the other drop-in entry
points in test_gpu_parity.py.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one.
"""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame  # noqa: E402


@pytest.mark.parametrize("variant", [capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT])
def test_render_noalloc_matches_render(variant):
    assert torch.cuda.is_available(), "needs a CUDA device"
    dev = torch.device("cuda:0")
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev, counts=False, stats=False)
    f.run(variant)
    torch.cuda.synchronize()
    want_rgba = f.d_rgba.clone()
    want_pts = f.d_points.clone()
    for call in range(2):
        f.d_rgba.fill_(0x5A)
        f.d_points.fill_(12345.0)
        capi.render_noalloc(f.cam, f.prm, f.d_seq, f.seq.size, f.d_lights, len(f.lights), f.d_rgba, f.d_points,
                            f.width, f.height, ext=capi.LyapRenderExt(variant=variant, light_model=f.light_model))
        torch.cuda.synchronize()
        assert torch.equal(f.d_rgba, want_rgba), f"rgba differs on call {call + 1}"
        assert torch.equal(f.d_points.view(torch.int32), want_pts.view(torch.int32)), \
            f"points differ on call {call + 1}"


def test_render_noalloc_rejects_oversized_image():
    """Images beyond LYAP_MAX_PIXELS (the shared 32-bit counter's range) are refused before any GPU work."""
    wl = scenes.small_render(8)
    cam = capi.cam_recalculate(wl.cam, 8, 8, 1)
    with pytest.raises(capi.LyapError) as e:
        capi.render_noalloc(cam, wl.params, 0x1000, 4, 0x2000, 1, 0x3000, 0x4000, 65536, 65536)
    assert e.value.code == capi.LYAP_ERR_INVALID_ARG and "exceeds" in e.value.message
