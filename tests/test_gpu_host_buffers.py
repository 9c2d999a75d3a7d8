"""The host-buffer entry points with page-locked and pageable outputs.

lyap_volume_host stores straight into an output buffer that is page-locked
host memory mapped for the device (cudaHostAlloc, torch's pin_memory,
cudaHostRegister), with no staging buffer and no download; any other buffer
goes through a device copy.  lyap_render_host always stages its outputs in
device memory.  Every route must give the same bytes as the device-buffer
entry points, including buffers that start inside their allocation.  The
page-locked buffers are filled with a marker first, so a byte the kernels
did not write would show.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame, DeviceVolume  # noqa: E402
from lyapunov3d_gb300.types import POINT_DTYPE  # noqa: E402


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


def _pinned(shape, dtype, offset=0):
    """A page-locked numpy array (marker-filled) and the tensor that owns its memory;
    `offset` bytes into the allocation to exercise interior addresses."""
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    t = torch.empty(n + offset + 64, dtype=torch.uint8, pin_memory=True)
    raw = t.numpy()
    raw.fill(0x5A)
    return t, raw[offset:offset + n].view(dtype).reshape(shape)


def _same_bytes(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("variant", [capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT])
def test_render_host_pinned_outputs(dev, variant):
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev)
    f.run(variant, jit=True)
    torch.cuda.synchronize()
    ref_rgba, ref_pts = f.rgba(), f.points()
    W, H = wl.width, wl.height
    ext = capi.LyapRenderExt(variant=variant, light_model=f.light_model)
    # pageable: the staging copy
    rgba0, pts0 = capi.render_host(f.cam, f.prm, f.seq, f.lights, W, H, ext=ext)
    assert _same_bytes(rgba0, ref_rgba) and _same_bytes(pts0, ref_pts)
    # both outputs page-locked (one at an interior offset of its allocation)
    keep1, rgba1 = _pinned((H, W, 4), np.uint8)
    keep2, pts1 = _pinned((H, W), POINT_DTYPE, offset=36)
    capi.render_host(f.cam, f.prm, f.seq, f.lights, W, H, ext=ext, rgba=rgba1, points=pts1)
    assert _same_bytes(rgba1, ref_rgba) and _same_bytes(pts1, ref_pts)
    # page-locked image, pageable points
    keep3, rgba2 = _pinned((H, W, 4), np.uint8, offset=4)
    pts2 = np.empty((H, W), dtype=POINT_DTYPE)
    capi.render_host(f.cam, f.prm, f.seq, f.lights, W, H, ext=ext, rgba=rgba2, points=pts2)
    assert _same_bytes(rgba2, ref_rgba) and _same_bytes(pts2, ref_pts)
    # page-locked image without points (the points stay on the device)
    keep4, rgba3 = _pinned((H, W, 4), np.uint8)
    capi.render_host(f.cam, f.prm, f.seq, f.lights, W, H, ext=ext, rgba=rgba3, want_points=False)
    assert _same_bytes(rgba3, ref_rgba)
    # twice in a row into the same page-locked buffers
    capi.render_host(f.cam, f.prm, f.seq, f.lights, W, H, ext=ext, rgba=rgba1, points=pts1)
    assert _same_bytes(rgba1, ref_rgba) and _same_bytes(pts1, ref_pts)


def test_volume_host_pinned_output(dev):
    wl = scenes.small_volume(40)
    dv = DeviceVolume(wl, device=dev)
    dv.run(capi.VARIANT_PRODUCT, jit=True)
    torch.cuda.synchronize()
    ref = dv.values()
    ext = capi.LyapVolumeExt(variant=capi.VARIANT_PRODUCT)
    n = 40
    pageable = capi.volume_host(n, n, n, wl.params, dv.seq, lo=wl.lo, hi=wl.hi, ext=ext)
    keep, out = _pinned((n, n, n), np.float32, offset=8)
    capi.volume_host(n, n, n, wl.params, dv.seq, lo=wl.lo, hi=wl.hi, ext=ext, out=out)
    assert _same_bytes(pageable, ref) and _same_bytes(out, ref)
