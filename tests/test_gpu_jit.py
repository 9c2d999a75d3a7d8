"""The kernels specialised at run time to one sequence (NVRTC, lyap_jit.cpp)
against the precompiled kernels, through the C ABI.  Both run the same
arithmetic, so every output byte must be identical; a specialisation handed
a host sequence that does not match the device sequence must still produce
the device sequence's results (it detects the mismatch and evaluates
generically)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame, DeviceVolume  # noqa: E402


@pytest.fixture(scope="module")
def dev():
    assert torch.cuda.is_available()
    ok, info = capi.jit_info()
    assert ok, info
    return torch.device("cuda:0")


def _bits(t):
    return t.view(torch.int32) if t.dtype == torch.float32 else t


@pytest.mark.parametrize("seqstr,settle,accum", [("A", 20, 100), ("ABC", 20, 100), ("AB3C2", 13, 40),
                                                 ("ABCBCBABCBCB", 200, 1000), ("ABCDABCDABCDABCD", 7, 9),
                                                 ("A6B6C6D6", 30, 50)])
def test_volume_jit_matches_precompiled(dev, seqstr, settle, accum):
    prm = scenes.make_params(settle, accum, d=3.1)
    wl = scenes.VolumeWorkload("j", (40, 9, 7), (2.0, 2.5, 3.0), (4.0, 3.9, 3.7), seqstr, prm)
    dv = DeviceVolume(wl, device=dev)
    for variant in (capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT):
        dv.run(variant, jit=False)
        ref = dv.d_out.clone()
        st_ref = dv.stats()
        dv.reset_stats()
        dv.run(variant, jit=True, flags=capi.FLAG_REQUIRE_JIT)
        torch.cuda.synchronize()
        assert torch.equal(_bits(dv.d_out), _bits(ref)), (seqstr, variant)
        st = dv.stats()
        assert st[capi.STAT_SAMPLES] == 40 * 9 * 7
        dv.reset_stats()


@pytest.mark.parametrize("variant", [capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT])
def test_render_jit_matches_precompiled(dev, variant):
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(variant, jit=False)
    rgba, pts, cnt = f.d_rgba.clone(), f.d_points.clone(), f.d_counts.clone()
    f.run(variant, jit=True, flags=capi.FLAG_REQUIRE_JIT)
    torch.cuda.synchronize()
    assert torch.equal(f.d_rgba, rgba)
    assert torch.equal(_bits(f.d_points), _bits(pts))
    assert torch.equal(f.d_counts, cnt)


def test_stale_specialisation_is_safe(dev):
    """h_seq says ABC, the device holds BCA: results must be BCA's."""
    prm = scenes.make_params(20, 100)
    wl = scenes.VolumeWorkload("s", (32, 4, 4), (2.5, 2.5, 2.5), (4.0, 4.0, 4.0), "BCA", prm)
    dv = DeviceVolume(wl, device=dev)
    dv.run(capi.VARIANT_PRODUCT, jit=False)
    ref = dv.d_out.clone()
    wrong = capi.seq_parse("ABC")
    dv.run(capi.VARIANT_PRODUCT, jit=True, h_seq=wrong.ctypes.data, flags=capi.FLAG_REQUIRE_JIT)
    torch.cuda.synchronize()
    assert torch.equal(_bits(dv.d_out), _bits(ref))


def test_require_jit_errors(dev):
    prm = scenes.make_params(2, 3)
    wl = scenes.VolumeWorkload("r", (4, 4, 4), (2, 2, 2), (4, 4, 4), "AB", prm)
    dv = DeviceVolume(wl, device=dev)
    with pytest.raises(capi.LyapError) as e:   # no host sequence given
        capi.volume(dv.d_out, 4, 4, 4, wl.lo, wl.hi, prm, dv.d_seq, dv.seq.size,
                    ext=capi.LyapVolumeExt(flags=capi.FLAG_REQUIRE_JIT))
    assert e.value.code == capi.LYAP_ERR_JIT
    long_seq = capi.seq_parse("A9B9C9D9A")   # period 37 > 32: not specialised
    d_long = torch.from_numpy(long_seq).to(dev)
    with pytest.raises(capi.LyapError) as e:
        capi.volume(dv.d_out, 4, 4, 4, wl.lo, wl.hi, prm, d_long, long_seq.size,
                    ext=capi.LyapVolumeExt(flags=capi.FLAG_REQUIRE_JIT, h_seq=long_seq.ctypes.data))
    assert e.value.code == capi.LYAP_ERR_JIT and "period" in e.value.message
    # without REQUIRE it falls back to the precompiled kernels and still works
    capi.volume(dv.d_out, 4, 4, 4, wl.lo, wl.hi, prm, d_long, long_seq.size,
                ext=capi.LyapVolumeExt(h_seq=long_seq.ctypes.data))
    torch.cuda.synchronize()
    ok, info = capi.jit_info()
    assert "compiled=" in info


def test_host_entry_points_use_specialisation(dev):
    wl = scenes.small_render(48)
    f = DeviceFrame(wl, device=dev)
    f.run(capi.VARIANT_PRODUCT, jit=False)
    before = capi.jit_info()[1]
    rgba, pts = capi.render_host(f.cam, f.prm, f.seq, f.lights, 48, 48,
                                 ext=capi.LyapRenderExt(variant=capi.VARIANT_PRODUCT, flags=capi.FLAG_REQUIRE_JIT))
    assert np.array_equal(rgba, f.rgba())
    assert np.array_equal(pts.view(np.uint8), f.points().view(np.uint8))
    assert capi.jit_info()[1] != before


@pytest.mark.parametrize("jit", [False, True])
def test_speculation_changes_nothing(dev, jit):
    """Idle lanes sampling ahead for running rays: same pixels, same counts."""
    wl = scenes.small_render(64)
    wl.params.refine = 8.0   # honing on, so rays pass through march -> hone -> normal
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PRODUCT, jit=jit, flags=capi.FLAG_NO_SPECULATION)
    rgba, pts, cnt = f.d_rgba.clone(), f.d_points.clone(), f.d_counts.clone()
    st0 = f.stats()
    f.reset_stats()
    f.run(capi.VARIANT_PRODUCT, jit=jit)
    torch.cuda.synchronize()
    st1 = f.stats()
    assert torch.equal(f.d_rgba, rgba)
    assert torch.equal(_bits(f.d_points), _bits(pts))
    assert torch.equal(f.d_counts, cnt)
    assert st0[capi.STAT_SPEC] == 0 and st1[capi.STAT_SPEC] > 0
    assert st1[capi.STAT_SAMPLES] == st0[capi.STAT_SAMPLES]
    assert 0 < st1[capi.STAT_SPEC_USED] <= st1[capi.STAT_SPEC]


@pytest.mark.parametrize("jit", [False, True])
def test_spread_queue_order_changes_nothing(dev, jit):
    """The pixel queue's spread order against scanline order (default): same
    pixels, points, per-pixel counts and sample totals; the frame timing
    statistics are filled in both."""
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PRODUCT, jit=jit, flags=capi.FLAG_SPREAD_ORDER)
    rgba, pts, cnt = f.d_rgba.clone(), f.d_points.clone(), f.d_counts.clone()
    st0 = f.stats()
    f.reset_stats()
    f.d_counts.zero_()
    f.run(capi.VARIANT_PRODUCT, jit=jit)
    torch.cuda.synchronize()
    st1 = f.stats()
    assert torch.equal(f.d_rgba, rgba)
    assert torch.equal(_bits(f.d_points), _bits(pts))
    assert torch.equal(f.d_counts, cnt)
    assert st1[capi.STAT_SAMPLES] == st0[capi.STAT_SAMPLES]
    mask = (1 << 64) - 1
    for st in (st0, st1):
        t0, td, te = (~int(st[capi.STAT_T_START])) & mask, (~int(st[capi.STAT_T_DRAIN])) & mask, int(st[capi.STAT_T_END])
        assert 0 < t0 <= td <= te


@pytest.mark.parametrize("jit", [False, True])
def test_speculation_changes_nothing_full_frame(dev, jit):
    """The 1080p bench frame with and without sampling ahead: the same pixels,
    points and per-pixel counts.  The frame has rays that walk the hone cap
    (grazing rays, sampled ahead in the hone phase) and rays in every phase
    at the end of the frame."""
    wl = scenes.full_render(1, 1920, 1080)
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PRODUCT, jit=jit, flags=capi.FLAG_NO_SPECULATION)
    rgba, pts, cnt = f.d_rgba.clone(), f.d_points.clone(), f.d_counts.clone()
    f.reset_stats()
    f.d_counts.zero_()
    f.run(capi.VARIANT_PRODUCT, jit=jit)
    torch.cuda.synchronize()
    st = f.stats()
    assert torch.equal(f.d_rgba, rgba)
    assert torch.equal(_bits(f.d_points), _bits(pts))
    assert torch.equal(f.d_counts, cnt)
    hone = f.counts()[..., 1]
    assert (hone == 256).sum() > 0 and hone.max() == 256
    assert st[capi.STAT_SPEC_USED] > 0
