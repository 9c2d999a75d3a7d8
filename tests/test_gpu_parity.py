"""GPU parity of the CUDA path against the oracle, through the C ABI.

Tolerances (stated per check):
  * the orbit iteration is bit-exact between the GPU and the oracle's
    emulation of the product's arithmetic (ORC_PLAIN / ORC_PRODUCT); only the
    logarithm differs (lg2.approx.f32 on the GPU, libm log2f in the oracle),
    so per-sample lambda agrees to LAM_TOL_PLAIN (absolute, accum <= 1000)
    and NaN positions agree exactly;
  * against the reference's own arithmetic (golden fixtures: double-promoted
    orbit, logf per step) lambda agrees to LAM_TOL_REF;
  * integer work -- pixel / voxel indexing, sample counts per ray, hit or
    miss -- is compared exactly wherever the lambda decisions agree, and the
    fraction of pixels whose decisions agree is asserted >= 99.9%.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame, DeviceVolume  # noqa: E402
from lyapunov3d_gb300.types import LyapCam, LyapLight, LyapParams, POINT_DTYPE, struct_from_bytes  # noqa: E402
from oracle import ORC_F64, ORC_PLAIN, ORC_PRODUCT, ORC_REF  # noqa: E402

LAM_TOL_PLAIN = 5e-5    # |lambda_gpu - lambda_oracle_plain|, accum <= 1000
LAM_TOL_PRODUCT = 5e-6  # |lambda_gpu - lambda_oracle_product| (one final log only)
LAM_TOL_REF = 1e-4      # |lambda_gpu_plain - lambda_reference_f32|, accum <= 1000


def _nan_equal_mask(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b))


def _maxdiff(a, b):
    f = np.isfinite(a) & np.isfinite(b)
    return float(np.max(np.abs(a[f].astype(np.float64) - b[f]))) if f.any() else 0.0


@pytest.fixture(scope="module")
def dev():
    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    return torch.device("cuda:0")


# ------------------------------------------------------------------ volume
@pytest.mark.parametrize("variant,mode,tol", [(capi.VARIANT_PLAIN, ORC_PLAIN, LAM_TOL_PLAIN),
                                              (capi.VARIANT_PRODUCT, ORC_PRODUCT, LAM_TOL_PRODUCT)])
def test_volume_64_vs_oracle(dev, oracle, variant, mode, tol):
    wl = scenes.small_volume(64)
    dv = DeviceVolume(wl, device=dev)
    dv.run(variant)
    got = dv.values()
    ref = oracle.volume(mode, 64, 64, 64, wl.params, dv.seq, lo=wl.lo, hi=wl.hi)
    assert _nan_equal_mask(got, ref)
    assert _maxdiff(got, ref) <= tol
    st = dv.stats()
    assert st[capi.STAT_SAMPLES] == 64 ** 3


@pytest.mark.parametrize("jit", [False, True])
def test_product_out_of_range_blocks_are_nan_without_redo(dev, oracle, jit):
    """Points just outside [2, 4] (r > 4: the orbit escapes to -inf) and
    orbits that land on 1/2 (a zero factor) give NaN in the plain form; the
    product form finds them NaN from its own state, with no plain redo
    (LYAP_STAT_FALLBACK stays 0), and otherwise matches the oracle."""
    prm = scenes.make_params(200, 1000)
    wl = scenes.VolumeWorkload("edge", (32, 32, 32), (1.95, 1.95, 1.95), (4.2, 4.2, 4.2), "AACACBACCAAB", prm)
    dv = DeviceVolume(wl, device=dev)
    dv.run(capi.VARIANT_PLAIN, jit=jit)
    plain = dv.values()
    dv.reset_stats()
    dv.run(capi.VARIANT_PRODUCT, jit=jit)
    prod = dv.values()
    st = dv.stats()
    ref = oracle.volume(ORC_PRODUCT, 32, 32, 32, prm, dv.seq, lo=wl.lo, hi=wl.hi)
    assert np.isnan(plain).mean() > 0.05
    assert _nan_equal_mask(prod, plain)
    assert _nan_equal_mask(prod, ref)
    assert _maxdiff(prod, ref) <= LAM_TOL_PRODUCT
    assert st[capi.STAT_FALLBACK] == 0


def test_volume_golden_reference(dev, golden):
    """kernel_calc_volume's 32^3 sweep over [0, 4) against the reference's own host build."""
    _, g = golden
    prm = struct_from_bytes(LyapParams, g["vol32_prm"].tobytes())
    seq = capi.seq_parse("ABC")
    d_seq = torch.from_numpy(seq).to(dev)
    out = torch.empty(32 ** 3, dtype=torch.float32, device=dev)
    capi.volume(out, 32, 32, 32, None, None, prm, d_seq, seq.size)
    got = out.cpu().numpy().reshape(32, 32, 32)
    ref = g["vol32_f32"]
    assert _nan_equal_mask(got, ref)
    assert _maxdiff(got, ref) <= LAM_TOL_REF
    # drop-in entry point with the reference's launch shape: identical bits
    out2 = torch.empty_like(out)
    capi.kernel_calc_volume((4, 4, 4), (8, 8, 8), out2, prm, d_seq)
    torch.cuda.synchronize()
    assert torch.equal(out.view(torch.int32), out2.view(torch.int32))


@pytest.mark.parametrize("seqstr", ["A", "AB", "ABC", "BCABA", "ABCD", "AAB3", "ABCABCA", "AB3C2", "A2B2C2D2",
                                    "ABCBCBABCBCB", "ABCDABCDABCDABC", "ABCDABCDABCDABCD", "ABCDABCDABCDABCDA",
                                    "A6B6C6D6A9B"])
@pytest.mark.parametrize("settle,accum", [(0, 1), (7, 9), (13, 40), (20, 100)])
def test_lambda_sequence_lengths(dev, oracle, seqstr, settle, accum):
    """Every unrolled period 1..16, the rolled remainders and the generic path (period > 16)."""
    seq = capi.seq_parse(seqstr)
    prm = scenes.make_params(settle, accum, d=3.3)
    wl = scenes.VolumeWorkload("t", (16, 8, 8), (2.0, 2.5, 3.0), (4.0, 3.9, 3.7), seqstr, prm)
    dv = DeviceVolume(wl, device=dev)
    for variant, mode, tol in [(capi.VARIANT_PLAIN, ORC_PLAIN, LAM_TOL_PLAIN),
                               (capi.VARIANT_PRODUCT, ORC_PRODUCT, LAM_TOL_PRODUCT)]:
        dv.run(variant)
        got = dv.values()
        ref = oracle.volume(mode, 16, 8, 8, prm, seq, lo=wl.lo, hi=wl.hi)
        assert _nan_equal_mask(got, ref), (seqstr, variant)
        assert _maxdiff(got, ref) <= tol, (seqstr, variant)


def test_lambda_edge_values(dev, oracle):
    """accum = 0 gives NaN; r = 0 (log 0) gives NaN; the superstable point r = 2 gives exactly 0."""
    seq = capi.seq_parse("A")
    for settle, accum, lo, hi in [(10, 0, 2.0, 4.0), (5, 20, 0.0, 4.0), (30, 50, 2.0, 2.0 + 2 ** -20)]:
        prm = scenes.make_params(settle, accum)
        wl = scenes.VolumeWorkload("e", (8, 2, 2), (lo, lo, lo), (hi, hi, hi), "A", prm)
        dv = DeviceVolume(wl, device=dev)
        for variant, mode in [(capi.VARIANT_PLAIN, ORC_PLAIN), (capi.VARIANT_PRODUCT, ORC_PRODUCT)]:
            dv.run(variant)
            got = dv.values()
            ref = oracle.volume(mode, 8, 2, 2, prm, seq, lo=wl.lo, hi=wl.hi)
            assert _nan_equal_mask(got, ref)
            assert np.array_equal(got == 0.0, ref == 0.0)
    prm = scenes.make_params(10, 0)
    dv = DeviceVolume(scenes.VolumeWorkload("e", (4, 4, 4), (2, 2, 2), (4, 4, 4), "AB", prm), device=dev)
    dv.run()
    assert np.isnan(dv.values()).all()


def test_volume_host_buffers_match_device(dev):
    wl = scenes.small_volume(32)
    dv = DeviceVolume(wl, device=dev)
    dv.run(capi.VARIANT_PRODUCT)
    host = capi.volume_host(32, 32, 32, wl.params, dv.seq, lo=wl.lo, hi=wl.hi,
                            ext=capi.LyapVolumeExt(variant=capi.VARIANT_PRODUCT))
    assert np.array_equal(host.view(np.int32), dv.values().view(np.int32))


# ------------------------------------------------------------------ render
def _compare_frames(got_rgba, got_pts, got_cnt, ref_rgba, ref_pts, ref_cnt, min_agree=0.999, exact_points=True):
    """Decisions (per-pixel sample counts) agree on >= min_agree of pixels; where
    they agree, hit/miss agree and the hit point is bit-identical (with
    jitter, the step length depends on the previous lambda, so there the
    hit point agrees to 1e-4 instead)."""
    agree = np.all(got_cnt == ref_cnt, axis=-1)
    frac = agree.mean()
    assert frac >= min_agree, f"decision agreement {frac:.5f}"
    gh, rh = ~np.isnan(got_pts["a"]), ~np.isnan(ref_pts["a"])
    assert np.array_equal(gh[agree], rh[agree])
    # miss pixels: all-NaN point bytes and RGBA 0 on both sides
    gb = got_pts.view(np.uint8).reshape(got_pts.shape + (36,))
    assert np.all(gb[~gh] == 0xFF)
    assert np.all(got_rgba[~gh] == 0)
    both = agree & gh
    if exact_points:
        assert np.array_equal(got_pts["P"][both], ref_pts["P"][both])
    else:
        assert np.max(np.abs(got_pts["P"][both] - ref_pts["P"][both]), initial=0.0) <= 1e-4
    return frac, both


@pytest.mark.parametrize("variant,mode", [(capi.VARIANT_PLAIN, ORC_PLAIN), (capi.VARIANT_PRODUCT, ORC_PRODUCT)])
def test_render_128_vs_oracle(dev, oracle, variant, mode):
    wl = scenes.small_render(128)
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(variant)
    rgba, pts, cnt = f.rgba(), f.points(), f.counts()
    r_rgba, r_pts, r_cnt = oracle.render(mode, 128, 128, f.cam, f.prm, f.seq, f.lights)
    frac, both = _compare_frames(rgba, pts, cnt, r_rgba, r_pts, r_cnt)
    # lambda at the hit (NaN counts as a hit, H7) and the normal: lambda
    # tolerance; colour bytes within 2
    assert _nan_equal_mask(pts["l"][both], r_pts["l"][both])
    assert _maxdiff(pts["l"][both], r_pts["l"][both]) <= LAM_TOL_PLAIN
    ndiff = np.nan_to_num(np.abs(pts["N"][both] - r_pts["N"][both]), nan=0.0).max(axis=-1)
    assert np.quantile(ndiff, 0.99) <= 1e-2
    cd = np.abs(rgba[both].astype(int) - r_rgba[both].astype(int)).max(axis=-1)
    assert np.quantile(cd, 0.99) <= 2
    # statistics agree with the per-pixel counts
    st = f.stats()
    assert st[capi.STAT_RAYS] == 128 * 128
    assert st[capi.STAT_SAMPLES] == cnt.sum()
    assert st[capi.STAT_MARCH] == cnt[..., 0].sum() and st[capi.STAT_HONE] == cnt[..., 1].sum()
    assert st[capi.STAT_HITS] == (~np.isnan(pts["a"])).sum()


@pytest.mark.parametrize("case", ["preset64", "abc64", "inside48x32", "away32"])
def test_render_golden_reference(dev, oracle, golden, case):
    """The reference's own renders (host build): the GPU's hit/miss agrees on
    >= 99.9% of pixels; without jitter the hit points are bit-identical to
    the reference's on >= 99.9% of the pixels both hit, with lambda within
    1e-4 there (jittered cases carry lambda differences of ~1e-6 into the
    step lengths, so their points are compared statistically below); the
    oracle with the GPU's arithmetic reproduces the GPU's decisions on
    >= 99.9%."""
    meta, g = golden
    info = next(c for c in meta["render_cases"] if c["name"] == case)
    W, H = info["w"], info["h"]
    cam = struct_from_bytes(LyapCam, g[f"render_{case}_cam"].tobytes())
    prm = struct_from_bytes(LyapParams, g[f"render_{case}_prm"].tobytes())
    lights = [struct_from_bytes(LyapLight, r.tobytes()) for r in g[f"render_{case}_lights"]]
    seq = capi.seq_parse(info["seq"])
    d_seq = torch.from_numpy(seq).to(dev)
    d_l = torch.from_numpy(capi.lights_array(lights)).to(dev)
    d_rgba = torch.empty(W * H * 4, dtype=torch.uint8, device=dev)
    d_pts = torch.empty(W * H * 9, dtype=torch.float32, device=dev)
    d_cnt = torch.zeros(W * H * 3, dtype=torch.int32, device=dev)
    capi.render(cam, prm, d_seq, seq.size, d_l, len(lights), d_rgba, d_pts, W, H,
                ext=capi.LyapRenderExt(d_counts=d_cnt.data_ptr()))
    rgba = d_rgba.cpu().numpy().reshape(H, W, 4)
    pts = d_pts.cpu().numpy().view(POINT_DTYPE).reshape(H, W)
    cnt = d_cnt.cpu().numpy().reshape(H, W, 3).astype(np.uint32)
    ref_pts = g[f"render_{case}_points"].view(POINT_DTYPE).reshape(H, W)
    hit_agree = (np.isnan(pts["a"]) == np.isnan(ref_pts["a"])).mean()
    assert hit_agree >= 0.999, hit_agree
    if prm.jitter == 0.0:
        both = ~np.isnan(pts["a"]) & ~np.isnan(ref_pts["a"])
        same = both & np.all(pts["P"] == ref_pts["P"], axis=-1)
        assert same.sum() >= 0.999 * both.sum(), f"{same.sum()} of {both.sum()} hit points equal the reference's"
        gl, rl = pts["l"][same].astype(np.float64), ref_pts["l"][same].astype(np.float64)
        fin = np.isfinite(gl) & np.isfinite(rl)
        assert np.array_equal(np.isnan(gl), np.isnan(rl))
        if fin.any():
            assert float(np.max(np.abs(gl[fin] - rl[fin]))) <= 1e-4
    r_rgba, r_pts, r_cnt = oracle.render(ORC_PLAIN, W, H, cam, prm, seq, lights)
    if prm.jitter == 0.0:
        _compare_frames(rgba, pts, cnt, r_rgba, r_pts, r_cnt)
    else:
        # jitter steps by frac(lambda): a 1e-6 lambda difference moves every
        # later sample a little, so step counts may differ by one; hit / miss
        # must still agree and the hit points stay close
        gh, rh = ~np.isnan(pts["a"]), ~np.isnan(r_pts["a"])
        assert (gh == rh).mean() >= 0.999
        both = gh & rh
        dP = np.abs(pts["P"][both] - r_pts["P"][both]).max(axis=-1)
        assert np.median(dP) <= 1e-5 and np.quantile(dP, 0.9) <= 1e-2
    # the drop-in kernel with the reference's launch shape gives the same bytes
    d_rgba2, d_pts2 = torch.empty_like(d_rgba), torch.empty_like(d_pts)
    capi.kernel_calc_render((W // 16, H // 16), (16, 16), d_rgba2, d_pts2, cam, prm, d_seq, d_l, len(lights))
    torch.cuda.synchronize()
    assert torch.equal(d_rgba, d_rgba2)
    assert torch.equal(d_pts.view(torch.int32), d_pts2.view(torch.int32))


def test_render_host_buffers_match_device(dev):
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev)
    f.run(capi.VARIANT_PLAIN)
    rgba, pts = capi.render_host(f.cam, f.prm, f.seq, f.lights, 96, 96, ext=capi.LyapRenderExt())
    assert np.array_equal(rgba, f.rgba())
    assert np.array_equal(pts.view(np.uint8), f.points().view(np.uint8))


@pytest.mark.parametrize("w,h", [(1, 1), (1, 37), (37, 1), (37, 23), (200, 3)])
def test_render_odd_sizes(dev, oracle, w, h):
    wl = scenes.small_render(8)
    wl.width, wl.height = w, h
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PLAIN)
    r_rgba, r_pts, r_cnt = oracle.render(ORC_PLAIN, w, h, f.cam, f.prm, f.seq, f.lights)
    _compare_frames(f.rgba(), f.points(), f.counts(), r_rgba, r_pts, r_cnt, min_agree=1.0 if w * h < 1000 else 0.999)
    assert f.stats()[capi.STAT_RAYS] == w * h


def test_render_deterministic_and_launch_shape_independent(dev):
    wl = scenes.small_render(64)
    f = DeviceFrame(wl, device=dev)
    f.run(capi.VARIANT_PLAIN)
    a = (f.d_rgba.clone(), f.d_points.clone())
    for bps, tpb in [(1, 32), (2, 64), (8, 128)]:
        f.run(capi.VARIANT_PLAIN, blocks_per_sm=bps, threads_per_block=tpb)
        assert torch.equal(f.d_rgba, a[0]) and torch.equal(f.d_points.view(torch.int32), a[1].view(torch.int32))


def test_directional_light_model(dev, oracle):
    """LYAP_LIGHT_DIRECTIONAL: ambient + diffuse * clamp(N . -V) per light."""
    wl = scenes.small_render(32)
    wl.light_model = capi.LIGHT_DIRECTIONAL
    f = DeviceFrame(wl, device=dev)
    f.run(capi.VARIANT_PLAIN)
    pts, rgba = f.points(), f.rgba()
    hit = ~np.isnan(pts["a"])
    L = f.lights[0]
    nd = -(pts["N"][..., 0] * L.V.x + pts["N"][..., 1] * L.V.y + pts["N"][..., 2] * L.V.z)
    i = np.clip(nd, 0, 1)
    expect_r = np.clip(np.floor(255.0 * (L.diffuseColor.x * (i * L.diffusePower) + L.ambient.x)), 0, 255)
    assert np.max(np.abs(rgba[..., 0][hit].astype(int) - expect_r[hit].astype(int))) <= 1


@pytest.mark.parametrize("block", [(8, 8), (12, 12), (16, 8), (32, 8)])
def test_dropin_block_shapes_give_lyap_render_bytes(dev, block):
    """kernel_calc_render samples ahead only in blocks of whole warps (8x8,
    16x8, 32x8); a 12x12 block (144 threads) takes the one-sample loop.
    Either way every pixel gets lyap_render's bytes."""
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev)
    f.run(capi.VARIANT_PLAIN)
    d_rgba2, d_pts2 = torch.empty_like(f.d_rgba), torch.empty_like(f.d_points)
    capi.kernel_calc_render((96 // block[0], 96 // block[1]), block, d_rgba2, d_pts2, f.cam, f.prm, f.d_seq,
                            f.d_lights, len(f.lights))
    torch.cuda.synchronize()
    assert torch.equal(f.d_rgba, d_rgba2)
    assert torch.equal(f.d_points.view(torch.int32), d_pts2.view(torch.int32))
