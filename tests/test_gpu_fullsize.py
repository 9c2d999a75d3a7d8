"""Parity at the benchmark's full sizes, through the C ABI.

The benchmark frame (1920x1080, 512 steps per ray, 12-symbol sequence,
200 + 1000 iterations) and the 512^3 volume are too large for the oracle to
recompute whole in a test, so they are checked by seeded samples and by
size-independent properties:
  * frame: 64 seeded rows of the GPU frame against the oracle's rows -- the
    drop-in (plain, precompiled kernel) against ORC_PLAIN and the chosen
    form (product, kernel compiled for the sequence at run time) against
    ORC_PRODUCT.  Per-pixel decisions (march / honing / normal sample
    counts) equal on >= 99.9 % of the sampled pixels, and where they are
    equal the hit point is bit-identical and lambda at the hit agrees to the
    lambda tolerance below;
  * the same frame's chosen form against the REFERENCE'S OWN arithmetic
    (ORC_REF: double-promoted orbit, logf per step; the restatement is
    pinned bit-exact to the reference's host build) on 64 seeded rows:
    per-pixel decisions equal on >= 99.9 %, hit / miss equal on >= 99.9 %,
    hit points bit-identical and lambda within 1e-4 where decisions agree;
    and lambda at the GPU's hit points against FP64 (ORC_F64), where the
    chosen form's error equals the reference arithmetic's own FP32 error
    to within 1e-4 at >= 99.9 % of the hit points;
  * volume: lambda at 8192 seeded voxels against the oracle (same voxel
    coordinates, float32 arithmetic as the kernel), NaN positions exact,
    against the reference's arithmetic (within 1e-4) and against FP64 (the
    same error as the reference arithmetic's, within 1e-4, per voxel);
    over all 134 M voxels the sweep is deterministic and the run-time
    specialised kernel is bit-identical to the precompiled one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame, DeviceVolume  # noqa: E402
from oracle import ORC_F64, ORC_PLAIN, ORC_PRODUCT, ORC_REF  # noqa: E402

LAM_TOL = {ORC_PLAIN: 5e-5, ORC_PRODUCT: 5e-6}   # |lambda_gpu - lambda_oracle|, accum <= 1000
# |lambda_gpu - lambda of the reference's arithmetic|: the orbits agree, only
# the logarithm differs (lg2.approx / renormalised product vs logf per step)
REF_TOL = 1e-4
ROWS = 64
VOXELS = 8192


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.fixture(scope="module")
def frame_wl():
    return scenes.full_render(1)


@pytest.mark.parametrize("variant,mode,jit", [(capi.VARIANT_PLAIN, ORC_PLAIN, False),
                                              (capi.VARIANT_PRODUCT, ORC_PRODUCT, True)])
def test_full_frame_rows_vs_oracle(dev, oracle, frame_wl, variant, mode, jit):
    wl = frame_wl
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(variant, jit=jit)
    torch.cuda.synchronize()
    rgba, pts, cnt = f.rgba(), f.points(), f.counts()
    st = f.stats()
    # whole-frame consistency of the kernel's statistics with its per-pixel counts
    assert st[capi.STAT_RAYS] == wl.width * wl.height
    assert st[capi.STAT_MARCH] == cnt[..., 0].sum() and st[capi.STAT_HONE] == cnt[..., 1].sum()
    assert st[capi.STAT_HITS] == (~np.isnan(pts["a"])).sum()
    rows = np.sort(np.random.default_rng(20261204 + variant).choice(wl.height, ROWS, replace=False))
    agree_n = total = 0
    for y in rows:
        r_rgba, r_pts, r_cnt = oracle.render(mode, wl.width, wl.height, f.cam, f.prm, f.seq, f.lights,
                                             y0=int(y), y1=int(y) + 1)
        g_pts, g_cnt = pts[y:y + 1], cnt[y:y + 1]
        agree = np.all(g_cnt == r_cnt, axis=-1)
        agree_n += int(agree.sum())
        total += agree.size
        gh, rh = ~np.isnan(g_pts["a"]), ~np.isnan(r_pts["a"])
        assert np.array_equal(gh[agree], rh[agree]), f"row {y}: hit/miss differ where decisions agree"
        both = agree & gh
        assert np.array_equal(g_pts["P"][both], r_pts["P"][both]), f"row {y}: hit points differ"
        gl, rl = g_pts["l"][both], r_pts["l"][both]
        assert np.array_equal(np.isnan(gl), np.isnan(rl))
        fin = np.isfinite(gl) & np.isfinite(rl)
        if fin.any():
            assert float(np.max(np.abs(gl[fin].astype(np.float64) - rl[fin]))) <= LAM_TOL[mode]
        # misses: all-NaN point bytes and a zero pixel
        gb = g_pts.view(np.uint8).reshape(g_pts.shape + (36,))
        assert np.all(gb[~gh] == 0xFF) and np.all(rgba[y:y + 1][~gh] == 0)
    frac = agree_n / total
    assert frac >= 0.999, f"decisions agree on {frac:.5f} of {total} sampled pixels"


def test_full_frame_rows_vs_reference_arithmetic(dev, oracle, frame_wl):
    """The chosen form (product, kernel compiled for the sequence) on the
    1080p frame against the reference's own FP32 arithmetic and against FP64."""
    wl = frame_wl
    f = DeviceFrame(wl, device=dev, counts=True, stats=False)
    f.run(capi.VARIANT_PRODUCT, jit=True)
    torch.cuda.synchronize()
    pts, cnt = f.points(), f.counts()
    rows = np.sort(np.random.default_rng(20261205).choice(wl.height, ROWS, replace=False))
    dec_n = hit_n = total = 0
    hit_P = []
    for y in rows:
        _, r_pts, r_cnt = oracle.render(ORC_REF, wl.width, wl.height, f.cam, f.prm, f.seq, f.lights,
                                        y0=int(y), y1=int(y) + 1)
        g_pts, g_cnt = pts[y:y + 1], cnt[y:y + 1]
        agree = np.all(g_cnt == r_cnt, axis=-1)
        gh, rh = ~np.isnan(g_pts["a"]), ~np.isnan(r_pts["a"])
        dec_n += int(agree.sum())
        hit_n += int((gh == rh).sum())
        total += agree.size
        both = agree & gh
        assert np.array_equal(gh[agree], rh[agree]), f"row {y}: hit/miss differ where decisions agree"
        assert np.array_equal(g_pts["P"][both], r_pts["P"][both]), f"row {y}: hit points differ"
        gl, rl = g_pts["l"][both], r_pts["l"][both]
        assert np.array_equal(np.isnan(gl), np.isnan(rl))
        fin = np.isfinite(gl) & np.isfinite(rl)
        if fin.any():
            err = float(np.max(np.abs(gl[fin].astype(np.float64) - rl[fin])))
            assert err <= REF_TOL, f"row {y}: lambda at hits differs from the reference arithmetic by {err}"
        hit_P.append(np.concatenate([g_pts["P"][gh].astype(np.float64), g_pts["l"][gh, None].astype(np.float64)], 1))
    assert dec_n / total >= 0.999, f"decisions agree with the reference arithmetic on {dec_n / total:.5f}"
    assert hit_n / total >= 0.999, f"hit / miss agree with the reference arithmetic on {hit_n / total:.5f}"
    # lambda at the GPU's hit points against FP64: in chaotic regions an FP32
    # orbit (the reference's too) decorrelates from the FP64 one, so the error
    # is bounded by the reference arithmetic's own, point by point
    H = np.concatenate(hit_P)
    assert len(H) > 1000
    q = np.concatenate([H[:, :3], np.full((len(H), 1), float(wl.params.d))], axis=1)
    l64 = oracle.lyap4d(ORC_F64, q, wl.params.settle, wl.params.accum, f.seq)
    lref = oracle.lyap4d(ORC_REF, q, wl.params.settle, wl.params.accum, f.seq)
    lgpu = H[:, 3]
    ok = np.isfinite(l64) & np.isfinite(lgpu) & np.isfinite(lref)
    assert (np.isnan(lgpu) == np.isnan(lref)).mean() >= 0.999
    e_gpu, e_ref = np.abs(lgpu[ok] - l64[ok]), np.abs(lref[ok] - l64[ok])
    assert float(np.median(e_gpu)) <= 1e-5
    # (a hit point whose march decisions differed from the reference's can sit
    # in a chaotic region where the two FP32 orbits part: 99.9 %, not all)
    assert (np.abs(e_gpu - e_ref) <= REF_TOL).mean() >= 0.999


def _voxel_coords(lo, hi, idx, n):
    """The kernel's voxel coordinate lo + ((hi - lo) * i) / n, each step rounded to float32."""
    lo32, hi32 = np.float32(lo), np.float32(hi)
    return lo32 + ((hi32 - lo32) * idx.astype(np.float32)) / np.float32(n)


def test_full_volume_512(dev, oracle):
    vw = scenes.full_volume(512, 1)
    n = 512
    vol = DeviceVolume(vw, device=dev, stats=False)
    out = {}
    for variant, jit in [(capi.VARIANT_PLAIN, True), (capi.VARIANT_PRODUCT, True), (capi.VARIANT_PRODUCT, False)]:
        vol.run(variant, jit=jit)
        torch.cuda.synchronize()
        out[(variant, jit)] = vol.d_out.clone()
    # determinism over the whole volume
    vol.run(capi.VARIANT_PRODUCT, jit=True)
    torch.cuda.synchronize()
    assert torch.equal(vol.d_out.view(torch.int32), out[(capi.VARIANT_PRODUCT, True)].view(torch.int32))
    # the kernel compiled for the sequence equals the precompiled one, bit for bit
    assert torch.equal(out[(capi.VARIANT_PRODUCT, True)].view(torch.int32),
                       out[(capi.VARIANT_PRODUCT, False)].view(torch.int32))
    # seeded voxels against the oracle
    idx = np.random.default_rng(512).choice(n * n * n, VOXELS, replace=False).astype(np.int64)
    x, y, z = idx % n, (idx // n) % n, idx // (n * n)
    pts = np.stack([_voxel_coords(vw.lo[0], vw.hi[0], x, n), _voxel_coords(vw.lo[1], vw.hi[1], y, n),
                    _voxel_coords(vw.lo[2], vw.hi[2], z, n),
                    np.full(VOXELS, vw.params.d, dtype=np.float32)], axis=1)
    d_idx = torch.from_numpy(idx).to(dev)
    for variant, mode in [(capi.VARIANT_PLAIN, ORC_PLAIN), (capi.VARIANT_PRODUCT, ORC_PRODUCT)]:
        got = out[(variant, True)][d_idx].cpu().numpy()
        ref = oracle.lyap4d(mode, pts.astype(np.float64), vw.params.settle, vw.params.accum, vol.seq)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), "NaN positions differ"
        fin = np.isfinite(ref)
        err = float(np.max(np.abs(got[fin].astype(np.float64) - ref[fin])))
        assert err <= LAM_TOL[mode], f"lambda differs by {err}"
        # the reference's own arithmetic, and FP64: the error against FP64 is the
        # reference arithmetic's own FP32 error, voxel by voxel
        lref = oracle.lyap4d(ORC_REF, pts.astype(np.float64), vw.params.settle, vw.params.accum, vol.seq)
        l64 = oracle.lyap4d(ORC_F64, pts.astype(np.float64), vw.params.settle, vw.params.accum, vol.seq)
        assert np.array_equal(np.isnan(got), np.isnan(lref)), "NaN positions differ from the reference arithmetic"
        fin = np.isfinite(lref)
        err = float(np.max(np.abs(got[fin].astype(np.float64) - lref[fin])))
        assert err <= REF_TOL, f"lambda differs from the reference arithmetic by {err}"
        ok = fin & np.isfinite(l64)
        e_gpu = np.abs(got[ok].astype(np.float64) - l64[ok])
        e_ref = np.abs(lref[ok] - l64[ok])
        assert float(np.median(e_gpu)) <= 1e-5
        assert float(np.max(np.abs(e_gpu - e_ref))) <= REF_TOL


@pytest.mark.parametrize("flags", [0, capi.FLAG_NO_SPECULATION])
def test_hone_cap_rays_vs_oracle(dev, oracle, frame_wl, flags):
    """Rays that take the honing cap of 256 samples (kernel.cu:420 leaves the
    loop unbounded; both the kernel and the oracle stop at 256): grazing rays
    whose hone step falls below an ulp of t, where the kernel takes the cap at
    once when a step no longer moves the point and otherwise samples the
    remaining steps ahead.  Every such pixel of the 1080p frame, with and
    without sampling ahead, has the oracle's sample counts, hit point and
    lambda bit for bit."""
    wl = frame_wl
    f = DeviceFrame(wl, device=dev, counts=True, stats=False)
    f.run(capi.VARIANT_PRODUCT, jit=True, flags=flags)
    torch.cuda.synchronize()
    pts, cnt = f.points(), f.counts()
    ys, xs = np.nonzero(cnt[..., 1] == 256)
    assert len(ys) >= 10, f"only {len(ys)} rays reach the honing cap"
    for y, x in zip(ys[:256], xs[:256]):
        rc, pt, rcnt = oracle.raymarch(ORC_PRODUCT, int(x), int(y), f.cam, f.prm, f.seq)
        assert tuple(int(v) for v in cnt[y, x]) == rcnt, f"pixel ({x}, {y}): counts {cnt[y, x]} vs {rcnt}"
        g = pts[y, x]
        assert rc == 0 and not np.isnan(g["a"])
        assert np.array_equal(np.array(g["P"]), np.array([pt.P.x, pt.P.y, pt.P.z], dtype=np.float32))
        assert abs(float(g["l"]) - pt.l) <= LAM_TOL[ORC_PRODUCT] or (np.isnan(g["l"]) and np.isnan(pt.l))


@pytest.mark.parametrize("jit,jitter", [(True, 0.0), (False, 0.0), (True, 0.5)])
def test_tail_handover_gives_the_same_frame(dev, jit, jitter):
    """After the pixel queue drains, warps hand their longest rays to warps
    of the block left without one (the whole ray state moves).  The frame is
    bit-identical to the render without hand-overs, which do happen."""
    wl = scenes.full_render(1, 960, 540)
    wl.params.jitter = jitter
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PRODUCT, jit=jit, flags=capi.FLAG_NO_TAIL_BALANCE)
    torch.cuda.synchronize()
    want = (f.d_rgba.clone(), f.d_points.clone(), f.d_counts.clone())
    assert f.stats()[capi.STAT_TAIL_HANDOVERS] == 0
    f.reset_stats()
    f.d_points.fill_(0.0)
    f.run(capi.VARIANT_PRODUCT, jit=jit)
    torch.cuda.synchronize()
    st = f.stats()
    assert st[capi.STAT_TAIL_HANDOVERS] > 0
    assert st[capi.STAT_RAYS] == wl.width * wl.height
    assert torch.equal(f.d_rgba, want[0])
    assert torch.equal(f.d_points.view(torch.int32), want[1].view(torch.int32))
    assert torch.equal(f.d_counts, want[2])
