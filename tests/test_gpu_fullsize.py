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
  * volume: lambda at 8192 seeded voxels against the oracle (same voxel
    coordinates, float32 arithmetic as the kernel), NaN positions exact;
    over all 134 M voxels the sweep is deterministic and the run-time
    specialised kernel is bit-identical to the precompiled one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame, DeviceVolume  # noqa: E402
from oracle import ORC_PLAIN, ORC_PRODUCT  # noqa: E402

LAM_TOL = {ORC_PLAIN: 5e-5, ORC_PRODUCT: 5e-6}   # |lambda_gpu - lambda_oracle|, accum <= 1000
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
