"""The precision form: lambda in the three forms at seeded points against the
oracle, and the FP64 bisection of every ray's crossing (through the C ABI).

Tolerances:
  * FP64 form vs the FP64 oracle: the orbit is the same double arithmetic,
    only the log accumulation differs (running product vs a log per step):
    |d lambda| <= 1e-10;
  * product form vs ORC_PRODUCT: <= 5e-6;  plain vs ORC_PLAIN: <= 5e-5;
  * bisected render: the stored lambda at every hit point is the FP64
    lambda there (<= 1e-10 against the FP64 oracle at the same float point);
    hit / miss agrees with the plain render on >= 99.9 % of pixels.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame  # noqa: E402
from oracle import ORC_F64, ORC_PLAIN, ORC_PRODUCT  # noqa: E402


@pytest.fixture(scope="module")
def dev():
    assert torch.cuda.is_available()
    return torch.device("cuda:0")


def _points(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)


@pytest.mark.parametrize("seqstr,settle,accum", [("ABC", 20, 100), ("AACACBACCAAB", 200, 1000)])
def test_lambda_points_three_forms(dev, oracle, seqstr, settle, accum):
    n = 1 << 14
    pts = _points(n, 2.5, 4.0, 11)
    prm = scenes.make_params(settle, accum, d=3.0)
    seq = capi.seq_parse(seqstr)
    d_seq = torch.from_numpy(seq).to(dev)
    d_xyz = torch.from_numpy(pts.reshape(-1)).to(dev)
    pts4 = np.column_stack([pts.astype(np.float64), np.full(n, prm.d, dtype=np.float64)])
    out32 = torch.empty(n, dtype=torch.float32, device=dev)
    out64 = torch.empty(n, dtype=torch.float64, device=dev)
    for form, mode, tol in [(capi.VARIANT_PLAIN, ORC_PLAIN, 5e-5), (capi.VARIANT_PRODUCT, ORC_PRODUCT, 5e-6)]:
        capi.lambda_points(d_xyz, n, prm, d_seq, seq.size, form, out32)
        got = out32.cpu().numpy()
        ref = oracle.lyap4d(mode, pts4, settle, accum, seq).astype(np.float32)
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        f = np.isfinite(ref)
        assert np.max(np.abs(got[f] - ref[f])) <= tol
    capi.lambda_points(d_xyz, n, prm, d_seq, seq.size, capi.FORM_F64, out64)
    got = out64.cpu().numpy()
    ref = oracle.lyap4d(ORC_F64, pts4, settle, accum, seq)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    f = np.isfinite(ref)
    assert np.max(np.abs(got[f] - ref[f])) <= 1e-10


def test_bisected_render(dev, oracle):
    wl = scenes.small_render(96)
    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PLAIN)
    plain_hit = ~np.isnan(f.points()["a"])
    plain_pts_P = f.points()["P"].copy()
    f.reset_stats()
    f.run(capi.VARIANT_PRODUCT, flags=capi.FLAG_BISECT_F64, bisect_halvings=20)
    torch.cuda.synchronize()
    pts, cnt, rgba = f.points(), f.counts(), f.rgba()
    hit = ~np.isnan(pts["a"])
    assert (hit == plain_hit).mean() >= 0.999
    # every crossing with a bracket was halved 20 times; normals sampled 6 times
    assert np.all(cnt[..., 1][hit & (cnt[..., 0] > 1)] == 20)
    assert np.all(cnt[..., 2][hit] == 6)
    st = f.stats()
    assert st[capi.STAT_HITS] == hit.sum()
    # the stored lambda is the FP64 lambda at the stored point
    P = pts["P"][hit].astype(np.float64)
    pts4 = np.column_stack([P, np.full(len(P), f.prm.d)])
    ref = oracle.lyap4d(ORC_F64, pts4, f.prm.settle, f.prm.accum, f.seq)
    got = pts["l"][hit].astype(np.float64)
    fin = np.isfinite(ref)
    # stored as float: compare the float-rounded FP64 value
    assert np.max(np.abs(got[fin] - ref[fin].astype(np.float32))) <= 1e-6
    # the bisected point lies on the last march step: between the previous
    # sample and the plain render's hit point (same march decisions, no honing)
    Pp = plain_pts_P[hit].astype(np.float64)
    dist = np.linalg.norm(Pp - P, axis=-1)
    # one march step is a 256th of the ray's chord through the [2.5, 4]^3 box (at most sqrt(3) * 1.5)
    assert np.max(dist) <= np.sqrt(3.0) * 1.5 / 256.0 * 1.01
    # colours exist for every hit
    assert (rgba[hit][:, 3] > 0).mean() > 0.99


def test_bisect_rejected_without_allocation(dev):
    wl = scenes.small_render(16)
    f = DeviceFrame(wl, device=dev)
    with pytest.raises(capi.LyapError) as e:
        capi.render_noalloc(f.cam, f.prm, f.d_seq, f.seq.size, f.d_lights, len(f.lights), f.d_rgba, f.d_points,
                            16, 16, ext=capi.LyapRenderExt(flags=capi.FLAG_BISECT_F64))
    assert e.value.code == capi.LYAP_ERR_INVALID_ARG
