"""The learned proposal on the GPU: the tensor-core forward and backward
kernels against the CPU oracle (oracle/net_oracle.py), training, and the
proposal render against the plain render it must reproduce."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceFrame  # noqa: E402
from oracle import net_oracle as no  # noqa: E402

LO, HI = (2.0, 2.0, 2.0), (4.0, 4.0, 4.0)


def _rand_net(seed):
    rng = np.random.default_rng(seed)
    p = no.init_params(seed)
    p[no.OFF_B1:no.OFF_W2] = rng.standard_normal(64) * 0.1
    p[no.OFF_B2:no.OFF_W3] = rng.standard_normal(64) * 0.1
    p[no.OFF_B3] = 0.2
    p = p.astype(np.float32).astype(np.float64)
    return capi.net_from_params(p, LO, HI), p


def _points(n, seed):
    return np.random.default_rng(seed).uniform(2.0, 4.0, (n, 3)).astype(np.float32)


def test_forward_matches_oracle():
    """Tensor-core forward vs the oracle's rounded forward.  The GPU differs
    by tanh.approx.f32 (relative error below 2^-10.9), the features'
    double-angle recurrence and FP32 accumulation; those move some BF16
    roundings of f and h1 by one unit.  Tolerance: max |diff| <= 0.02 * std
    of the outputs, mean |diff| <= 0.002 * std."""
    net, p = _rand_net(1)
    n = 6000   # not a multiple of the 128-point tile
    xyz = _points(n, 2)
    d_xyz = torch.from_numpy(xyz).cuda()
    d_out = torch.full((n,), float("nan"), device="cuda")
    capi.net_eval(net, d_xyz, n, d_out)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy().astype(np.float64)
    ref, _ = no.forward(p, no.to_unit(xyz, LO, HI))
    err = np.abs(got - ref)
    s = np.std(ref)
    assert np.isfinite(got).all()
    assert err.max() <= 0.02 * s and err.mean() <= 0.002 * s, (err.max(), err.mean(), s)


def test_gradient_matches_oracle():
    """lyap_net_grad (forward + backward on the tensor cores, dz rounded to
    BF16 as the products' operands) vs the oracle's exact gradient of the
    rounded forward pass: every parameter block within 3% relative (L2) and
    cosine similarity above 0.999; the loss within 1%."""
    net, p = _rand_net(3)
    n = 4096
    xyz = _points(n, 4)
    tgt = np.random.default_rng(5).standard_normal(n).astype(np.float32) * 0.5
    d_xyz, d_t = torch.from_numpy(xyz).cuda(), torch.from_numpy(tgt).cuda()
    d_g = torch.zeros(capi.NET_PARAMS, device="cuda")
    d_l = torch.zeros(1, device="cuda")
    capi.net_grad(net, d_xyz, d_t, n, d_g, d_l)
    torch.cuda.synchronize()
    g = d_g.cpu().numpy().astype(np.float64)
    loss_ref, g_ref = no.loss_grad(p, no.to_unit(xyz, LO, HI), tgt.astype(np.float64))
    assert abs(float(d_l.item()) - loss_ref) <= 0.01 * loss_ref
    blocks = {"w1": (no.OFF_W1, no.OFF_B1), "b1": (no.OFF_B1, no.OFF_W2), "w2": (no.OFF_W2, no.OFF_B2),
              "b2": (no.OFF_B2, no.OFF_W3), "w3": (no.OFF_W3, no.OFF_B3), "b3": (no.OFF_B3, no.NPARAM)}
    for name, (a, b) in blocks.items():
        x, y = g[a:b], g_ref[a:b]
        rel = np.linalg.norm(x - y) / np.linalg.norm(y)
        cos = float(x @ y / (np.linalg.norm(x) * np.linalg.norm(y)))
        assert rel < 0.03 and cos > 0.999, (name, rel, cos)


def test_gradient_of_a_single_tile_and_many_tiles_agree():
    """The per-CTA partials are summed in a fixed order: the gradient of 256
    points equals the mean of the two 128-point halves' gradients."""
    net, _ = _rand_net(7)
    xyz = _points(256, 8)
    tgt = np.random.default_rng(9).standard_normal(256).astype(np.float32)
    d_xyz, d_t = torch.from_numpy(xyz).cuda(), torch.from_numpy(tgt).cuda()
    gs = []
    for lo, n in ((0, 256), (0, 128), (128, 128)):
        d_g = torch.zeros(capi.NET_PARAMS, device="cuda")
        capi.net_grad(net, d_xyz[lo:lo + n].contiguous(), d_t[lo:lo + n].contiguous(), n, d_g)
        gs.append(d_g.cpu().numpy().astype(np.float64))
    np.testing.assert_allclose(gs[0], 0.5 * (gs[1] + gs[2]), rtol=1e-4, atol=1e-6)


def _train(steps=768, seed=11, n=1 << 16):
    wl = scenes.full_render(1)
    return capi.net_train(wl.params, capi.seq_parse(wl.seq), n_samples=n, n_val=1 << 13, steps=steps, seed=seed,
                          with_loss=True)


def test_training_reduces_loss_and_is_deterministic():
    net1, loss1 = _train()
    net2, loss2 = _train()
    assert bytes(net1) == bytes(net2) and np.array_equal(loss1, loss2)
    assert np.isfinite(loss1).all()
    assert loss1[-50:].mean() < 0.4 * loss1[:10].mean(), (loss1[:10].mean(), loss1[-50:].mean())
    assert net1.val_mse < 0.1 and net1.val_mse < 0.5 * loss1[:10].mean()
    assert net1.magic == capi.NET_MAGIC and net1.steps == 768 and net1.n_samples == 1 << 16


def test_trained_net_predicts_plain_lambda():
    """The trained net's error at fresh points against the plain FP32 method
    (lambda from lyap_lambda_points, clamped as in training)."""
    net, _ = _train(steps=2048, n=1 << 18)
    wl = scenes.full_render(1)
    seq = capi.seq_parse(wl.seq)
    n = 8192
    xyz = _points(n, 21)
    d_xyz = torch.from_numpy(xyz).cuda()
    d_seq = torch.from_numpy(seq).cuda()
    d_lam = torch.empty(n, device="cuda")
    d_pred = torch.empty(n, device="cuda")
    capi.lambda_points(d_xyz, n, wl.params, d_seq, seq.size, capi.VARIANT_PLAIN, d_lam)
    capi.net_eval(net, d_xyz, n, d_pred)
    torch.cuda.synchronize()
    lam = np.nan_to_num(d_lam.cpu().numpy(), nan=-3.0).clip(-3.0, 1.0)
    pred = d_pred.cpu().numpy()
    mse = float(np.mean((pred - lam) ** 2))
    assert mse < 0.1 and mse < 0.3 * float(np.var(lam)), (mse, float(np.var(lam)))


def _frame(w=320, h=180):
    return DeviceFrame(scenes.full_render(1, width=w, height=h), counts=True)


def _run(f, net=None, margin=0.0, **kw):
    f.reset_stats()
    extra = {}
    if net is not None:
        extra = dict(proposal=ctypes.pointer(net), proposal_margin=margin)
    f.run(capi.VARIANT_PRODUCT, **extra, **kw)
    torch.cuda.synchronize()
    return f.rgba().copy(), f.points().copy(), f.counts().copy(), f.stats()


def _const_net(value):
    """A net whose output is `value` everywhere (all weights 0, output bias `value`)."""
    p = np.zeros(capi.NET_PARAMS, dtype=np.float64)
    p[no.OFF_B3] = value
    return capi.net_from_params(p, LO, HI)


def _grid(net, n=capi.PROPOSAL_GRID_DEFAULT, dilate=0):
    d = torch.empty(n ** 3, device="cuda")
    capi.net_grid(net, n, dilate, d)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def test_proposal_grid_is_the_corner_minimum():
    """lyap_net_grid: each cell holds the minimum of the net at its 8 corners,
    with dilation the minimum over the 27 cells around."""
    net, _ = _rand_net(4)
    n = 16
    g = _grid(net, n).reshape(n, n, n)
    g1 = np.linspace(2.0, 4.0, n + 1)
    zz, yy, xx = np.meshgrid(g1, g1, g1, indexing="ij")
    xyz = np.ascontiguousarray(np.stack([xx, yy, zz], -1).reshape(-1, 3)).astype(np.float32)   # x fastest
    d_xyz = torch.from_numpy(xyz).cuda()
    d_o = torch.empty(len(xyz), device="cuda")
    capi.net_eval(net, d_xyz, len(xyz), d_o)
    torch.cuda.synchronize()
    corner = d_o.cpu().numpy().reshape(n + 1, n + 1, n + 1)
    want = np.minimum.reduce([corner[k:k + n, j:j + n, i:i + n] for k in (0, 1) for j in (0, 1) for i in (0, 1)])
    # the grid's corners are u = i / n in the net's unit box; lyap_net_eval maps xyz there itself
    assert np.max(np.abs(g - want)) <= 1e-4 * max(1.0, np.abs(want).max())
    gd = _grid(net, n, 1).reshape(n, n, n)
    pad = np.pad(g, 1, mode="constant", constant_values=np.inf)
    wantd = np.minimum.reduce([pad[k:k + n, j:j + n, i:i + n] for k in range(3) for j in range(3) for i in range(3)])
    assert np.array_equal(gd, wantd)


def test_proposal_that_skips_nothing_is_bit_identical():
    f = _frame()
    rgba0, pts0, cnt0, st0 = _run(f)
    net, _ = _rand_net(1)
    rgba1, pts1, cnt1, st1 = _run(f, net, margin=1e30)
    assert st1[capi.STAT_PROPOSAL_POINTS] > 0 and st1[capi.STAT_PROPOSAL_SKIPPED] == 0
    assert np.array_equal(rgba0, rgba1)
    assert pts0.tobytes() == pts1.tobytes()
    assert np.array_equal(cnt0, cnt1)
    # the net's grid is cached: a second render evaluates no net points
    _, _, _, st2 = _run(f, net, margin=1e30)
    assert st2[capi.STAT_PROPOSAL_POINTS] == 0


@pytest.mark.parametrize("seg", [8, 5])
def test_proposal_skipping_everywhere_only_moves_hits_back(seg):
    """With every position skippable the march skips runs of seg - 1
    positions and confirms each with the next sample: no pixel gains a hit,
    every hit lies at or beyond the plain render's hit on the same ray, and
    far fewer march samples are evaluated."""
    f = _frame()
    rgba0, pts0, cnt0, st0 = _run(f)
    net = _const_net(100.0)
    rgba1, pts1, cnt1, st1 = _run(f, net, margin=0.0, proposal_segment=seg)
    # a hit writes a finite position (its lambda may be NaN: a NaN sample counts as a hit)
    hit0, hit1 = ~np.isnan(pts0["P"][..., 0]), ~np.isnan(pts1["P"][..., 0])
    assert not (hit1 & ~hit0).any()
    assert st1[capi.STAT_PROPOSAL_SKIPPED] > 0 and st1[capi.STAT_PROPOSAL_REWOUND] > 0
    assert st1[capi.STAT_MARCH] < 0.5 * st0[capi.STAT_MARCH]
    cam = f.cam
    C = np.array([cam.C.x, cam.C.y, cam.C.z])
    both = hit0 & hit1
    d0 = np.linalg.norm(pts0["P"][both].astype(np.float64) - C, axis=1)
    d1 = np.linalg.norm(pts1["P"][both].astype(np.float64) - C, axis=1)
    assert (d1 >= d0 - 1e-4).all()
    # confirmation keeps most surfaces even with nothing known about the field
    assert hit1.sum() >= 0.8 * hit0.sum()


def _oracle_prop_frame(oracle, f, grid, n, seg, tau):
    from oracle import ORC_PRODUCT, proposal
    pr = proposal(grid, n, seg - 1, LO, HI, tau)
    return oracle.render_prop(ORC_PRODUCT, f.width, f.height, f.cam, f.prm, f.seq, f.lights, pr)


@pytest.mark.parametrize("which,margin,seg,flags", [("everywhere", 0.0, 8, 0), ("everywhere", 0.0, 5, 0),
                                                    ("trained", 0.5, 8, 0),
                                                    ("trained", 0.5, 8, capi.FLAG_NO_SPECULATION)])
def test_proposal_march_matches_oracle(oracle, which, margin, seg, flags):
    """The proposal render (kernel compiled for the sequence, paired rounds,
    samples taken ahead along the skipped runs) against the oracle's
    restatement of the proposal march on the same grid: per-pixel sample
    counts equal on >= 99.9 % of pixels (the product form's lambda differs
    from the oracle's by <= 5e-6, which can flip a decision), and where they
    are equal the hit point is bit-identical; the frame's skipped and rewound
    totals agree with the oracle's within the same share."""
    f = _frame()
    net = _const_net(100.0) if which == "everywhere" else _train(steps=2048, n=1 << 18)[0]
    _, pts1, cnt1, st1 = _run(f, net, margin=margin, proposal_segment=seg, jit=True, flags=flags)
    grid = _grid(net)
    tau = float(np.float32(f.prm.opaqueThreshold) + np.float32(margin))
    _, r_pts, r_cnt, r_pc = _oracle_prop_frame(oracle, f, grid, capi.PROPOSAL_GRID_DEFAULT, seg, tau)
    agree = np.all(cnt1 == r_cnt, axis=-1)
    assert agree.mean() >= 0.999, agree.mean()
    gh, rh = ~np.isnan(pts1["a"]), ~np.isnan(r_pts["a"])
    assert np.array_equal(gh[agree], rh[agree])
    both = agree & gh
    assert np.array_equal(pts1["P"][both], r_pts["P"][both])
    sk, rw = int(st1[capi.STAT_PROPOSAL_SKIPPED]), int(st1[capi.STAT_PROPOSAL_REWOUND])
    rsk, rrw = int(r_pc[..., 0].sum()), int(r_pc[..., 1].sum())
    assert abs(sk - rsk) <= 0.01 * max(1, rsk) and abs(rw - rrw) <= 0.01 * max(1, rrw) + 2, (sk, rsk, rw, rrw)
    assert st1[capi.STAT_MARCH] == cnt1[..., 0].sum()


def test_trained_proposal_gain_and_agreement():
    """What the trained net gains over the march without it, on the 1080p
    scene at 480x270, at the default margin (PROPOSAL_MARGIN_DEFAULT): fewer
    lambda evaluations, with >= 99.9 % of the plain render's surface pixels
    hit too (>= 99.8 % at the bit-identical sample).  Every hit of the
    proposal render is a hit of the plain render at the same sample
    (bit-identical position, normal and lambda) or a later one."""
    net, _ = _train(steps=4096, n=1 << 20)
    f = _frame(480, 270)
    rgba0, pts0, cnt0, st0 = _run(f, jit=True)
    rgba1, pts1, cnt1, st1 = _run(f, net, margin=capi.PROPOSAL_MARGIN_DEFAULT, jit=True)
    hit0, hit1 = ~np.isnan(pts0["P"][..., 0]), ~np.isnan(pts1["P"][..., 0])
    assert not (hit1 & ~hit0).any()
    bits0 = np.ascontiguousarray(pts0["P"]).view(np.uint32)
    bits1 = np.ascontiguousarray(pts1["P"]).view(np.uint32)
    same = hit0 & hit1 & (bits0 == bits1).all(-1)
    surf = hit1.sum() / max(1, hit0.sum())
    evaluated = st1[capi.STAT_SAMPLES] / st0[capi.STAT_SAMPLES]
    print(f"proposal: {evaluated:.3f} of the plain samples evaluated, surface agreement {surf:.4f}, "
          f"same-sample {same.sum() / max(1, hit0.sum()):.4f}, skipped {st1[capi.STAT_PROPOSAL_SKIPPED]}, "
          f"rewound {st1[capi.STAT_PROPOSAL_REWOUND]}")
    assert st1[capi.STAT_PROPOSAL_SKIPPED] > 0 and evaluated < 1.0
    assert surf >= 0.999 and same.sum() >= 0.998 * hit0.sum()
    # where the hit is the same sample, everything but the a/c sums is the plain render's
    for k in ("P", "N", "l"):
        a, b = np.ascontiguousarray(pts0[k][same]), np.ascontiguousarray(pts1[k][same])
        assert a.tobytes() == b.tobytes(), k
