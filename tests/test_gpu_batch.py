"""The batched renderer (lyap_batch_*): one graph launch over requests of
different sizes, sequences, iteration counts and parameters must give every
request exactly the bytes lyap_render gives it alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from lyapunov3d_gb300 import capi, scenes  # noqa: E402
from lyapunov3d_gb300.device import DeviceBatch, DeviceFrame  # noqa: E402
from oracle import ORC_PLAIN  # noqa: E402


def _small_batch():
    wls = scenes.batch_workloads(seed=7, scale=32, n_render=10, n_slices=3)
    for wl in wls:   # keep the iteration counts test-sized
        wl.params.settle = 20
        wl.params.accum = max(20, wl.params.accum // 40)
        wl.params.depth = max(32.0, wl.params.depth / 8)
    # a jittered request (no speculation) and a small explicit one
    wls[1].params.jitter = 0.4
    wls.append(scenes.small_render(40))
    return wls


@pytest.mark.parametrize("variant", [capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT])
@pytest.mark.parametrize("autotune", [True, False])
def test_batch_matches_single_renders(variant, autotune):
    dev = torch.device("cuda:0")
    wls = _small_batch()
    db = DeviceBatch(wls, device=dev, variant=variant, autotune=autotune, counts=True)
    db.run()
    torch.cuda.synchronize()
    info = db.batch.info()
    assert info.requests == len(wls) and info.chunks > 0
    if autotune:
        assert info.candidates == 12
    for wl, bf in zip(wls, db.frames):
        f = DeviceFrame(wl, device=dev, counts=True)
        f.run(variant)
        torch.cuda.synchronize()
        assert torch.equal(bf.d_rgba, f.d_rgba), wl.name
        assert torch.equal(bf.d_points.view(torch.int32), f.d_points.view(torch.int32)), wl.name
        assert torch.equal(bf.d_counts, f.d_counts), wl.name
    # a replay of the graph gives the same bytes again
    first = [bf.d_points.clone() for bf in db.frames]
    for bf in db.frames:
        bf.d_points.fill_(0.0)
    db.run()
    torch.cuda.synchronize()
    for a, bf in zip(first, db.frames):
        assert torch.equal(a.view(torch.int32), bf.d_points.view(torch.int32))
    st = db.stats()
    assert st[capi.STAT_RAYS] == 2 * sum(wl.width * wl.height for wl in wls)


def test_batch_vs_oracle(oracle):
    dev = torch.device("cuda:0")
    wls = _small_batch()[-4:]
    for wl in wls:
        wl.params.jitter = 0.0
    db = DeviceBatch(wls, device=dev, counts=True)
    db.run()
    torch.cuda.synchronize()
    for wl, bf in zip(wls, db.frames):
        rgba, pts, cnt = oracle.render(ORC_PLAIN, wl.width, wl.height, bf.cam, bf.prm, bf.seq, bf.lights)
        agree = np.all(bf.counts() == cnt, axis=-1)
        assert agree.mean() >= 0.99, wl.name
        hit = agree & ~np.isnan(pts["a"])
        assert np.array_equal(bf.points()["P"][hit], pts["P"][hit])


def test_batch_rejects_bad_request():
    dev = torch.device("cuda:0")
    wl = scenes.small_render(16)
    f = DeviceFrame(wl, device=dev)
    q = capi.LyapRequest()
    q.cam, q.prm = f.cam, f.prm
    q.d_seq, q.d_lights, q.d_rgba, q.d_points = f.d_seq.data_ptr(), f.d_lights.data_ptr(), 0, f.d_points.data_ptr()
    q.seq_len, q.n_lights, q.width, q.height = f.seq.size, 1, 16, 16
    with pytest.raises(capi.LyapError) as e:
        capi.Batch([q])
    assert e.value.code == capi.LYAP_ERR_INVALID_ARG and "request 0" in e.value.message


def _one_sequence_batch(seq):
    wls = scenes.batch_workloads(seed=9, scale=32, n_render=10, n_slices=0, one_seq=seq)
    for wl in wls:   # keep the iteration counts test-sized
        wl.params.settle = 20 + 7 * (wl.params.accum % 3)   # settle counts differing by whole periods
        wl.params.accum = max(20, wl.params.accum // 40)
        wl.params.depth = max(32.0, wl.params.depth / 8)
    return wls


@pytest.mark.parametrize("variant", [capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT])
def test_one_sequence_batch_runs_the_specialised_kernel(variant):
    """A batch whose requests share one sequence (and settle count mod its
    period) runs the batch kernel compiled for that sequence at run time
    (paired rounds for the product form); every request still gets exactly
    lyap_render's bytes.  LYAP_FLAG_NO_JIT keeps the library's kernel."""
    dev = torch.device("cuda:0")
    wls = _one_sequence_batch("ABCCABB")   # period 7: settle 20, 27, 34 share settle mod 7
    db = DeviceBatch(wls, device=dev, variant=variant, autotune=False, counts=True)
    db.run()
    torch.cuda.synchronize()
    info = db.batch.info()
    if not capi.jit_info()[0]:
        pytest.skip("NVRTC unavailable")
    assert info.specialised == len(wls)
    for wl, bf in zip(wls, db.frames):
        f = DeviceFrame(wl, device=dev, counts=True)
        f.run(variant)
        torch.cuda.synchronize()
        assert torch.equal(bf.d_rgba, f.d_rgba), wl.name
        assert torch.equal(bf.d_points.view(torch.int32), f.d_points.view(torch.int32)), wl.name
        assert torch.equal(bf.d_counts, f.d_counts), wl.name
    off = DeviceBatch(wls, device=dev, variant=variant, autotune=False, counts=True, flags=capi.FLAG_NO_JIT)
    assert off.batch.info().specialised == 0


def _cost(wl):
    return wl.width * wl.height * (wl.params.settle + wl.params.accum) * max(1.0, wl.params.depth)


@pytest.mark.parametrize("variant", [capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT])
def test_mixed_batch_compiles_its_heaviest_sequence_groups(variant):
    """Requests that share a sequence form a group; the batch compiles its
    kernel for the heaviest groups (jit_groups of them) and runs each as a
    launch of its own, the rest on the library's kernel.  Every request gets
    lyap_render's bytes whichever kernel ran it."""
    dev = torch.device("cuda:0")
    wls = _one_sequence_batch("ABCCABB")[:4] + _one_sequence_batch("CAB")[:3] + _small_batch()[:3]
    wls[0].width, wls[0].height = 96, 80   # the first group is the heaviest
    groups = {}
    for wl in wls:
        key = (wl.seq, wl.params.settle % len(wl.seq))
        groups.setdefault(key, []).append(wl)
    heavy = max(groups.values(), key=lambda g: sum(_cost(w) for w in g))
    one = DeviceBatch(wls, device=dev, variant=variant, autotune=False, counts=True, jit_groups=1)
    one.run()
    torch.cuda.synchronize()
    if not capi.jit_info()[0]:
        pytest.skip("NVRTC unavailable")
    assert one.batch.info().specialised == len(heavy)
    every = DeviceBatch(wls, device=dev, variant=variant, autotune=False, counts=True)
    every.run()
    torch.cuda.synchronize()
    total = sum(_cost(w) for w in wls)
    eligible = [g for g in groups.values() if sum(_cost(w) for w in g) * 1000 >= total]
    assert every.batch.info().specialised == sum(len(g) for g in eligible)
    for i, wl in enumerate(wls):
        f = DeviceFrame(wl, device=dev, counts=True)
        f.run(variant)
        torch.cuda.synchronize()
        for bf in (one.frames[i], every.frames[i]):
            assert torch.equal(bf.d_rgba, f.d_rgba), wl.name
            assert torch.equal(bf.d_points.view(torch.int32), f.d_points.view(torch.int32)), wl.name
            assert torch.equal(bf.d_counts, f.d_counts), wl.name
