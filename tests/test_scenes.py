"""The seeded workloads the benchmark and the reports are defined on.

A seed names the same scene on every machine only if the generator and the
scene construction never change, so they are pinned here: SplitMix64 against
the published reference outputs for seed 1234567, and the benchmark frame,
the 512^3 volume and the batched workload by their parameters and by the
exact bytes of their cameras and lights (SHA-256 prefixes).  The cameras are
computed in double with the host libm's sin / cos before rounding to float;
the digests below were recorded on an x86-64 host and agree with those
computed on the aarch64 (Grace) GPU host, so they hold on both.
"""
import hashlib

from lyapunov3d_gb300 import scenes


def _h(*parts):
    h = hashlib.sha256()
    for p in parts:
        h.update(p)
    return h.hexdigest()[:16]


def test_splitmix64_reference_outputs():
    r = scenes.SplitMix64(1234567)
    assert [r.next_u64() for _ in range(5)] == [6457827717110365317, 3203168211198807973, 9817491932198370423,
                                                 4593380528125082431, 16408922859458223821]


def test_bench_frame_definition():
    wl = scenes.full_render(1)
    assert (wl.name, wl.seq, wl.width, wl.height) == ("frame1080_seq12_200+1000_seed1", "AACACBACCAAB", 1920, 1080)
    p = wl.params
    assert (p.settle, p.accum, p.stepMethod, p.depth, p.jitter, p.nearMultiplier) == (200, 1000, 1, 512.0, 0.0, 1.0)
    assert (p.opaqueThreshold, p.chaosThreshold, p.nearThreshold, p.refine) == (-0.75, -0.5, -1.0, 32.0)
    assert (p.lMin, p.lMax) == (2.0, 4.0)
    assert len(wl.lights) == 1
    assert _h(bytes(wl.cam)) == "6145a3e00ef72a7f"
    assert _h(bytes(wl.lights[0])) == "f71170854ada571f"


def test_volume_definition():
    vw = scenes.full_volume(512, 1)
    assert (vw.name, vw.seq, vw.n, vw.lo, vw.hi) == ("volume512_seq12_200+1000_seed1", "AACACBACCAAB",
                                                      (512, 512, 512), (2.0, 2.0, 2.0), (4.0, 4.0, 4.0))
    assert (vw.params.settle, vw.params.accum) == (200, 1000)


def test_batch_workload_definition():
    b = scenes.batch_workloads(seed=4)
    assert len(b) == 288 and sum(w.width * w.height for w in b) == 283790336
    parts = []
    for w in b:
        parts += [w.seq.encode(), bytes(w.params), bytes(w.cam), f"{w.width}x{w.height}".encode()]
    assert _h(*parts) == "f93bd7874221d60d"
