#!/usr/bin/env python3
"""Headline benchmark of the lyapunov3d hot path on GB300.

Workload (one "step"): one 1920x1080 frame of the Lyapunov-field raymarch --
512 steps per ray (step method 1), a seeded 12-symbol sequence over {A,B,C},
200 settle + 1000 accumulated iterations per sample, parameter cube
[2, 4]^3, camera uniform on S^3 at distance 5-8 from the cube centre, one
directional light (scenes.full_render(seed=1)); synthetic inputs, no dataset.

Metric: G logistic-iters/s -- logistic-map iterations the plain method
performs for the frame (exact per-sample counts from the kernel's statistics)
divided by the device time of the frame; frames/s beside it.  `value` is
the chosen form (the renormalised-product lambda); `plain` is the plain
FP32 drop-in on the same GPU, same frame.  `e2e` is the same metric through
the host-buffer C-ABI call (lyap_render_host: upload, render, download of
the RGBA image and the LyapPoint buffer, synchronise), timed on the host.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --gpus N > 1 (under torchrun) every rank renders the same frame as an
independent replica (the path does not shard); value = total iterations of
all ranks / max rank time.  --impl reference times the reference algorithm
on the host cores instead (the oracle's restatement of the reference's
arithmetic, all host threads, a bounded band of rows per step).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 512 << 20   # > 129 MB of L2
# DRAM bytes (read + write) of one launch of the chosen render on the default
# frame (1920x1080, seed 1), from one ncu capture of that kernel on that frame
# (dram__bytes_read.sum + dram__bytes_write.sum, 1 pass, mean of 2 launches):
# the listed rays' setup (32 B per ray, 66 MB) and the outputs (40 B per
# pixel) mostly stay in L2
RENDER_DRAM_BYTES_FRAME1080 = 20285440 + 598656


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--volume", type=int, default=512, help="edge of the secondary volume sweep (0 = skip)")
    ap.add_argument("--no-jit", action="store_true", help="precompiled kernels only (no run-time specialisation)")
    ap.add_argument("--margins", default="0.25,0.5,0.75,1.0,1.25",
                    help="--report proposal: skip thresholds above the opaque threshold")
    ap.add_argument("--proposal-segment", type=int, default=8, help="--report proposal: samples per segment")
    ap.add_argument("--train-steps", type=int, default=8192, help="--report proposal: Adam steps")
    ap.add_argument("--proposal-grid", type=int, default=0, help="--report proposal: grid cells per axis (0 = 128)")
    ap.add_argument("--proposal-dilate", type=int, default=0, help="--report proposal: 1 = dilate the grid")
    ap.add_argument("--report", choices=["precision", "batch", "proposal"], default=None,
                    help="instead of the benchmark, print the precision form's error report or time the batch")
    ap.add_argument("--batch-scale", type=int, default=1, help="--report batch: divide every image side by this")
    ap.add_argument("--batch-seq", default=None,
                    help="--report batch: every request takes this sequence (the frames of one field)")
    ap.add_argument("--batch-jit-groups", type=int, default=0,
                    help="--report batch: sequence groups compiled for (0: the library's default; -1: none)")
    return ap.parse_args()


# --------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu), "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) >= 9:
                        rows.append(p)
            os.unlink(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        pw = [num(r[3]) for r in rows if num(r[3])]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(values, world, device=None):
    """Element-wise maximum of `values` over the ranks of the default process
    group (the slowest rank's times); `values` itself at world size 1."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def whole_job_rate(world, units_per_step, steps, seconds):
    """Replicas: every rank does `units_per_step` per step, so the job's rate is
    world x units x steps over the slowest rank's time (in G units/s)."""
    return world * units_per_step * steps / seconds / 1e9


# --------------------------------------------------------------- CPU arms
def bench_config(wl, world):
    """The workload as both arms print it (identical dicts: same frame, same
    iteration counts, same timing policy)."""
    return {"workload": wl.name, "width": wl.width, "height": wl.height, "steps_per_ray": int(wl.params.depth),
            "step_method": int(wl.params.stepMethod), "settle": int(wl.params.settle),
            "accum": int(wl.params.accum), "sequence": wl.seq, "box": [float(wl.params.lMin), float(wl.params.lMax)],
            "l2": f"flushed between timed GPU frames ({L2_FLUSH_BYTES >> 20} MiB write)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def cpu_render_rate(wl, seconds, threads=0, fast_math=False, keep=False):
    """The reference algorithm (the oracle's restatement of the reference's own
    arithmetic, ORC_REF; camera, lights and sequence prepared by the oracle's
    restatement of scene.cu too) on the host cores over seeded rows of the
    frame until `seconds` of wall time.  fast_math: the same restatement built
    -O3 -ffast-math (keeping IEEE infinities and NaN, which the ray setup needs).  Returns (G iters/s, description, threads, seconds, rows)
    where rows = [(y, points, counts)] when `keep`, else []."""
    from oracle import ORC_REF, Oracle
    orc = Oracle(fast_math=fast_math)
    if threads:
        orc.set_threads(threads)
    cam = orc.cam_recalculate(wl.cam, wl.width, wl.height, 1)
    lights = orc.lights_recalculate(wl.lights)
    rc, seq = orc.seq_parse(wl.seq)
    if rc != 0:
        raise ValueError(f"sequence {wl.seq!r}: oracle parse status {rc}")
    rows = np.random.default_rng(12345).permutation(wl.height)
    iters, t, done, kept = 0, 0.0, 0, []
    per = wl.params.settle + wl.params.accum
    while done < len(rows) and t < seconds:
        y = int(rows[done])
        t0 = time.perf_counter()
        _, pts, cnt = orc.render(ORC_REF, wl.width, wl.height, cam, wl.params, seq, lights, y0=y, y1=y + 1)
        t += time.perf_counter() - t0
        iters += int(cnt.sum()) * per
        done += 1
        if keep:
            kept.append((y, pts[0], cnt[0]))
    build = "-O3 -ffast-math -fno-finite-math-only" if fast_math else "-O2"
    desc = (f"{done} of {wl.height} rows (seeded permutation) x {wl.width} px of the frame, reference arithmetic "
            f"(double-promoted orbit, logf per step), C restatement built {build}, {orc.threads()} OpenMP threads")
    return iters / t / 1e9, desc, orc.threads(), t, kept


def frame_parity(wl, rows, g_pts, g_cnt):
    """The GPU frame against the reference's arithmetic on the CPU-baseline rows
    (the oracle's ORC_REF, bit-exact to the reference's host build) and
    against FP64 at the GPU frame's hit points in those rows.  Checker only;
    runs after the timed region."""
    from oracle import ORC_F64, ORC_REF, Oracle
    orc = Oracle()
    rc, seq = orc.seq_parse(wl.seq)
    ys = np.array([y for y, _, _ in rows], dtype=np.int64)
    r_pts = np.stack([p for _, p, _ in rows])
    r_cnt = np.stack([c for _, _, c in rows])
    gp, gc = g_pts[ys], g_cnt[ys]
    dec = np.all(gc == r_cnt, axis=-1)
    gh, rh = ~np.isnan(gp["a"]), ~np.isnan(r_pts["a"])
    both = dec & gh & rh
    same_p = both & np.all(gp["P"] == r_pts["P"], axis=-1)
    gl, rl = gp["l"][both].astype(np.float64), r_pts["l"][both].astype(np.float64)
    fin = np.isfinite(gl) & np.isfinite(rl)
    dl = np.abs(gl[fin] - rl[fin])
    # FP64 lambda at the GPU's hit points of those rows (float coordinates, the frame's d)
    P = gp["P"][gh].astype(np.float64)
    pts = np.concatenate([P, np.full((len(P), 1), float(wl.params.d))], axis=1)
    l64 = orc.lyap4d(ORC_F64, pts, wl.params.settle, wl.params.accum, seq)
    lref = orc.lyap4d(ORC_REF, pts, wl.params.settle, wl.params.accum, seq)
    lgpu = gp["l"][gh].astype(np.float64)

    def vs64(v):
        ok = np.isfinite(v) & np.isfinite(l64)
        d = np.abs(v[ok] - l64[ok])
        return {"max_abs": float(d.max()) if d.size else 0.0, "mean_abs": float(d.mean()) if d.size else 0.0,
                "median_abs": float(np.median(d)) if d.size else 0.0,
                "p99_abs": float(np.quantile(d, 0.99)) if d.size else 0.0,
                "nan_mismatch": int((np.isnan(v) != np.isnan(l64)).sum())}
    return {
        "rows": int(len(ys)), "pixels": int(dec.size),
        "vs_reference_arithmetic": {
            "oracle": "ORC_REF (restatement pinned bit-exact to the reference's host build)",
            "decisions_agree": float(dec.mean()),
            "hit_agreement": float((gh == rh).mean()),
            "surface_pixel_agreement": float((gh & rh).sum() / max(1, (gh | rh).sum())),
            "hit_points_identical_where_decisions_agree": float(same_p.sum() / max(1, both.sum())),
            "lambda_at_hits_max_abs": float(dl.max()) if dl.size else 0.0,
            "lambda_at_hits_mean_abs": float(dl.mean()) if dl.size else 0.0},
        "vs_f64_at_gpu_hits": {"hits": int(gh.sum()), "chosen": vs64(lgpu), "reference_arithmetic": vs64(lref)},
    }


def volume_parity(vw, values, idx):
    """lambda of the GPU volume at seeded voxels against FP64 and against the
    reference's arithmetic (oracle), at the kernel's float32 voxel coordinates."""
    from oracle import ORC_F64, ORC_REF, Oracle
    orc = Oracle()
    rc, seq = orc.seq_parse(vw.seq)
    n = vw.n[0]
    x, y, z = idx % n, (idx // n) % n, idx // (n * n)

    def coord(lo, hi, i):
        lo32, hi32 = np.float32(lo), np.float32(hi)
        return lo32 + ((hi32 - lo32) * i.astype(np.float32)) / np.float32(n)
    pts = np.stack([coord(vw.lo[0], vw.hi[0], x), coord(vw.lo[1], vw.hi[1], y), coord(vw.lo[2], vw.hi[2], z),
                    np.full(len(idx), vw.params.d, dtype=np.float32)], axis=1).astype(np.float64)
    l64 = orc.lyap4d(ORC_F64, pts, vw.params.settle, vw.params.accum, seq)
    lref = orc.lyap4d(ORC_REF, pts, vw.params.settle, vw.params.accum, seq)
    v = values.astype(np.float64)

    def diff(a, b):
        ok = np.isfinite(a) & np.isfinite(b)
        d = np.abs(a[ok] - b[ok])
        return {"max_abs": float(d.max()), "mean_abs": float(d.mean()), "median_abs": float(np.median(d)),
                "p99_abs": float(np.quantile(d, 0.99)), "nan_mismatch": int((np.isnan(a) != np.isnan(b)).sum())}
    return {"voxels": int(len(idx)), "chosen_vs_f64": diff(v, l64), "reference_arithmetic_vs_f64": diff(lref, l64),
            "chosen_vs_reference_arithmetic": diff(v, lref)}


def run_reference_arm(args):
    """--impl reference: the reference algorithm on the host cores, same metric.
    Nothing of the product library is loaded: scene preparation and the
    render both run in the oracle's restatement of the reference."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from lyapunov3d_gb300 import scenes
    wl = scenes.full_render(args.seed, args.width, args.height)
    per_step = max(2.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_render_rate(wl, per_step / 4)
    rates, secs = [], 0.0
    desc, threads = "", 0
    for _ in range(args.steps):
        r, desc, threads, t, _ = cpu_render_rate(wl, per_step)
        rates.append(r)
        secs += t
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": "G logistic-iters/s (1080p Lyapunov raymarch frame)", "value": value,
        "unit": "G iters/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene)",
        "config": bench_config(wl, world),
        "cpu_baseline": {"value": value, "unit": "G iters/s", "cores": threads, "kind": "port",
                         "sample": f"per step: {desc}"},
        "e2e": {"value": value, "unit": "G iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "host cores only; the reference's GPU path needs its GL front-end and its sources are not on "
                "this host, so its algorithm runs through the oracle's bit-exact restatement",
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- GPU arm
def run_ours(args):
    import torch
    world, rank, local = dist_env()
    if not torch.cuda.is_available():
        print(json.dumps({"error": "no CUDA device"}))
        sys.exit(1)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    from lyapunov3d_gb300 import capi, scenes
    from lyapunov3d_gb300.device import DeviceFrame, DeviceVolume

    wl = scenes.full_render(args.seed, args.width, args.height)
    frame = DeviceFrame(wl, device=dev)
    jit = not args.no_jit
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed_frames(variant, k, w):
        """w untimed + k timed frames; each frame timed with its own events, L2 flushed between."""
        for _ in range(w):
            frame.run(variant, stream=stream, jit=jit)
        torch.cuda.synchronize()
        frame.reset_stats()
        total_ms = 0.0
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for i in range(k):
            flush.fill_(float(i))
            evs[i][0].record(stream)
            frame.run(variant, stream=stream, jit=jit)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        times = [a.elapsed_time(b) for a, b in evs]
        total_ms = sum(times)
        st = frame.stats()
        return total_ms, times, st

    # pipe-rate probes (the FP32 / MUFU roofline denominators), timed alone
    sink = torch.zeros(4, dtype=torch.float32, device=dev)
    probe = {}
    for kind, name in [(0, "ffma"), (1, "lg2"), (2, "ffma2")]:
        capi.pipe_probe(kind, 64, sink, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ops = capi.pipe_probe(kind, 512, sink, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        probe[name] = ops / (e0.elapsed_time(e1) * 1e-3)   # lane-ops per second

    S, A = wl.params.settle, wl.params.accum
    # plain FP32 drop-in, same frame, same GPU
    barrier()
    plain_ms, plain_times, plain_st = timed_frames(capi.VARIANT_PLAIN, args.steps, args.warmup)
    plain_rgba = frame.d_rgba.clone()
    plain_pts = frame.d_points.clone()
    # chosen form, with clocks sampled during the timed region
    barrier()
    sampler = ClockSampler(local)
    with sampler:
        time.sleep(0.3)
        chosen_ms, chosen_times, chosen_st = timed_frames(capi.VARIANT_PRODUCT, args.steps, args.warmup)
    clocks = sampler.summary()
    barrier()

    iters_frame = frame.iterations(chosen_st) // args.steps
    plain_iters_frame = frame.iterations(plain_st) // args.steps

    # the reference's own entry point and launch shape: kernel_calc_render<<<(W/16, H/16), (16, 16)>>>
    # (plain lambda; the grid covers H/16 whole rows of blocks, as the reference's launch does).
    # Its iterations: the plain frame's per-pixel sample counts over the rows the grid covers.
    gx, gy = wl.width // 16, wl.height // 16
    dropin = None
    if gx and gy:
        cf = DeviceFrame(wl, device=dev, counts=True, stats=False)
        cf.run(capi.VARIANT_PLAIN, stream=stream)
        torch.cuda.synchronize()
        dropin_iters = int(cf.counts()[:gy * 16].sum()) * (S + A)
        del cf

        def dropin_frame():
            capi.kernel_calc_render((gx, gy), (16, 16), frame.d_rgba, frame.d_points, frame.cam, frame.prm,
                                    frame.d_seq, frame.d_lights, len(frame.lights), stream=stream)
        for _ in range(args.warmup):
            dropin_frame()
        torch.cuda.synchronize()
        dts = []
        for i in range(args.steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dropin_frame()
            e1.record(stream)
            torch.cuda.synchronize()
            dts.append(e0.elapsed_time(e1))
        dms = max_over_ranks([statistics.mean(dts)], world, dev)[0]
        dropin = {"kernel": f"kernel_calc_render<<<({gx}, {gy}), (16, 16)>>>", "rows": gy * 16,
                  "value": dropin_iters / (dms * 1e-3) / 1e9 * world, "unit": "G iters/s", "ms_per_step": dms,
                  "frame_ms": [round(t, 4) for t in dts]}

    # surface agreement and lambda difference between the chosen and the plain frame
    pts_c = frame.d_points.view(-1, 9).cpu().numpy()
    pts_p = plain_pts.view(-1, 9).cpu().numpy()
    hit_c, hit_p = ~np.isnan(pts_c[:, 6]), ~np.isnan(pts_p[:, 6])
    surf_px = int((hit_c | hit_p).sum())
    agree = float(((hit_c == hit_p) | ~(hit_c | hit_p)).mean())
    surf_agree = float((hit_c & hit_p).sum() / max(1, surf_px))
    both = hit_c & hit_p & np.isfinite(pts_c[:, 8]) & np.isfinite(pts_p[:, 8])
    dl = np.abs(pts_c[both, 8].astype(np.float64) - pts_p[both, 8])
    lam_diff = {"max_abs": float(dl.max()) if dl.size else 0.0, "mean_abs": float(dl.mean()) if dl.size else 0.0}

    # max over ranks
    t_chosen, t_plain = max_over_ranks([chosen_ms, plain_ms], world, dev)

    value = whole_job_rate(world, iters_frame, args.steps, t_chosen * 1e-3)
    plain_value = whole_job_rate(world, plain_iters_frame, args.steps, t_plain * 1e-3)
    kernel_ms = statistics.mean(chosen_times)
    achieved = iters_frame / (kernel_ms * 1e-3) / 1e9
    # FP32-pipe bound of the chosen (product) form: 2 FP32 ops per settle step,
    # 4 per accumulated step, at the higher of the two measured FP32 rates (the
    # packed FFMA2 probe: scalar FFMA needs an issue slot per 32 lane-ops and
    # stops short of the pipe); the plain form is MUFU-bound at one lg2 per
    # accumulated step
    fp32_rate = max(probe["ffma"], probe["ffma2"])
    peak_fp32 = fp32_rate * (S + A) / (2 * S + 4 * A) / 1e9
    peak_plain = min(probe["lg2"] * (S + A) / A, probe["ffma"] * (S + A) / (2 * S + 4 * A)) / 1e9
    plain_achieved = plain_iters_frame / (statistics.mean(plain_times) * 1e-3) / 1e9

    # end to end through the host-buffer entry point
    e2e = None
    if not args.no_e2e:
        npix = wl.width * wl.height
        rgba_h = torch.empty(npix * 4, dtype=torch.uint8, pin_memory=True).numpy().reshape(wl.height, wl.width, 4)
        pts_h = torch.empty(npix * 9, dtype=torch.float32, pin_memory=True).numpy()
        from lyapunov3d_gb300.types import POINT_DTYPE
        pts_h = pts_h.view(POINT_DTYPE).reshape(wl.height, wl.width)
        ext = capi.LyapRenderExt(variant=capi.VARIANT_PRODUCT, light_model=frame.light_model,
                                 flags=capi.FLAG_NO_JIT if args.no_jit else 0)
        for _ in range(max(1, args.warmup)):
            capi.render_host(frame.cam, frame.prm, frame.seq, frame.lights, wl.width, wl.height, ext=ext,
                             stream=stream, rgba=rgba_h, points=pts_h)
        e2e_s = 0.0
        for i in range(args.steps):
            flush.fill_(float(i))
            torch.cuda.synchronize()
            barrier()
            t0 = time.perf_counter()
            capi.render_host(frame.cam, frame.prm, frame.seq, frame.lights, wl.width, wl.height, ext=ext,
                             stream=stream, rgba=rgba_h, points=pts_h)
            e2e_s += time.perf_counter() - t0
        e2e_s = max_over_ranks([e2e_s], world, dev)[0]
        e2e = {"value": whole_job_rate(world, iters_frame, args.steps, e2e_s), "unit": "G iters/s",
               "h2d_bytes_per_step": int(frame.seq.nbytes + 224 * len(frame.lights)),
               "d2h_bytes_per_step": int(npix * 4 + npix * 36),
               "frames_per_s": world * args.steps / e2e_s,
               "call": "lyap_render_host (pinned host buffers; upload, render, download RGBA + LyapPoint, sync)"}

    # how much of one frame is spent after the pixel queue drained (the tail)
    frame.reset_stats()
    frame.run(capi.VARIANT_PRODUCT, stream=stream, jit=jit)
    torch.cuda.synchronize()
    tst = frame.stats()
    mask = (1 << 64) - 1
    t_start, t_drain, t_end = (~int(tst[capi.STAT_T_START])) & mask, (~int(tst[capi.STAT_T_DRAIN])) & mask, \
        int(tst[capi.STAT_T_END])
    tail = {"frame_ms": (t_end - t_start) / 1e6, "after_queue_drained_ms": (t_end - t_drain) / 1e6,
            "tail_frac": (t_end - t_drain) / max(1, t_end - t_start)} if t_end > t_drain > t_start else None

    # secondary: the dense volume sweep (HBM write-out roofline)
    volume = vol_sample = None
    if args.volume > 0:
        vw = scenes.full_volume(args.volume, args.seed)
        vol = DeviceVolume(vw, device=dev)
        vol.run(capi.VARIANT_PRODUCT, stream=stream, jit=jit)
        vol.run(capi.VARIANT_PLAIN, stream=stream, jit=jit)
        torch.cuda.synchronize()
        vol.reset_stats()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(2)]
        for variant, (e0, e1) in zip([capi.VARIANT_PRODUCT, capi.VARIANT_PLAIN], evs):
            flush.fill_(0.0)
            e0.record(stream)
            vol.run(variant, stream=stream, jit=jit)
            e1.record(stream)
        torch.cuda.synchronize()
        tp, tq = evs[0][0].elapsed_time(evs[0][1]), evs[1][0].elapsed_time(evs[1][1])
        n = args.volume ** 3
        vit = n * (S + A)
        peaks, src = measured_peaks()
        volume = {"workload": vw.name, "voxels": n, "product_ms": tp, "plain_ms": tq,
                  "product_g_iters_s": vit / (tp * 1e-3) / 1e9, "plain_g_iters_s": vit / (tq * 1e-3) / 1e9,
                  "product_fp32_frac": vit / (tp * 1e-3) / 1e9 / peak_fp32,
                  "plain_mufu_frac": vit / (tq * 1e-3) / 1e9 / peak_plain,
                  "write_gbs": n * 4 / (tp * 1e-3) / 1e9,
                  "write_frac_of_hbm": n * 4 / (tp * 1e-3) / 1e9 / peaks["hbm_gbs"]}
        vidx = np.random.default_rng(512).choice(n, 8192, replace=False).astype(np.int64)
        vol.run(capi.VARIANT_PRODUCT, stream=stream, jit=jit)
        torch.cuda.synchronize()
        vol_sample = (vw, vol.d_out[torch.from_numpy(vidx).to(dev)].cpu().numpy(), vidx)
        del vol
        if not args.no_e2e:
            # end to end through lyap_volume_host into a page-locked host array (written in place)
            pin = torch.empty(n * 4, dtype=torch.uint8, pin_memory=True)
            out_h = pin.numpy().view(np.float32).reshape(args.volume, args.volume, args.volume)
            vext = capi.LyapVolumeExt(variant=capi.VARIANT_PRODUCT, flags=capi.FLAG_NO_JIT if args.no_jit else 0)
            capi.volume_host(args.volume, args.volume, args.volume, vw.params, capi.seq_parse(vw.seq), lo=vw.lo,
                             hi=vw.hi, ext=vext, stream=stream, out=out_h)
            hts = []
            for i in range(3):
                flush.fill_(float(i))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                capi.volume_host(args.volume, args.volume, args.volume, vw.params, capi.seq_parse(vw.seq),
                                 lo=vw.lo, hi=vw.hi, ext=vext, stream=stream, out=out_h)
                hts.append(time.perf_counter() - t0)
            volume["e2e"] = {"call": "lyap_volume_host (page-locked output, written in place)",
                             "ms": 1e3 * statistics.mean(hts),
                             "g_iters_s": vit / statistics.mean(hts) / 1e9, "d2h_bytes": n * 4}
            del pin, out_h

    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, desc, threads, t, kept = cpu_render_rate(wl, args.cpu_seconds, keep=True)
        rf, descf, _, tf, _ = cpu_render_rate(wl, args.cpu_seconds / 2, fast_math=True)
        cpu = {"value": r, "unit": "G iters/s", "cores": threads, "kind": "port",
               "sample": desc + f" ({t:.1f} s)",
               "fast_math": {"value": rf, "unit": "G iters/s", "sample": descf + f" ({tf:.1f} s)"}}
        # the checker, after the timed region: the CPU rows against the chosen frame
        pf = DeviceFrame(wl, device=dev, counts=True, stats=False)
        pf.run(capi.VARIANT_PRODUCT, stream=stream, jit=jit)
        torch.cuda.synchronize()
        parity = {"frame": frame_parity(wl, kept, pf.points(), pf.counts())}
        del pf
        if vol_sample is not None:
            parity["volume"] = volume_parity(*vol_sample)

    default_frame = (args.seed, wl.width, wl.height) == (1, 1920, 1080)
    if rank == 0:
        line = {
            "metric": "G logistic-iters/s (1080p Lyapunov raymarch frame)",
            "value": value, "unit": "G iters/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_chosen / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene)",
            "config": bench_config(wl, world),
            "form": "product (renormalised FP32 product, one log2 per sample), kernel specialised for the sequence",
            "frames_per_s": world * args.steps / (t_chosen * 1e-3),
            "frame_ms": [round(t, 4) for t in chosen_times],
            "iters_per_frame": iters_frame,
            "samples_per_frame": int(chosen_st[capi.STAT_SAMPLES]) // args.steps,
            "hits_per_frame": int(chosen_st[capi.STAT_HITS]) // args.steps,
            "queue_tail": tail,
            "warp_rounds": {"lane_utilisation": float(chosen_st[capi.STAT_LANE_ROUNDS]) /
                                                max(1.0, 32.0 * float(chosen_st[capi.STAT_ROUNDS])),
                            "rounds_per_frame": int(chosen_st[capi.STAT_ROUNDS]) // args.steps,
                            "max_rounds_one_warp": int(chosen_st[capi.STAT_MAX_ROUNDS]),
                            "speculative_samples": int(chosen_st[capi.STAT_SPEC]) // args.steps,
                            "speculative_used": int(chosen_st[capi.STAT_SPEC_USED]) // args.steps},
            "plain": {"value": plain_value, "unit": "G iters/s", "ms_per_step": t_plain / args.steps,
                      "frame_ms": [round(t, 4) for t in plain_times],
                      "frames_per_s": world * args.steps / (t_plain * 1e-3),
                      "roofline_frac": plain_achieved / peak_plain},
            "speedup_vs_plain": value / plain_value,
            "dropin_reference_launch": dropin,
            "speedup_vs_dropin_reference_launch": value / dropin["value"] if dropin else None,
            "surface": {"pixel_agreement": agree, "surface_pixel_agreement": surf_agree,
                        "lambda_at_hits_vs_plain": lam_diff},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32, "unit": "G iters/s",
                         "frac": achieved / peak_fp32,
                         "traffic": RENDER_DRAM_BYTES_FRAME1080 if default_frame else None,
                         "traffic_unit": "DRAM bytes per launch (ncu capture of this frame)",
                         "algorithmic_bytes": 40 * wl.width * wl.height,
                         "peak_source": "measured live: the higher of the FFMA and packed FFMA2 pipe-rate probes "
                                        "(lyap_pipe_probe) x (S+A)/(2S+4A) FP32 ops per iteration",
                         "probe_ffma_tops": probe["ffma"] / 1e12, "probe_ffma2_tops": probe["ffma2"] / 1e12,
                         "probe_lg2_tops": probe["lg2"] / 1e12,
                         "kernel": "render_persistent<MODE_PRODUCT>"},
            "e2e": e2e,
            "volume": volume,
            "cpu_baseline": cpu,
            "parity": parity,
            # per timed frame: ray_list (the pre-pass) and render_persistent
            "gpu_launches": 2 * args.steps,
            "jit": capi.jit_info()[1].split("\n")[0] if jit else "off",
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_precision_report(args):
    """The precision form on the CPU-runnable workload (ABC, 20 + 100, [2.5, 4]^3):
    lambda of the plain and product forms at 2^20 seeded points against the
    FP64 form (lambda in double on the GPU, which tests/test_gpu_precision.py
    holds to the FP64 oracle within 1e-14); a 128^2 frame rendered with the
    product form and FP64 bisection (20 halvings) of every crossing, its
    hit-point lambdas against the FP64 form, and its surface agreement with
    the plain frame."""
    import torch
    from lyapunov3d_gb300 import capi, scenes
    from lyapunov3d_gb300.device import DeviceFrame
    dev = torch.device("cuda", 0)
    wl = scenes.small_render(128)
    prm = wl.params
    seq = capi.seq_parse(wl.seq)
    d_seq = torch.from_numpy(seq).to(dev)
    n = 1 << 20
    pts = np.random.default_rng(20240).uniform(prm.lMin, prm.lMax, size=(n, 3)).astype(np.float32)
    d_xyz = torch.from_numpy(pts.reshape(-1)).to(dev)
    o64 = torch.empty(n, dtype=torch.float64, device=dev)
    capi.lambda_points(d_xyz, n, prm, d_seq, seq.size, capi.FORM_F64, o64)
    ref = o64.cpu().numpy()
    fin = np.isfinite(ref)

    def stats(got):
        g = got.astype(np.float64)
        ok = fin & np.isfinite(g)
        d = np.abs(g[ok] - ref[ok])
        return {"max_abs": float(d.max()), "mean_abs": float(d.mean()), "median_abs": float(np.median(d)),
                "p99_abs": float(np.quantile(d, 0.99)), "nan_mismatch": int((np.isnan(g) != np.isnan(ref)).sum())}
    out = {}
    o32 = torch.empty(n, dtype=torch.float32, device=dev)
    for name, form in [("plain", capi.VARIANT_PLAIN), ("product", capi.VARIANT_PRODUCT)]:
        capi.lambda_points(d_xyz, n, prm, d_seq, seq.size, form, o32)
        out[name] = stats(o32.cpu().numpy())

    f = DeviceFrame(wl, device=dev, counts=True)
    f.run(capi.VARIANT_PLAIN)
    plain_pts = f.points().copy()
    f.reset_stats()
    f.run(capi.VARIANT_PRODUCT, flags=capi.FLAG_BISECT_F64, bisect_halvings=20)
    torch.cuda.synchronize()
    pp = f.points()
    hit, phit = ~np.isnan(pp["a"]), ~np.isnan(plain_pts["a"])
    P = np.ascontiguousarray(pp["P"][hit].astype(np.float32))
    d_P = torch.from_numpy(P.reshape(-1)).to(dev)
    h64 = torch.empty(len(P), dtype=torch.float64, device=dev)
    hp = torch.empty(len(P), dtype=torch.float32, device=dev)
    capi.lambda_points(d_P, len(P), prm, d_seq, seq.size, capi.FORM_F64, h64)
    capi.lambda_points(d_P, len(P), prm, d_seq, seq.size, capi.VARIANT_PRODUCT, hp)
    href = h64.cpu().numpy()
    hp = hp.cpu().numpy().astype(np.float64)
    ok = np.isfinite(href) & np.isfinite(hp)
    stored = pp["l"][hit].astype(np.float64)
    ok2 = np.isfinite(href) & np.isfinite(stored)
    report = {
        "workload": wl.name, "points": n, "reference": "FP64 form on the GPU (lyap_lambda_points, LYAP_FORM_F64)",
        "lambda_vs_f64_at_points": out,
        "frame": {"pixels": int(hit.size), "hits": int(hit.sum()), "plain_hits": int(phit.sum()),
                  "surface_pixel_agreement_vs_plain": float((hit == phit).mean()),
                  "hit_lambda_product_vs_f64": {"max_abs": float(np.abs(hp[ok] - href[ok]).max()),
                                                "mean_abs": float(np.abs(hp[ok] - href[ok]).mean())},
                  "hit_lambda_stored_vs_f64": {"max_abs": float(np.abs(stored[ok2] - href[ok2]).max())},
                  "halvings": 20},
    }
    print(json.dumps(report), flush=True)


def run_batch_report(args):
    """The batched workload (scenes.batch_workloads: 256 frames + 32 4-D slices,
    sides divided by --batch-scale) as one autotuned, graph-captured launch,
    product form: device time per launch, plain-method iterations per second,
    the tuner's choice and candidate times."""
    import torch
    from lyapunov3d_gb300 import capi, scenes
    from lyapunov3d_gb300.device import DeviceBatch
    dev = torch.device("cuda", 0)
    wls = scenes.batch_workloads(seed=4, scale=args.batch_scale, one_seq=args.batch_seq)
    jit = {"flags": capi.FLAG_NO_JIT} if args.batch_jit_groups < 0 else {"jit_groups": args.batch_jit_groups}
    t0 = time.perf_counter()
    db = DeviceBatch(wls, device=dev, variant=capi.VARIANT_PRODUCT, autotune=True, counts=True, **jit)
    t_create = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    db.run(stream)
    torch.cuda.synchronize()
    iters = db.iterations()
    times = []
    for _ in range(max(1, args.steps)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        db.run(stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    info = db.batch.info()
    ms = statistics.mean(times)
    db.d_stats.zero_()
    db.run(stream)
    torch.cuda.synchronize()
    st = db.stats()
    print(json.dumps({
        "report": "batch", "requests": len(wls), "pixels": sum(w.width * w.height for w in wls),
        "scale": args.batch_scale, "one_sequence": args.batch_seq,
        "sequence_groups": len({(w.seq, w.params.settle % len(w.seq)) for w in wls}),
        "jit_groups": args.batch_jit_groups, "specialised_requests": int(info.specialised),
        "create_s": t_create, "ms_per_launch": ms, "launch_ms": times,
        "plain_iters_per_launch": iters, "g_iters_per_s": iters / (ms * 1e-3) / 1e9,
        "tuned": {"tile": [info.tile_w, info.tile_h], "tiles_per_chunk": info.tiles_per_chunk,
                  "blocks_per_sm": info.blocks_per_sm, "candidates_ms": list(info.tuned_ms)[:info.candidates]},
        "chunks": info.chunks,
        "one_launch": {"samples": int(st[capi.STAT_SAMPLES]), "rays": int(st[capi.STAT_RAYS]),
                       "rounds": int(st[capi.STAT_ROUNDS]),
                       "lane_utilisation": float(st[capi.STAT_LANE_ROUNDS]) / max(1.0, 32.0 * float(st[capi.STAT_ROUNDS])),
                       "max_rounds_one_warp": int(st[capi.STAT_MAX_ROUNDS]),
                       "speculative_used": int(st[capi.STAT_SPEC_USED])}}), flush=True)


def run_proposal_report(args):
    """The learned proposal on the 1080p frame (scenes.full_render): the net
    trained on the GPU (2^20 plain-method lambda samples; its kernels'
    gradients are checked against the CPU oracle in tests/test_gpu_net.py),
    its grid over the box built once (the minimum of the net at each cell's
    corners), then the product-form frame with the proposal at each margin
    against the same frame without it (and with an untrained net at the same
    margins): device time, lambda samples evaluated, skipped positions,
    rewound runs, surface agreement (pixels hit in both / hit by the exact
    march) and same-sample agreement (hit at the bit-identical point)."""
    import ctypes
    import torch
    from lyapunov3d_gb300 import capi, scenes
    from lyapunov3d_gb300.device import DeviceFrame
    dev = torch.device("cuda", 0)
    wl = scenes.full_render(args.seed, args.width, args.height)
    seq = capi.seq_parse(wl.seq)
    t0 = time.perf_counter()
    net, loss = capi.net_train(wl.params, seq, steps=args.train_steps, seed=args.seed, with_loss=True)
    t_train = time.perf_counter() - t0
    untrained = capi.net_train(wl.params, seq, steps=1, seed=args.seed)
    frame = DeviceFrame(wl, device=dev, counts=False)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    # the grid: built once per net (timed here on its own), then cached by the library
    n = args.proposal_grid or capi.PROPOSAL_GRID_DEFAULT
    d_grid = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    capi.net_grid(net, n, args.proposal_dilate, d_grid, stream=stream)
    torch.cuda.synchronize()
    t_grid = time.perf_counter() - t0

    def timed(**kw):
        for _ in range(max(1, args.warmup)):
            frame.run(capi.VARIANT_PRODUCT, stream=stream, jit=True, **kw)
        torch.cuda.synchronize()
        frame.reset_stats()
        ts = []
        for i in range(max(1, args.steps)):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            frame.run(capi.VARIANT_PRODUCT, stream=stream, jit=True, **kw)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts), frame.stats() // max(1, args.steps), frame.d_points.view(-1, 9).cpu().numpy()

    mask64 = (1 << 64) - 1

    def kernel_times(st):
        """the render launch's own span and its share after the queue drained (%globaltimer)"""
        t0_, td, te = (~int(st[capi.STAT_T_START])) & mask64, (~int(st[capi.STAT_T_DRAIN])) & mask64, \
            int(st[capi.STAT_T_END])
        if not te > td > t0_:
            return {}
        return {"kernel_ms": (te - t0_) / 1e6, "after_drain_ms": (te - td) / 1e6,
                "rounds": int(st[capi.STAT_ROUNDS]),
                "lane_utilisation": float(st[capi.STAT_LANE_ROUNDS]) / max(1.0, 32.0 * float(st[capi.STAT_ROUNDS]))}

    def timed_kernel(**kw):
        """one more frame with the statistics of that frame alone (start / drain / end stamps)"""
        frame.reset_stats()
        frame.run(capi.VARIANT_PRODUCT, stream=stream, jit=True, **kw)
        torch.cuda.synchronize()
        return kernel_times(frame.stats())

    ms0, st0, p0 = timed()
    k0 = timed_kernel()
    hit0 = ~np.isnan(p0[:, 0])
    rows = []
    for which, nt in (("trained", net), ("untrained", untrained)):
        for m in (float(x) for x in args.margins.split(",")):
            kw = dict(proposal=ctypes.pointer(nt), proposal_margin=m, proposal_segment=args.proposal_segment,
                      proposal_grid=n, proposal_dilate=args.proposal_dilate)
            ms, st, p1 = timed(**kw)
            kt = timed_kernel(**kw)
            hit1 = ~np.isnan(p1[:, 0])
            same = hit0 & hit1 & (p0[:, :3].view(np.uint32) == p1[:, :3].view(np.uint32)).all(1)
            rows.append({"net": which, "margin": m, "ms": ms, "speedup": ms0 / ms,
                         "samples_evaluated_frac": float(st[capi.STAT_SAMPLES] / st0[capi.STAT_SAMPLES]),
                         "positions_skipped": int(st[capi.STAT_PROPOSAL_SKIPPED]),
                         "runs_rewound": int(st[capi.STAT_PROPOSAL_REWOUND]),
                         "net_timeouts": int(st[capi.STAT_NET_TIMEOUTS]),
                         "surface_agreement": float(hit1.sum() / max(1, hit0.sum())),
                         "same_sample_agreement": float(same.sum() / max(1, hit0.sum())),
                         "extra_hits": int((hit1 & ~hit0).sum()), "kernel": kt})
    print(json.dumps({
        "report": "proposal", "workload": wl.name, "width": wl.width, "height": wl.height,
        "train": {"seconds": t_train, "steps": net.steps, "batch": net.batch, "samples": net.n_samples,
                  "train_mse": net.train_mse, "val_mse": net.val_mse,
                  "loss_first10": float(np.mean(loss[:10])), "loss_last100": float(np.mean(loss[-100:]))},
        "grid": {"cells_per_axis": n, "dilate": args.proposal_dilate, "build_s": t_grid,
                 "net_points": (n + 1) ** 3},
        "segment": args.proposal_segment,
        "without_proposal": {"ms": ms0, "samples": int(st0[capi.STAT_SAMPLES]), "hits": int(hit0.sum()),
                             "kernel": k0},
        "with_proposal": rows}), flush=True)


def main():
    args = parse_args()
    if args.report == "proposal":
        run_proposal_report(args)
        return
    if args.report == "precision":
        run_precision_report(args)
        return
    if args.report == "batch":
        run_batch_report(args)
        return
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
