"""bench.py's multi-GPU logic (replicas: no data-path collective) on two gloo
ranks on the CPU: the slowest rank's times decide, the job's rate counts every
rank's work, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_env()
        times = bench.max_over_ranks([10.0 + rank, 20.0 - rank, 0.5 * rank], w)
        out.put((r, w, times))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for _, w, times in got:
        assert w == 2
        assert times == [11.0, 20.0, 0.5]


def test_whole_job_rate_and_single_rank():
    import bench
    assert bench.max_over_ranks([3.0, 4.0], 1) == [3.0, 4.0]
    # 2 replicas, 1e9 iterations per frame, 5 frames in 2.5 s on the slowest rank
    assert bench.whole_job_rate(2, 1e9, 5, 2.5) == pytest.approx(4.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    bench.run_reference_arm(bench.parse_args())
    assert capsys.readouterr().out == ""


def test_reference_arm_json_line():
    """--impl reference on a small frame prints one JSON line with the keys a
    bench line carries: the metric and unit of the GPU arm, a cpu_baseline
    describing the run, and an e2e object with no host-device traffic."""
    import json
    import subprocess
    # run bench.py as __main__, then report which of this repository's shared
    # libraries the process loaded: the reference arm must not load the product's
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--width', '64', '--height', '36', "
            "'--steps', '1', '--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('LOADED', sorted({l.split()[-1].rsplit('/', 1)[-1] for l in open('/proc/self/maps') "
            "if l.rstrip().endswith('.so') and 'lyap' in l}))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT,
                       env={k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")})
    assert r.returncode == 0, r.stderr[-2000:]
    loaded = [l for l in r.stdout.splitlines() if l.startswith("LOADED")]
    assert loaded and "liblyap_gb300.so" not in loaded[0] and "liblyap_oracle.so" in loaded[0], loaded
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    # the same config dict as the GPU arm prints for this frame
    import bench
    from lyapunov3d_gb300 import scenes
    assert d["config"] == json.loads(json.dumps(bench.bench_config(scenes.full_render(1, 64, 36), 1)))
    assert d["impl"] == "reference"
    assert d["metric"] == "G logistic-iters/s (1080p Lyapunov raymarch frame)" and d["unit"] == "G iters/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 1
    assert d["config"]["width"] == 64 and d["config"]["height"] == 36
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "G iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
