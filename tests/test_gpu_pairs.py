"""The specialised render with paired rounds (two samples per lane per round
on packed FP32 pairs, the default) and with one sample per lane
(LYAP_JIT_PAIRS=0, read once per process) gives the same frame, bit for bit,
as the precompiled render."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from lyapunov3d_gb300 import capi, scenes
from lyapunov3d_gb300.device import DeviceFrame
for wl in (scenes.full_render(1, 320, 180), scenes.small_render(64)):
    f = DeviceFrame(wl, counts=True)
    out = []
    for variant in (capi.VARIANT_PLAIN, capi.VARIANT_PRODUCT):
        for jit in (False, True):
            f.run(variant, jit=jit)
            torch.cuda.synchronize()
            out.append((f.rgba().tobytes(), f.points().tobytes(), f.counts().tobytes()))
    assert out[0] == out[1] and out[2] == out[3], wl.name
ok, info = capi.jit_info()
assert ok and "compiled=" in info
print("PAIRS-OK")
"""


@pytest.mark.parametrize("pairs", ["1", "0"])
def test_paired_rounds_bit_identical(pairs):
    pytest.importorskip("torch")
    env = dict(os.environ, LYAP_JIT_PAIRS=pairs)
    r = subprocess.run([sys.executable, "-c", SCRIPT, ROOT], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "PAIRS-OK" in r.stdout, r.stderr[-3000:]
