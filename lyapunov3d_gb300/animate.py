"""The reference's animation driver (scale.pl) on the batched renderer.

scale.pl sweeps t = 0, 0.01, ... while t <= 1.00001, eases it
(easeInOutQuart, scale.pl:5-11), writes the eased value into params.cu's
camera block and re-runs the one-frame renderer once per value.  Here the
same camera path (lyap_anim_camera: the params_init camera block at the
eased value) is rendered as one batch -- every frame a request of a single
graph-captured launch (lyap_batch) -- and each frame is written as the
reference names it (Render_<time>_<w>x<h>_<seq>_cx=..._time=...ppm).

    python -m lyapunov3d_gb300.animate [--width W] [--height H] [--out-dir DIR]
        [--variant plain|product] [--binary] [--first K] [--last K] [-n]

-n prints scale.pl's "t<TAB>i" lines without rendering.
"""
import argparse
import os
import sys
import time

from . import capi
from .scenes import RenderWorkload


def path_values(step=0.01, limit=1.00001):
    """(t, eased i) for every frame, t accumulated in double as scale.pl does."""
    out, t = [], 0.0
    while t <= limit:
        out.append((t, capi.ease_in_out_quart(t, 0.0, 1.0, 1.0)))
        t += step
    return out


def frame_workloads(width, height, values, light_model=capi.LIGHT_SPOT):
    """One RenderWorkload per eased value, on the params_init preset."""
    prm, cam, lights, seq, _ = capi.params_init()
    wls = []
    for k, (_, i) in enumerate(values):
        c = capi.anim_camera(i, cam)
        wls.append(RenderWorkload(f"anim{k:03d}", width, height, seq, prm, c, lights, light_model))
    return wls


def render_path(width, height, values, variant=capi.VARIANT_PLAIN, autotune=False):
    """Render the frames of `values` as one batch; returns (workloads, frames, seconds)."""
    import torch
    from .device import DeviceBatch
    wls = frame_workloads(width, height, values)
    batch = DeviceBatch(wls, variant=variant, autotune=autotune)
    t0 = time.time()
    batch.run()
    torch.cuda.synchronize()
    return wls, batch.frames, time.time() - t0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--width", type=int, default=384)
    ap.add_argument("--height", type=int, default=216)
    ap.add_argument("--out-dir", default=".")
    ap.add_argument("--variant", choices=["plain", "product"], default="plain")
    ap.add_argument("--binary", action="store_true", help="P6 instead of the reference's P3")
    ap.add_argument("--first", type=int, default=0)
    ap.add_argument("--last", type=int, default=None)
    ap.add_argument("-n", action="store_true", help="print the path only (scale.pl -n)")
    a = ap.parse_args(argv)
    values = path_values()[a.first:(a.last + 1 if a.last is not None else None)]
    if a.n:
        for t, i in values:
            print(f"{t}\t{i}")
        return 0
    stamp = int(time.time())
    variant = capi.VARIANT_PRODUCT if a.variant == "product" else capi.VARIANT_PLAIN
    wls, frames, secs = render_path(a.width, a.height, values, variant)
    os.makedirs(a.out_dir, exist_ok=True)
    for wl, f in zip(wls, frames):
        name = capi.output_name("Render", stamp, a.width, a.height, wl.seq, f.cam, f.prm, int(secs), "ppm")
        capi.write_ppm(os.path.join(a.out_dir, name), f.rgba(), binary=a.binary)
        print(name)
    print(f"{len(frames)} frames of {a.width}x{a.height} in one batch: {secs:.3f} s", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
