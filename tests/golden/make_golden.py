#!/usr/bin/env python3
"""Regenerate the golden fixtures from the reference's OWN code.

Runs `make -C oracle ref` (the reference's kernel.cu / scene.cu / params.cu
compiled as host C++ from the reference checkout: LYAP_REF=..., else a
checkout named `reference` beside this repository) and records what that build computes for seeded
inputs.  The fixtures pin the oracle restatement (tests/test_oracle_golden.py)
and are compared with the CUDA path on the GPU (tests/test_gpu_parity.py).

    python tests/golden/make_golden.py

Nothing here is needed at test time: the .npz files are committed.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lyapunov3d_gb300 import scenes  # noqa: E402
from lyapunov3d_gb300.types import LyapCam, LyapCamD, LyapLight, LyapParams, struct_to_bytes  # noqa: E402
from oracle import Reference, params_to_double  # noqa: E402

SEQ_CASES = ["A", "AB", "ABC", "BCABA", "abc", "A3B", "A6B6C6D6", "9", "1A", "dcba",
             "AABAB", "C9", "ABCD2", "bbbbbbbbbbbbbbbb"]


def cam_to_double(c):
    d = LyapCamD()
    for name, _ in LyapCam._fields_:
        if name.startswith("_pad"):
            continue
        v = getattr(c, name)
        if hasattr(v, "_fields_"):
            dv = getattr(d, name)
            for f, _ in v._fields_:
                setattr(dv, f, getattr(v, f))
        else:
            setattr(d, name, v)
    return d


def b(s):
    return np.frombuffer(struct_to_bytes(s), dtype=np.uint8).copy()


def main():
    ref_dir = os.environ.get("LYAP_REF") or os.path.join(os.path.dirname(ROOT), "reference")
    if not os.path.isfile(os.path.join(ref_dir, "kernel.cu")):
        sys.exit(f"make_golden: no reference checkout at {ref_dir} (set LYAP_REF=<checkout>)")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref_dir}"], check=True)
    R32, R64 = Reference("f32"), Reference("f64")
    out = {}
    meta = {"layout_f32": R32.layout(), "layout_f64": R64.layout(), "seq": {}}

    # scene_convert_sequence (scene.cu:69)
    for s in SEQ_CASES:
        meta["seq"][s] = R32.seq_parse(s).tolist()

    # params_init (params.cu:21) preset, both widths
    prm, cam, lights, seqs, (w, h) = R32.params_init()
    out["preset_prm"], out["preset_cam"] = b(prm), b(cam)
    out["preset_lights"] = np.concatenate([b(l) for l in lights])
    meta["preset"] = {"seq": seqs, "n_lights": len(lights), "width": w, "height": h}
    prmd, camd, lightsd, _, _ = R64.params_init()
    out["preset_prm_d"], out["preset_cam_d"] = b(prmd), b(camd)
    out["preset_lights_d"] = np.concatenate([b(l) for l in lightsd])

    # scene_cam_recalculate / scene_lights_recalculate (scene.cu:20-63)
    rng = scenes.SplitMix64(20260101)
    cams_in, cams_out, cams_out_d, dims = [], [], [], []
    for k in range(24):
        q = scenes.uniform_quaternion(rng)
        scale = 1.0 if k % 3 else rng.uniform(0.5, 1.5)   # non-unit quaternions too (H9)
        q = tuple(x * scale for x in q)
        c = scenes.orbit_camera(q, (2.0, 2.0, 2.0), rng.uniform(2.0, 9.0), M=rng.uniform(1e-7, 1.5))
        tw, th, td = [(64, 64, 1), (1920, 1080, 1), (3840, 2160, 2), (128, 96, 4)][k % 4]
        cams_in.append(b(c))
        cams_out.append(b(R32.cam_recalculate(c, tw, th, td)))
        cams_out_d.append(b(R64.cam_recalculate(cam_to_double(c), tw, th, td)))
        dims.append((tw, th, td))
    out["cams_in"], out["cams_out"], out["cams_out_d"] = map(np.stack, (cams_in, cams_out, cams_out_d))
    out["cams_dims"] = np.array(dims, dtype=np.uint32)
    lights_in = [scenes.headlight(scenes.orbit_camera(scenes.uniform_quaternion(rng), (2, 2, 2), 4.0), M=rng.uniform(0.1, 3))
                 for _ in range(8)]
    out["lights_in"] = np.stack([b(l) for l in lights_in])
    out["lights_out"] = np.stack([b(l) for l in R32.lights_recalculate(lights_in)])
    out["lights_out_d"] = np.stack([b(l) for l in R64.lights_recalculate([cam_to_double(l) for l in lights_in])])

    # lyap4d (kernel.cu:108) at seeded points
    lam_cases = [("BCABA", 18, 1008, 0.0, 4.0), ("ABC", 20, 100, 2.5, 4.0), ("A3B", 0, 7, 0.0, 4.0),
                 ("ABCD2", 200, 1000, 2.0, 4.0), ("AB", 600, 40, 0.0, 4.5)]
    for i, (s, st, ac, lo, hi) in enumerate(lam_cases):
        pr = scenes.SplitMix64(777 + i)
        pts = np.column_stack([pr.uniform_array(2048 * 3, lo, hi).reshape(-1, 3), pr.uniform_array(2048, lo, hi)])
        seq = R32.seq_parse(s)
        out[f"lam{i}_pts"] = pts
        out[f"lam{i}_f32"] = R32.lyap4d(pts, st, ac, seq)
        out[f"lam{i}_f64"] = R64.lyap4d(pts, st, ac, seq)
    meta["lam_cases"] = lam_cases

    # kernel_calc_render (kernel.cu:500) on small grids of 16x16 blocks
    render_cases = []
    # (a) the params_init preset with lighter iteration counts (jitter, honing, near switch, 2 steps)
    p = R32.params_init()[0]
    p.accum, p.depth = 200, 512.0
    c = R32.cam_recalculate(cam, 64, 64, 1)
    render_cases.append(("preset64", 64, 64, c, p, seqs, R32.lights_recalculate(lights)))
    # (b) the 128^2 workload's scene in the reference's fixed [0, 4]^3 box at 64^2
    wl = scenes.small_render()
    p = wl.params
    p.lMin, p.lMax = 0.0, 4.0
    wl.cam.C.x, wl.cam.C.y, wl.cam.C.z = (2.0 - 6.0 * v for v in scenes.quat_rotate(tuple(wl.cam.Q), (0, 0, 1)))
    c = R32.cam_recalculate(wl.cam, 64, 64, 1)
    render_cases.append(("abc64", 64, 64, c, p, "ABC", R32.lights_recalculate(wl.lights)))
    # (c) camera inside the box, honing on, jitter, near switch, method 1
    q = scenes.uniform_quaternion(scenes.SplitMix64(99))
    ci = scenes.orbit_camera(q, (2.2, 2.9, 3.1), 0.3, M=0.8)
    p = scenes.make_params(30, 150, step_method=1, depth=96.0, opaque=-0.2, near=0.1, near_mul=3.0,
                           chaos=0.2, jitter=0.3, refine=16.0, gradient=0.02)
    c = R32.cam_recalculate(ci, 48, 32, 1)
    L = scenes.headlight(ci, M=1.0, specular=10.0)
    L.chaosColor.z, L.chaosColor.w = 1.0, 0.5
    render_cases.append(("inside48x32", 48, 32, c, p, "BCABA", R32.lights_recalculate([L])))
    # (d) looking away from the box: every ray misses
    q = scenes.uniform_quaternion(scenes.SplitMix64(5))
    co = scenes.orbit_camera(q, (2.0, 2.0, 2.0), -8.0)
    c = R32.cam_recalculate(co, 32, 32, 1)
    render_cases.append(("away32", 32, 32, c, scenes.make_params(10, 20), "AB", R32.lights_recalculate([scenes.headlight(co)])))
    meta["render_cases"] = []
    for name, W, H, c, p, s, ls in render_cases:
        seq = R32.seq_parse(s)
        rgba, pts = R32.render(W // 16, H // 16, c, p, seq, ls)
        colors = np.zeros((H, W, 4), dtype=np.float64)
        col = (ctypes.c_double * 4)()
        px = (ctypes.c_ubyte * 4)()
        arr = (LyapLight * len(ls))(*ls)
        for y in range(H):
            for x in range(W):
                R32.lib.ref_shade(ctypes.c_void_p(pts.ctypes.data + (x + y * W) * 36), ctypes.byref(c), arr,
                                  len(ls), col, px)
                colors[y, x] = col[:]
        rcs = np.zeros((H, W), dtype=np.int8)
        for y in range(H):
            for x in range(W):
                rcs[y, x] = R32.raymarch(x, y, c, p, seq)[0]
        out[f"render_{name}_cam"] = b(c)
        out[f"render_{name}_prm"] = b(p)
        out[f"render_{name}_lights"] = np.stack([b(l) for l in ls])
        out[f"render_{name}_rgba"] = rgba
        out[f"render_{name}_points"] = pts.view(np.uint8).reshape(H, W, 36)
        out[f"render_{name}_color"] = colors.astype(np.float32)
        out[f"render_{name}_rc"] = rcs
        meta["render_cases"].append({"name": name, "w": W, "h": H, "seq": s, "n_lights": len(ls)})

    # kernel_calc_volume (kernel.cu:518) at 32^3 over its fixed [0, 4)
    vp = scenes.make_params(20, 100)
    seq = R32.seq_parse("ABC")
    out["vol32_prm"] = b(vp)
    out["vol32_f32"] = R32.volume(32, vp, seq)
    out["vol32_f64"] = R64.volume(32, params_to_double(vp), seq)

    # the reference's kernel entry points as its own kernel.cu exports them
    # (nvcc on the reference source; only the symbol table is read)
    obj = os.path.join(ROOT, "oracle", "_ref", "kernel_ref.o")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-c", os.path.join(ref_dir, "kernel.cu"),
                    "-o", obj, f"-I{ref_dir}", "-w"], check=True, capture_output=True)
    nm = subprocess.run(["nm", obj], check=True, capture_output=True, text=True).stdout.split("\n")
    meta["ref_kernel_symbols"] = sorted(l.split()[-1] for l in nm if " T _Z18kernel_calc_" in l)

    np.savez_compressed(os.path.join(HERE, "golden_reference.npz"), **out)
    with open(os.path.join(HERE, "golden_reference.json"), "w") as f:
        json.dump(meta, f, indent=1)
    sz = os.path.getsize(os.path.join(HERE, "golden_reference.npz"))
    print(f"wrote golden_reference.npz ({sz / 1e6:.2f} MB) and golden_reference.json")


if __name__ == "__main__":
    main()
