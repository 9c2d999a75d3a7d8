"""Seeded synthetic scenes for the hot path's workloads.

The reference has no scene files: its one scene is hard-coded in
params_init (params.cu:21-114).  The workloads below are described by a
seed and a few sizes and rebuilt bit-identically anywhere:

* ``SplitMix64`` -- the project's PRNG (Steele, Lea & Flood's SplitMix64
  finaliser over a Weyl sequence), so a seed names the same scene on every
  machine independent of numpy's generators;
* ``uniform_quaternion`` -- a rotation uniform on S^3 (Shoemake's method);
* ``orbit_camera`` -- a camera ``dist`` from ``centre`` looking at it along
  Q*(0,0,1), the axis scene_cam_recalculate uses (scene.cu:51);
* ``volume_workload`` / ``render_workload`` -- the dense-volume and frame
  workloads: a 64^3 volume + 128^2 frame over [2.5, 4]^3 with sequence ABC
  and 20 + 100 iterations (the CPU-runnable case), and a 1920x1080 frame with
  512 steps per ray, a seeded 12-symbol sequence over {A, B, C}, 200 + 1000
  iterations over [2, 4]^3 plus a 512^3 volume (the full-size case).
"""
import math
from dataclasses import dataclass, field

import numpy as np

from .types import LyapCam, LyapLight, LyapParams

MASK64 = (1 << 64) - 1


class SplitMix64:
    """64-bit SplitMix generator; next_float() is uniform on [0, 1) with 53 bits."""

    def __init__(self, seed):
        self.state = int(seed) & MASK64

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def next_float(self):
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def uniform(self, lo, hi):
        return lo + (hi - lo) * self.next_float()

    def randint(self, n):
        return self.next_u64() % n

    def uniform_array(self, n, lo=0.0, hi=1.0):
        return np.array([self.uniform(lo, hi) for _ in range(n)], dtype=np.float64)


def uniform_quaternion(rng):
    """(x, y, z, w) uniform on S^3 from three uniforms (Shoemake 1992)."""
    u1, u2, u3 = rng.next_float(), rng.next_float(), rng.next_float()
    a, b = math.sqrt(1.0 - u1), math.sqrt(u1)
    return (a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2),
            b * math.sin(2 * math.pi * u3), b * math.cos(2 * math.pi * u3))


def quat_rotate(q, v):
    """Rotate v by unit quaternion q = (x, y, z, w) (double precision)."""
    x, y, z, w = q
    vx, vy, vz = v
    # t = 2 * cross(q.xyz, v); v' = v + w * t + cross(q.xyz, t)
    tx = 2 * (y * vz - z * vy)
    ty = 2 * (z * vx - x * vz)
    tz = 2 * (x * vy - y * vx)
    return (vx + w * tx + (y * tz - z * ty),
            vy + w * ty + (z * tx - x * tz),
            vz + w * tz + (x * ty - y * tx))


def orbit_camera(q, centre, dist, M=0.45):
    """A LyapCam at centre - dist * Q*(0,0,1), oriented by q (not yet recalculated)."""
    cam = LyapCam()
    f = quat_rotate(q, (0.0, 0.0, 1.0))
    cam.C.x, cam.C.y, cam.C.z = (centre[i] - dist * f[i] for i in range(3))
    cam.Q.x, cam.Q.y, cam.Q.z, cam.Q.w = q
    cam.M = M
    cam.renderDenominator = 1
    return cam


def headlight(cam, M=2.0, range_=None, colour=(1.0, 0.85, 0.7, 1.0), power=1.0,
              ambient=(0.05, 0.05, 0.05, 1.0), specular=0.0):
    """A wide spot light at the camera, pointing where it looks (Lambert-only
    when specular = 0).  Cones are filled in by lights_recalculate."""
    L = LyapLight()
    L.C = cam.C
    L.Q = cam.Q
    L.M = M
    d = math.sqrt(cam.C.x ** 2 + cam.C.y ** 2 + cam.C.z ** 2)
    L.lightRange = float(range_ if range_ is not None else max(1.0, d * d))
    L.ambient.x, L.ambient.y, L.ambient.z, L.ambient.w = ambient
    L.diffuseColor.x, L.diffuseColor.y, L.diffuseColor.z, L.diffuseColor.w = colour
    L.diffusePower = power
    L.specularColor.x = L.specularColor.y = L.specularColor.z = L.specularColor.w = 1.0
    L.specularPower = specular
    L.specularHardness = 10.0
    return L


def make_params(settle, accum, *, d=2.1, step_method=1, depth=256.0, opaque=0.0,
                near=None, near_mul=1.0, chaos=-0.5, jitter=0.0, refine=1.0,
                gradient=0.01, lmin=0.0, lmax=4.0):
    p = LyapParams()
    p.d = d
    p.settle = settle
    p.accum = accum
    p.stepMethod = step_method
    p.nearThreshold = opaque if near is None else near
    p.nearMultiplier = near_mul
    p.opaqueThreshold = opaque
    p.chaosThreshold = chaos
    p.depth = depth
    p.jitter = jitter
    p.refine = refine
    p.gradient = gradient
    p.lMin = lmin
    p.lMax = lmax
    return p


def random_sequence(rng, length, letters="ABC"):
    return "".join(letters[rng.randint(len(letters))] for _ in range(length))


@dataclass
class RenderWorkload:
    name: str
    width: int
    height: int
    seq: str
    params: LyapParams
    cam: LyapCam            # before cam_recalculate
    lights: list = field(default_factory=list)   # before lights_recalculate
    light_model: int = 0    # 0: the reference's spot model; 1: directional Lambert


@dataclass
class VolumeWorkload:
    name: str
    n: tuple
    lo: tuple
    hi: tuple
    seq: str
    params: LyapParams


def small_render(size=128):
    """128^2 frame of the [2.5, 4]^3 field of ABC, 20 + 100 iterations: camera
    6 from the cube centre, 256 uniform steps per ray (method 1), surface at
    the first sample with lambda <= 0, honing off (refine 1), no jitter, one
    Lambert headlight."""
    rng = SplitMix64(0x4C59415031)
    q = uniform_quaternion(rng)
    cam = orbit_camera(q, (3.25, 3.25, 3.25), 6.0)
    prm = make_params(20, 100, step_method=1, depth=256.0, opaque=0.0, near_mul=1.0,
                      jitter=0.0, refine=1.0, gradient=0.01, lmin=2.5, lmax=4.0)
    return RenderWorkload("frame128_abc_20+100", size, size, "ABC", prm, cam, [headlight(cam)])


def small_volume(n=64):
    prm = make_params(20, 100, lmin=2.5, lmax=4.0)
    return VolumeWorkload(f"volume{n}_abc_20+100", (n, n, n), (2.5, 2.5, 2.5), (4.0, 4.0, 4.0), "ABC", prm)


def full_render(seed=1, width=1920, height=1080, seq=None):
    """1920x1080, 512 uniform steps per ray (method 1, no jitter), seeded
    12-symbol sequence over {A, B, C}, 200 + 1000 iterations over [2, 4]^3,
    camera uniform on S^3 at distance 5-8 from the cube centre, one
    directional light.  Thresholds, honing and gradient are the reference's
    params_init defaults (opaque -0.75, chaos -0.5, near -1, refine 32,
    gradient 0.01; params.cu:23-36): with the surface at lambda <= -0.75 a
    ray crosses the weakly stable shell before it stops, ~140 samples per
    ray inside the box for seed 1."""
    rng = SplitMix64(0x4C594150_00000000 | seed)
    drawn = random_sequence(rng, 12)
    seq = drawn if seq is None else seq   # a given sequence replaces the drawn one; the camera stays
    q = uniform_quaternion(rng)
    dist = rng.uniform(5.0, 8.0)
    cam = orbit_camera(q, (3.0, 3.0, 3.0), dist)
    prm = make_params(200, 1000, step_method=1, depth=512.0, opaque=-0.75, near=-1.0, near_mul=1.0,
                      chaos=-0.5, jitter=0.0, refine=32.0, gradient=0.01, lmin=2.0, lmax=4.0)
    light = headlight(cam, ambient=(0.08, 0.08, 0.08, 1.0))
    lq = uniform_quaternion(rng)
    light.Q.x, light.Q.y, light.Q.z, light.Q.w = lq
    tag = "seq12" if seq == drawn else f"seq{seq}"
    return RenderWorkload(f"frame{height}_{tag}_200+1000_seed{seed}", width, height, seq, prm, cam,
                          [light], light_model=1)


def full_volume(n=512, seed=1):
    rng = SplitMix64(0x4C594150_00000000 | seed)
    seq = random_sequence(rng, 12)
    prm = make_params(200, 1000, lmin=2.0, lmax=4.0)
    return VolumeWorkload(f"volume{n}_seq12_200+1000_seed{seed}", (n, n, n), (2.0, 2.0, 2.0),
                          (4.0, 4.0, 4.0), seq, prm)


def batch_workloads(seed=4, scale=1, n_render=256, n_slices=32, one_seq=None):
    """The batched workload: n_render frames with resolution drawn from
    {256^2, 512^2, 1024^2, 1920x1080} (each side divided by `scale`), 128-1024
    steps per ray, 200 settle + 200-4000 accumulated iterations (log-uniform),
    sequences of length 2-16 over {A, B, C}; plus n_slices 4-D slices: the
    same kind of frame with sequences over {A, B, C, D} and D uniform in
    [2.5, 4].  Cameras orbit the [2, 4]^3 box at distance 5-8; thresholds are
    the reference's defaults.  one_seq: every request takes this sequence
    instead (the frames of one field; everything else is drawn as above)."""
    rng = SplitMix64(0x4C594150_BA7C0000 | seed)
    sizes = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]
    out = []
    for i in range(n_render + n_slices):
        w, h = sizes[rng.randint(4)]
        w, h = max(1, w // scale), max(1, h // scale)
        depth = float(128 + rng.randint(1024 - 128 + 1))
        accum = int(round(math.exp(rng.uniform(math.log(200.0), math.log(4000.0)))))
        L = 2 + rng.randint(15)
        slice4d = i >= n_render
        seq = random_sequence(rng, L, "ABCD" if slice4d else "ABC")
        if slice4d and "D" not in seq:
            seq = seq[:-1] + "D"
        if one_seq is not None:
            seq = one_seq
        d = rng.uniform(2.5, 4.0) if slice4d else 2.1
        q = uniform_quaternion(rng)
        dist = rng.uniform(5.0, 8.0)
        cam = orbit_camera(q, (3.0, 3.0, 3.0), dist)
        prm = make_params(200, accum, d=d, step_method=1, depth=depth, opaque=-0.75, near=-1.0, near_mul=1.0,
                          chaos=-0.5, jitter=0.0, refine=32.0, gradient=0.01, lmin=2.0, lmax=4.0)
        light = headlight(cam, ambient=(0.08, 0.08, 0.08, 1.0))
        kind = "slice" if slice4d else "frame"
        out.append(RenderWorkload(f"batch{seed}_{i}_{kind}_{w}x{h}_{seq}_{accum}", w, h, seq, prm, cam, [light],
                                  light_model=1))
    return out
