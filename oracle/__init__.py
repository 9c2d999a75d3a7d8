"""Python binding of the ORACLE (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module, and only as the checker / the timed CPU restatement; the
product package (lyapunov3d_gb300) never imports it.

* ``Oracle``    -- ctypes view of oracle/_build/liblyap_oracle.so, the C
  restatement of the reference hot path (lyap_oracle.c);
* ``Reference`` -- ctypes view of oracle/_ref/libref_{f32,f64}.so, the
  reference's own kernel.cu / scene.cu / params.cu built as host C++ where
  the reference sources are present (``make -C oracle ref``).
"""
import ctypes
import os
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_size_t, c_uint32, c_void_p

import numpy as np

from lyapunov3d_gb300.types import (LyapCam, LyapCamD, LyapLight, LyapLightD, LyapParams,
                                    LyapParamsD, LyapPoint, LyapPointD, RGBA, POINT_DTYPE,
                                    RGBA_DTYPE)

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liblyap_oracle.so")
# the same restatement built -O3 -ffast-math: a second CPU-baseline build
# (timing only; fast-math reorders the arithmetic, so it is not the pin)
ORACLE_FASTMATH_SO = os.path.join(HERE, "_build", "liblyap_oracle_fastmath.so")
REF_DIR = os.path.join(HERE, "_ref")

ORC_REF, ORC_PLAIN, ORC_PRODUCT, ORC_F64 = 0, 1, 2, -1
ORC_HONE_CAP = 256


def build_oracle(force=False, fast_math=False):
    """Compile oracle/_build/liblyap_oracle.so (and its -O3 -ffast-math twin)
    with make (gcc); returns the path of the one asked for."""
    path = ORACLE_FASTMATH_SO if fast_math else ORACLE_SO
    if force or not os.path.exists(path):
        subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return path


def _ptr(a):
    return c_void_p(a.ctypes.data) if a is not None else None


def _seq_array(seq):
    a = np.ascontiguousarray(np.asarray(seq, dtype=np.int32))
    if a.ndim != 1 or a.size < 2 or a[-1] != -1:
        raise ValueError("sequence must be a -1 terminated int32 array")
    return a


class Oracle:
    """The C restatement.  All array results are numpy arrays."""

    def __init__(self, path=None, fast_math=False):
        path = path or build_oracle(fast_math=fast_math)
        L = ctypes.CDLL(path)
        self.lib = L
        L.orc_seq_parse.argtypes = [c_char_p, POINTER(c_int32), c_size_t, POINTER(c_size_t)]
        L.orc_lyap4d.argtypes = [c_int, c_float, c_float, c_float, c_float, c_uint32, c_uint32, c_void_p]
        L.orc_lyap4d.restype = c_float
        L.orc_lyap4d_d.argtypes = [c_double] * 4 + [c_uint32, c_uint32, c_void_p]
        L.orc_lyap4d_d.restype = c_double
        L.orc_lyap4d_batch.argtypes = [c_int, c_void_p, c_size_t, c_uint32, c_uint32, c_void_p, c_void_p]
        L.orc_volume.argtypes = [c_int, c_void_p, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
        L.orc_volume_d.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
        L.orc_raymarch.argtypes = [c_int, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
        L.orc_raymarch_d.argtypes = [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
        L.orc_shade.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p]
        L.orc_render_rows.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_uint32, c_uint32, c_uint32, c_uint32, c_void_p]
        L.orc_cam_recalculate.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32]
        L.orc_lights_recalculate.argtypes = [c_void_p, c_size_t]
        L.orc_cam_recalculate_d.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32]
        L.orc_lights_recalculate_d.argtypes = [c_void_p, c_size_t]
        L.orc_render_rows_prop.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                           c_uint32, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]
        L.orc_set_threads.argtypes = [c_int]
        L.orc_get_threads.restype = c_int

    # -- threads --
    def set_threads(self, n):
        self.lib.orc_set_threads(int(n))

    def threads(self):
        return self.lib.orc_get_threads()

    # -- scene --
    def seq_parse(self, s, cap=4096):
        out = (c_int32 * cap)()
        n = c_size_t(0)
        rc = self.lib.orc_seq_parse(s.encode() if isinstance(s, str) else s, out, cap, ctypes.byref(n))
        if rc != 0:
            return rc, None
        return 0, np.array(out[:n.value], dtype=np.int32)

    def cam_recalculate(self, cam, tw, th, td):
        c = LyapCam.from_buffer_copy(cam)
        self.lib.orc_cam_recalculate(ctypes.byref(c), tw, th, td)
        return c

    def lights_recalculate(self, lights):
        arr = (LyapLight * len(lights))(*[LyapLight.from_buffer_copy(l) for l in lights])
        self.lib.orc_lights_recalculate(arr, len(lights))
        return list(arr)

    def cam_recalculate_d(self, cam, tw, th, td):
        c = LyapCamD.from_buffer_copy(cam)
        self.lib.orc_cam_recalculate_d(ctypes.byref(c), tw, th, td)
        return c

    def lights_recalculate_d(self, lights):
        arr = (LyapLightD * len(lights))(*[LyapLightD.from_buffer_copy(l) for l in lights])
        self.lib.orc_lights_recalculate_d(arr, len(lights))
        return list(arr)

    # -- lambda --
    def lyap4d(self, mode, pts, settle, accum, seq):
        """lambda at points pts[:, 0:4] = (x, y, z, d); mode ORC_F64 = double."""
        p = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).reshape(-1, 4))
        s = _seq_array(seq)
        out = np.empty(p.shape[0], dtype=np.float64)
        self.lib.orc_lyap4d_batch(mode, _ptr(p), p.shape[0], settle, accum, _ptr(s), _ptr(out))
        return out

    def volume(self, mode, nx, ny, nz, prm, seq, lo=None, hi=None):
        s = _seq_array(seq)
        lo_a = np.asarray(lo, dtype=np.float32) if lo is not None else None
        hi_a = np.asarray(hi, dtype=np.float32) if hi is not None else None
        if mode == ORC_F64:
            out = np.empty(nx * ny * nz, dtype=np.float64)
            pd = params_to_double(prm) if isinstance(prm, LyapParams) else prm
            self.lib.orc_volume_d(_ptr(out), nx, ny, nz, _ptr(lo_a), _ptr(hi_a), ctypes.byref(pd), _ptr(s))
        else:
            out = np.empty(nx * ny * nz, dtype=np.float32)
            self.lib.orc_volume(mode, _ptr(out), nx, ny, nz, _ptr(lo_a), _ptr(hi_a), ctypes.byref(prm), _ptr(s))
        return out.reshape(nz, ny, nx)

    def raymarch(self, mode, sx, sy, cam, prm, seq):
        s = _seq_array(seq)
        pt = LyapPoint()
        ctypes.memset(ctypes.byref(pt), 0xFF, ctypes.sizeof(pt))
        cnt = (c_uint32 * 3)()
        rc = self.lib.orc_raymarch(mode, ctypes.byref(pt), sx, sy, ctypes.byref(cam), ctypes.byref(prm), _ptr(s), cnt)
        return rc, pt, tuple(cnt)

    def raymarch_d(self, sx, sy, cam, prm, seq):
        """orc_raymarch_d: the DOUBLE_REALS raymarch of one pixel."""
        s = _seq_array(seq)
        pt = LyapPointD()
        ctypes.memset(ctypes.byref(pt), 0xFF, ctypes.sizeof(pt))
        cnt = (c_uint32 * 3)()
        rc = self.lib.orc_raymarch_d(ctypes.byref(pt), sx, sy, ctypes.byref(cam), ctypes.byref(prm), _ptr(s), cnt)
        return rc, pt, tuple(cnt)

    def shade(self, pt, cam, lights):
        arr = (LyapLight * max(1, len(lights)))(*[LyapLight.from_buffer_copy(l) for l in lights])
        col = (c_float * 4)()
        px = RGBA()
        self.lib.orc_shade(ctypes.byref(pt), ctypes.byref(cam), arr, len(lights), col, ctypes.byref(px))
        return tuple(col), (px.r, px.g, px.b, px.a)

    def render_prop(self, mode, w, h, cam, prm, seq, lights, prop, y0=0, y1=None):
        """render() with the product's proposal march (prop: from proposal());
        also returns pcounts[h', w, 2] (skipped positions, rewound runs)."""
        y1 = h if y1 is None else y1
        s = _seq_array(seq)
        rgba = np.zeros((y1 - y0) * w, dtype=RGBA_DTYPE)
        pts = np.zeros((y1 - y0) * w, dtype=POINT_DTYPE)
        cnt = np.zeros((y1 - y0) * w * 3, dtype=np.uint32)
        pcnt = np.zeros((y1 - y0) * w * 2, dtype=np.uint32)
        arr = (LyapLight * max(1, len(lights)))(*[LyapLight.from_buffer_copy(l) for l in lights])
        off = y0 * w
        self.lib.orc_render_rows_prop(mode, c_void_p(rgba.ctypes.data - off * 4), c_void_p(pts.ctypes.data - off * 36),
                                      ctypes.byref(cam), ctypes.byref(prm), _ptr(s), arr, len(lights), w, y0, y1,
                                      ctypes.byref(prop[0]), c_void_p(cnt.ctypes.data - off * 12),
                                      c_void_p(pcnt.ctypes.data - off * 8))
        return (rgba.view(np.uint8).reshape(y1 - y0, w, 4), pts.reshape(y1 - y0, w), cnt.reshape(y1 - y0, w, 3),
                pcnt.reshape(y1 - y0, w, 2))

    def render(self, mode, w, h, cam, prm, seq, lights, y0=0, y1=None):
        """Rows [y0, y1) of a w-wide image: (rgba[h', w, 4] u8, points[h', w], counts[h', w, 3])."""
        y1 = h if y1 is None else y1
        s = _seq_array(seq)
        n = w * (y1 - y0)
        rgba = np.zeros((y1 - y0) * w, dtype=RGBA_DTYPE)
        pts = np.zeros((y1 - y0) * w, dtype=POINT_DTYPE)
        cnt = np.zeros((y1 - y0) * w * 3, dtype=np.uint32)
        arr = (LyapLight * max(1, len(lights)))(*[LyapLight.from_buffer_copy(l) for l in lights])
        # orc_render_rows indexes x + y * w from row 0: offset the buffers so row y0 lands at 0
        off = y0 * w
        base_rgba = rgba.ctypes.data - off * 4
        base_pts = pts.ctypes.data - off * 36
        base_cnt = cnt.ctypes.data - off * 12
        self.lib.orc_render_rows(mode, c_void_p(base_rgba), c_void_p(base_pts), ctypes.byref(cam),
                                 ctypes.byref(prm), _ptr(s), arr, len(lights), w, y0, y1,
                                 c_void_p(base_cnt))
        return (rgba.view(np.uint8).reshape(y1 - y0, w, 4), pts.reshape(y1 - y0, w),
                cnt.reshape(y1 - y0, w, 3))


class OrcProposal(ctypes.Structure):
    """lyap_oracle.h OrcProposal: the product's proposal grid as its march reads it."""
    _fields_ = [("grid", c_void_p), ("n", c_uint32), ("run", c_uint32), ("lo", c_float * 3), ("scale", c_float * 3),
                ("tau", c_float)]


def proposal(grid, n, run, lo, hi, tau):
    """An OrcProposal over the box [lo, hi] (the net's) for a grid of n^3
    float32 cells (kept alive by the returned tuple's second item)."""
    g = np.ascontiguousarray(np.asarray(grid, dtype=np.float32).reshape(-1))
    assert g.size == n ** 3
    p = OrcProposal()
    p.grid = g.ctypes.data
    p.n, p.run, p.tau = n, run, tau
    for k in range(3):
        p.lo[k] = lo[k]
        p.scale[k] = np.float32(n) / (np.float32(hi[k]) - np.float32(lo[k]))
    return p, g


def params_to_double(p):
    d = LyapParamsD()
    for name, _ in LyapParams._fields_:
        setattr(d, name, getattr(p, name))
    return d


class Reference:
    """The reference's own code built as host C++ (one Real width per library)."""

    def __init__(self, real="f32", path=None):
        path = path or os.path.join(REF_DIR, f"libref_{real}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        self.lib = L
        self.real = real
        self.Cam = LyapCam if real == "f32" else LyapCamD
        self.Params = LyapParams if real == "f32" else LyapParamsD
        self.Point = LyapPoint if real == "f32" else LyapPointD
        L.ref_layout.argtypes = [POINTER(ctypes.c_longlong), c_int]
        L.ref_seq_parse.argtypes = [c_char_p, POINTER(c_int), c_size_t]
        L.ref_seq_parse.restype = c_size_t
        L.ref_params_init.argtypes = [c_void_p] * 3 + [POINTER(c_uint32), c_char_p, c_size_t,
                                                       POINTER(c_uint32), POINTER(c_uint32)]
        L.ref_cam_recalculate.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32]
        L.ref_lights_recalculate.argtypes = [c_void_p, c_size_t]
        L.ref_lyap4d.argtypes = [c_void_p, c_size_t, c_uint32, c_uint32, c_void_p, c_void_p]
        L.ref_raymarch.argtypes = [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]
        L.ref_shade.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p]
        L.ref_render.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_uint32, c_uint32, c_uint32, c_uint32, c_uint32]
        L.ref_volume.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32, c_uint32]

    def layout(self):
        a = (ctypes.c_longlong * 64)()
        n = self.lib.ref_layout(a, 64)
        return list(a[:n])

    def seq_parse(self, s):
        out = (c_int * 4096)()
        n = self.lib.ref_seq_parse(s.encode() if isinstance(s, str) else s, out, 4096)
        return np.array(out[:n], dtype=np.int32)

    def params_init(self):
        prm = self.Params()
        cam = self.Cam()
        lights = (self.Cam * 16)()
        nl = c_uint32(0)
        seq = ctypes.create_string_buffer(256)
        w, h = c_uint32(0), c_uint32(0)
        self.lib.ref_params_init(ctypes.byref(prm), ctypes.byref(cam), lights, ctypes.byref(nl), seq, 256,
                                 ctypes.byref(w), ctypes.byref(h))
        return prm, cam, list(lights)[:nl.value], seq.value.decode(), (w.value, h.value)

    def cam_recalculate(self, cam, tw, th, td):
        c = self.Cam.from_buffer_copy(cam)
        self.lib.ref_cam_recalculate(ctypes.byref(c), tw, th, td)
        return c

    def lights_recalculate(self, lights):
        arr = (self.Cam * len(lights))(*[self.Cam.from_buffer_copy(l) for l in lights])
        self.lib.ref_lights_recalculate(arr, len(lights))
        return list(arr)

    def lyap4d(self, pts, settle, accum, seq):
        p = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).reshape(-1, 4))
        s = _seq_array(seq)
        out = np.empty(p.shape[0], dtype=np.float64)
        self.lib.ref_lyap4d(_ptr(p), p.shape[0], settle, accum, _ptr(s), _ptr(out))
        return out

    def raymarch(self, sx, sy, cam, prm, seq):
        s = _seq_array(seq)
        pt = self.Point()
        ctypes.memset(ctypes.byref(pt), 0xFF, ctypes.sizeof(pt))
        rc = self.lib.ref_raymarch(ctypes.byref(pt), sx, sy, ctypes.byref(cam), ctypes.byref(prm), _ptr(s))
        return rc, pt

    def render(self, gw, gh, cam, prm, seq, lights, bw=16, bh=16):
        """kernel_calc_render on a (gw, gh) grid of (bw, bh) blocks; points pre-filled with 0xFF."""
        assert self.real == "f32"
        s = _seq_array(seq)
        W, H = gw * bw, gh * bh
        rgba = np.zeros(W * H * 4, dtype=np.uint8)
        pts = np.full(W * H * 36, 0xFF, dtype=np.uint8)
        arr = (LyapLight * max(1, len(lights)))(*[LyapLight.from_buffer_copy(l) for l in lights])
        self.lib.ref_render(_ptr(rgba), _ptr(pts), ctypes.byref(cam), ctypes.byref(prm), _ptr(s), arr,
                            len(lights), gw, gh, bw, bh)
        return rgba.reshape(H, W, 4), pts.view(POINT_DTYPE).reshape(H, W)

    def volume(self, n, prm, seq, bs=8):
        s = _seq_array(seq)
        out = np.empty(n * n * n, dtype=np.float32)
        self.lib.ref_volume(_ptr(out), ctypes.byref(prm), _ptr(s), n, bs)
        return out.reshape(n, n, n)
