"""ctypes binding of the C ABI (include/lyap_gb300.h).

Every call goes to the in-tree library lyapunov3d_gb300/_lib/liblyap_gb300.so;
if it is missing the import of this module fails loudly (there is no CPU
fallback).  A non-zero status from the library raises LyapError carrying the
library's own message.  Device pointers are plain integers (e.g. a torch
tensor's data_ptr()); streams are cudaStream_t handles as integers (0 = the
legacy default stream).
"""
import ctypes
import os
from ctypes import POINTER, c_char_p, c_float, c_int, c_int32, c_size_t, c_uint32, c_void_p

import numpy as np

from .types import LyapCam, LyapLight, LyapParams, POINT_DTYPE, RGBA_DTYPE

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "liblyap_gb300.so")

LYAP_OK = 0
LYAP_ERR_INVALID_ARG = -1
LYAP_ERR_SEQUENCE = -2
LYAP_ERR_CUDA = -3
LYAP_ERR_NO_DEVICE = -4
LYAP_ERR_OUT_OF_MEMORY = -5
LYAP_ERR_CAPACITY = -6
LYAP_ERR_JIT = -7
FLAG_NO_JIT = 1
FLAG_REQUIRE_JIT = 2
FLAG_NO_SPECULATION = 4
FLAG_NO_TAIL_BALANCE = 32
FLAG_BISECT_F64 = 8
FLAG_SPREAD_ORDER = 16
FORM_F64 = 2

VARIANT_PLAIN = 0
VARIANT_PRODUCT = 1
LIGHT_SPOT = 0
LIGHT_DIRECTIONAL = 1
MAX_SEQ_LEN = 4096
MAX_LIGHTS = 16

(STAT_SAMPLES, STAT_SKIPPED, STAT_MARCH, STAT_HONE, STAT_NORMAL, STAT_HITS, STAT_RAYS, STAT_FALLBACK, STAT_SPEC,
 STAT_SPEC_USED, STAT_ROUNDS, STAT_LANE_ROUNDS, STAT_MAX_ROUNDS, STAT_PROPOSAL_SKIPPED, STAT_PROPOSAL_POINTS,
 STAT_NET_TIMEOUTS, STAT_T_START, STAT_T_DRAIN, STAT_T_END, STAT_PROPOSAL_REWOUND, STAT_TAIL_HANDOVERS) = range(21)
STAT_COUNT = 21
PROPOSAL_GRID_DEFAULT = 64
BATCH_JIT_GROUPS_DEFAULT = 255
BATCH_JIT_GROUPS_MAX = 255
# the proposal margin the library's users are pointed to: the smallest of the
# measured margins at which the 1080p bench frame keeps >= 99.9 % of its
# surface pixels (bench.py --report proposal)
PROPOSAL_MARGIN_DEFAULT = 1.0

NET_MAGIC = 0x4E50594C
NET_VERSION = 1
NET_FEATURES = 48
NET_HIDDEN = 64
NET_PARAMS = 7361


class LyapError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[{code}] {message}")
        self.code = code
        self.message = message


class LyapNet(ctypes.Structure):
    """The learned proposal's network (include/lyap_gb300.h)."""
    _fields_ = [("magic", c_uint32), ("version", c_uint32), ("lo", c_float * 3), ("hi", c_float * 3),
                ("params", c_float * NET_PARAMS), ("train_mse", c_float), ("val_mse", c_float),
                ("steps", c_uint32), ("batch", c_uint32), ("n_samples", c_uint32), ("seq_hash", c_uint32),
                ("hash", ctypes.c_uint64)]

    def param_array(self):
        return np.ctypeslib.as_array(self.params).astype(np.float64)


class LyapNetTrainOptions(ctypes.Structure):
    _fields_ = [("size", c_uint32), ("n_samples", c_uint32), ("n_val", c_uint32), ("batch", c_uint32),
                ("steps", c_uint32), ("lr", c_float), ("target_lo", c_float), ("target_hi", c_float),
                ("seed", ctypes.c_uint64), ("box_lo", c_void_p), ("box_hi", c_void_p), ("h_loss", c_void_p)]

    def __init__(self, **kw):
        super().__init__()
        self.size = ctypes.sizeof(LyapNetTrainOptions)
        for k, v in kw.items():
            setattr(self, k, v)


class LyapRenderExt(ctypes.Structure):
    _fields_ = [("size", c_uint32), ("variant", c_uint32), ("light_model", c_uint32), ("flags", c_uint32),
                ("d_counts", c_void_p), ("d_stats", c_void_p), ("blocks_per_sm", c_uint32),
                ("threads_per_block", c_uint32), ("h_seq", c_void_p), ("bisect_halvings", c_uint32),
                ("pad_", c_uint32), ("proposal", POINTER(LyapNet)), ("proposal_margin", c_float),
                ("proposal_segment", c_uint32), ("proposal_dilate", c_uint32), ("proposal_grid", c_uint32)]

    def __init__(self, **kw):
        super().__init__()
        self.size = ctypes.sizeof(LyapRenderExt)
        for k, v in kw.items():
            setattr(self, k, v)


class LyapRequest(ctypes.Structure):
    """One request of a batch (include/lyap_gb300.h)."""
    _fields_ = [("cam", LyapCam), ("prm", LyapParams), ("d_seq", c_void_p), ("d_lights", c_void_p),
                ("d_rgba", c_void_p), ("d_points", c_void_p), ("d_counts", c_void_p), ("seq_len", c_uint32),
                ("n_lights", c_uint32), ("width", c_uint32), ("height", c_uint32), ("light_model", c_uint32),
                ("flags", c_uint32), ("_pad_tail", ctypes.c_uint8 * 8)]   # C pads to LyapCam's 16-byte alignment


assert ctypes.sizeof(LyapRequest) == 352


class LyapBatchOptions(ctypes.Structure):
    _fields_ = [("size", c_uint32), ("variant", c_uint32), ("autotune", c_uint32), ("tile_w", c_uint32),
                ("tile_h", c_uint32), ("tiles_per_chunk", c_uint32), ("blocks_per_sm", c_uint32),
                ("flags", c_uint32), ("d_stats", c_void_p), ("jit_groups", c_uint32)]

    def __init__(self, **kw):
        super().__init__()
        self.size = ctypes.sizeof(LyapBatchOptions)
        for k, v in kw.items():
            setattr(self, k, v)


class LyapBatchInfo(ctypes.Structure):
    _fields_ = [("size", c_uint32), ("requests", c_uint32), ("chunks", c_uint32), ("tile_w", c_uint32),
                ("tile_h", c_uint32), ("tiles_per_chunk", c_uint32), ("blocks_per_sm", c_uint32),
                ("threads_per_block", c_uint32), ("candidates", c_uint32), ("specialised", c_uint32),
                ("tuned_ms", ctypes.c_float * 16)]


class LyapVolumeExt(ctypes.Structure):
    _fields_ = [("size", c_uint32), ("variant", c_uint32), ("d_stats", c_void_p), ("blocks_per_sm", c_uint32),
                ("threads_per_block", c_uint32), ("flags", c_uint32), ("pad_", c_uint32), ("h_seq", c_void_p)]

    def __init__(self, **kw):
        super().__init__()
        self.size = ctypes.sizeof(LyapVolumeExt)
        for k, v in kw.items():
            setattr(self, k, v)


# every extern "C" symbol include/lyap_gb300.h declares (checked by tests)
EXPORTED = ["lyap_abi_version", "lyap_version", "lyap_last_error_string", "lyap_status_string",
            "lyap_seq_parse", "lyap_cam_recalculate", "lyap_lights_recalculate", "lyap_render",
            "lyap_volume", "lyap_render_host", "lyap_volume_host", "lyap_kernel_calc_render",
            "lyap_kernel_calc_volume", "lyap_pipe_probe", "lyap_render_noalloc", "lyap_jit_info",
            "lyap_lambda_points", "lyap_batch_create", "lyap_batch_run", "lyap_batch_info", "lyap_batch_destroy",
            "lyap_net_train", "lyap_net_eval", "lyap_net_grid", "lyap_net_grad", "lyap_net_save", "lyap_net_load",
            "lyap_params_init", "lyap_params_init_d", "lyap_ease_in_out_quart", "lyap_anim_camera",
            "lyap_anim_camera_d", "lyap_write_ppm", "lyap_write_points", "lyap_write_exps", "lyap_output_name",
            "lyap_cam_recalculate_d", "lyap_lights_recalculate_d", "lyap_render_d"]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m lyapunov3d_gb300.build` "
                          "(or __graft_entry__.build())")
    L = ctypes.CDLL(LIB_PATH)
    L.lyap_abi_version.restype = c_int
    L.lyap_version.restype = c_char_p
    L.lyap_last_error_string.restype = c_char_p
    L.lyap_status_string.restype = c_char_p
    L.lyap_status_string.argtypes = [c_int]
    L.lyap_seq_parse.argtypes = [c_char_p, POINTER(c_int32), c_size_t, POINTER(c_size_t)]
    L.lyap_cam_recalculate.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32]
    L.lyap_lights_recalculate.argtypes = [c_void_p, c_size_t]
    L.lyap_render.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_uint32, c_void_p, c_void_p,
                              c_uint32, c_uint32, c_void_p, c_void_p]
    L.lyap_volume.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_size_t, c_void_p, c_void_p]
    L.lyap_render_host.argtypes = L.lyap_render.argtypes
    L.lyap_render_noalloc.argtypes = L.lyap_render.argtypes
    L.lyap_volume_host.argtypes = L.lyap_volume.argtypes
    L.lyap_kernel_calc_render.argtypes = [c_uint32] * 4 + [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                           c_void_p, c_uint32, c_void_p]
    L.lyap_kernel_calc_volume.argtypes = [POINTER(c_uint32), POINTER(c_uint32), c_void_p, c_void_p, c_void_p,
                                          c_void_p]
    L.lyap_pipe_probe.argtypes = [c_uint32, c_uint32, c_void_p, POINTER(ctypes.c_double), c_void_p]
    L.lyap_jit_info.argtypes = [ctypes.c_char_p, c_size_t]
    L.lyap_lambda_points.argtypes = [c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_uint32, c_void_p, c_void_p]
    L.lyap_batch_create.argtypes = [c_void_p, c_uint32, c_void_p, POINTER(c_void_p)]
    L.lyap_batch_run.argtypes = [c_void_p, c_void_p]
    L.lyap_batch_info.argtypes = [c_void_p, c_void_p]
    L.lyap_batch_destroy.argtypes = [c_void_p]
    L.lyap_net_train.argtypes = [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p]
    L.lyap_net_eval.argtypes = [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p]
    L.lyap_net_grid.argtypes = [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p]
    L.lyap_net_grad.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p]
    L.lyap_net_save.argtypes = [c_void_p, c_char_p]
    L.lyap_net_load.argtypes = [c_void_p, c_char_p]
    L.lyap_params_init.argtypes = [c_void_p, c_void_p, c_void_p, c_uint32, POINTER(c_uint32), c_char_p, c_size_t,
                                   POINTER(c_uint32), POINTER(c_uint32)]
    L.lyap_params_init_d.argtypes = L.lyap_params_init.argtypes
    L.lyap_ease_in_out_quart.argtypes = [ctypes.c_double] * 4
    L.lyap_cam_recalculate_d.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32]
    L.lyap_lights_recalculate_d.argtypes = [c_void_p, c_size_t]
    L.lyap_render_d.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_uint32, c_void_p, c_void_p,
                                c_uint32, c_uint32, c_uint32, c_void_p, c_void_p]
    L.lyap_anim_camera.argtypes = [ctypes.c_double, c_void_p]
    L.lyap_anim_camera_d.argtypes = [ctypes.c_double, c_void_p]
    L.lyap_write_ppm.argtypes = [c_char_p, c_void_p, c_uint32, c_uint32, c_int]
    L.lyap_write_points.argtypes = [c_char_p, c_void_p, c_size_t]
    L.lyap_write_exps.argtypes = [c_char_p, c_void_p, c_size_t]
    L.lyap_output_name.argtypes = [c_char_p, c_size_t, c_char_p, ctypes.c_long, c_uint32, c_uint32, c_char_p,
                                   c_void_p, c_void_p, c_uint32, c_char_p]
    for name in EXPORTED:
        if name not in ("lyap_abi_version", "lyap_version", "lyap_last_error_string", "lyap_status_string"):
            getattr(L, name).restype = c_int
    L.lyap_ease_in_out_quart.restype = ctypes.c_double
    return L


lib = _load()


def _check(rc):
    if rc != LYAP_OK:
        raise LyapError(rc, lib.lyap_last_error_string().decode(errors="replace"))
    return rc


def jit_info():
    """(nvrtc_loaded, description) of the run-time specialisation."""
    buf = ctypes.create_string_buffer(4096)
    ok = lib.lyap_jit_info(buf, 4096)
    return bool(ok), buf.value.decode(errors="replace")


def version():
    return lib.lyap_version().decode()


def last_error():
    return lib.lyap_last_error_string().decode(errors="replace")


def _vp(p):
    if p is None:
        return None
    if hasattr(p, "data_ptr"):
        return c_void_p(p.data_ptr())
    if isinstance(p, np.ndarray):
        return c_void_p(p.ctypes.data)
    return c_void_p(int(p))


def _stream(s):
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return c_void_p(s.cuda_stream)
    return c_void_p(int(s))


# ---- host scene helpers (scene.hpp:11-15) -------------------------------
def seq_parse(s, cap=MAX_SEQ_LEN):
    """scene_convert_sequence: the -1 terminated symbol array (np.int32)."""
    out = (c_int32 * cap)()
    n = c_size_t(0)
    _check(lib.lyap_seq_parse(s.encode() if isinstance(s, str) else s, out, cap, ctypes.byref(n)))
    return np.array(out[:n.value], dtype=np.int32)


def cam_recalculate(cam, tw, th, td=1):
    """scene_cam_recalculate on a copy of cam; returns the copy."""
    c = LyapCam.from_buffer_copy(cam)
    _check(lib.lyap_cam_recalculate(ctypes.byref(c), tw, th, td))
    return c


def lights_recalculate(lights):
    arr = (LyapLight * max(1, len(lights)))(*[LyapLight.from_buffer_copy(l) for l in lights])
    _check(lib.lyap_lights_recalculate(arr, len(lights)))
    return list(arr)[:len(lights)]


def lights_array(lights):
    """LyapLight[] as a numpy byte array (for upload)."""
    arr = (LyapLight * max(1, len(lights)))(*[LyapLight.from_buffer_copy(l) for l in lights])
    return np.frombuffer(bytes(arr), dtype=np.uint8)[:ctypes.sizeof(LyapLight) * len(lights)].copy()


# ---- device entry points --------------------------------------------------
def render(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height, ext=None, stream=None):
    """lyap_render: asynchronous on `stream`; pointers are device addresses."""
    _check(lib.lyap_render(ctypes.byref(cam), ctypes.byref(prm), _vp(d_seq), seq_len, _vp(d_lights), n_lights,
                           _vp(d_rgba), _vp(d_points), width, height,
                           ctypes.byref(ext) if ext is not None else None, _stream(stream)))


def render_noalloc(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height, ext=None,
                   stream=None):
    """lyap_render_noalloc: lyap_render without any device allocation (shared static scratch)."""
    _check(lib.lyap_render_noalloc(ctypes.byref(cam), ctypes.byref(prm), _vp(d_seq), seq_len, _vp(d_lights),
                                   n_lights, _vp(d_rgba), _vp(d_points), width, height,
                                   ctypes.byref(ext) if ext is not None else None, _stream(stream)))


def volume(d_out, nx, ny, nz, lo, hi, prm, d_seq, seq_len, ext=None, stream=None):
    lo_a = (c_float * 3)(*lo) if lo is not None else None
    hi_a = (c_float * 3)(*hi) if hi is not None else None
    _check(lib.lyap_volume(_vp(d_out), nx, ny, nz, lo_a, hi_a, ctypes.byref(prm), _vp(d_seq), seq_len,
                           ctypes.byref(ext) if ext is not None else None, _stream(stream)))


def kernel_calc_render(grid, block, d_rgba, d_points, cam, prm, d_seq, d_lights, n_lights, stream=None):
    """kernel_calc_render<<<grid, block>>> (the reference's entry point and launch shape)."""
    _check(lib.lyap_kernel_calc_render(grid[0], grid[1], block[0], block[1], _vp(d_rgba), _vp(d_points),
                                       ctypes.byref(cam), ctypes.byref(prm), _vp(d_seq), _vp(d_lights), n_lights,
                                       _stream(stream)))


def kernel_calc_volume(grid, block, d_exps, prm, d_seq, stream=None):
    """kernel_calc_volume<<<grid, block>>> (the reference's entry point and launch shape)."""
    g = (c_uint32 * 3)(*grid)
    b = (c_uint32 * 3)(*block)
    _check(lib.lyap_kernel_calc_volume(g, b, _vp(d_exps), ctypes.byref(prm), _vp(d_seq), _stream(stream)))


def lambda_points(d_xyz, n, prm, d_seq, seq_len, form, d_out, stream=None):
    """lyap_lambda_points: lambda at n points (x, y, z per point) in the given form."""
    _check(lib.lyap_lambda_points(_vp(d_xyz), n, ctypes.byref(prm), _vp(d_seq), seq_len, form, _vp(d_out),
                                  _stream(stream)))


class Batch:
    """A batch of render requests captured in one CUDA graph (lyap_batch_*)."""

    def __init__(self, requests, variant=VARIANT_PLAIN, autotune=True, d_stats=None, **shape):
        arr = (LyapRequest * len(requests))(*requests)
        opt = LyapBatchOptions(variant=variant, autotune=1 if autotune else 0,
                               d_stats=d_stats.data_ptr() if hasattr(d_stats, "data_ptr") else d_stats, **shape)
        h = c_void_p()
        _check(lib.lyap_batch_create(arr, len(requests), ctypes.byref(opt), ctypes.byref(h)))
        self.handle = h
        self._keep = (arr, opt)

    def run(self, stream=None):
        _check(lib.lyap_batch_run(self.handle, _stream(stream)))

    def info(self):
        i = LyapBatchInfo()
        _check(lib.lyap_batch_info(self.handle, ctypes.byref(i)))
        return i

    def close(self):
        if self.handle:
            lib.lyap_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pipe_probe(kind, iters, d_sink, stream=None):
    """Launch the FFMA (kind 0) or lg2 (kind 1) rate probe; returns the op count."""
    ops = ctypes.c_double(0)
    _check(lib.lyap_pipe_probe(kind, iters, _vp(d_sink), ctypes.byref(ops), _stream(stream)))
    return ops.value


def render_host(cam, prm, seq, lights, width, height, ext=None, stream=None, rgba=None, points=None,
                want_points=True):
    """lyap_render_host with numpy buffers; returns (rgba[h, w, 4] u8, points[h, w] or None)."""
    seq = np.ascontiguousarray(seq, dtype=np.int32)
    la = lights_array(lights)
    if rgba is None:
        rgba = np.empty((height, width, 4), dtype=np.uint8)
    if want_points and points is None:
        points = np.empty((height, width), dtype=POINT_DTYPE)
    _check(lib.lyap_render_host(ctypes.byref(cam), ctypes.byref(prm), _vp(seq), seq.size, _vp(la), len(lights),
                                _vp(rgba), _vp(points) if want_points else None, width, height,
                                ctypes.byref(ext) if ext is not None else None, _stream(stream)))
    return rgba, points


def volume_host(nx, ny, nz, prm, seq, lo=None, hi=None, ext=None, stream=None, out=None):
    seq = np.ascontiguousarray(seq, dtype=np.int32)
    if out is None:
        out = np.empty((nz, ny, nx), dtype=np.float32)
    lo_a = (c_float * 3)(*lo) if lo is not None else None
    hi_a = (c_float * 3)(*hi) if hi is not None else None
    _check(lib.lyap_volume_host(_vp(out), nx, ny, nz, lo_a, hi_a, ctypes.byref(prm), _vp(seq), seq.size,
                                ctypes.byref(ext) if ext is not None else None, _stream(stream)))
    return out


# ---- learned proposal ------------------------------------------------------
def net_train(prm, seq, stream=None, box_lo=None, box_hi=None, with_loss=False, **opts):
    """lyap_net_train: a LyapNet trained on the GPU for this sequence and
    params (options as LyapNetTrainOptions fields); with_loss also returns
    each step's batch loss."""
    seq = np.ascontiguousarray(seq, dtype=np.int32)
    lo = (c_float * 3)(*box_lo) if box_lo is not None else None
    hi = (c_float * 3)(*box_hi) if box_hi is not None else None
    o = LyapNetTrainOptions(**opts)
    if lo is not None:
        o.box_lo = ctypes.cast(lo, c_void_p)
    if hi is not None:
        o.box_hi = ctypes.cast(hi, c_void_p)
    steps = o.steps or 8192
    loss = np.zeros(steps, dtype=np.float32) if with_loss else None
    if loss is not None:
        o.h_loss = loss.ctypes.data
    net = LyapNet()
    _check(lib.lyap_net_train(ctypes.byref(prm), _vp(seq), seq.size, ctypes.byref(o), ctypes.byref(net),
                              _stream(stream)))
    return (net, loss) if with_loss else net


def net_grid(net, n, dilate, d_out, stream=None):
    """lyap_net_grid: the proposal grid lyap_render reads (n^3 floats, x fastest) into d_out."""
    _check(lib.lyap_net_grid(ctypes.byref(net), n, dilate, _vp(d_out), _stream(stream)))


def net_eval(net, d_xyz, n, d_out, stream=None):
    """lyap_net_eval: the net at n device points (3 floats each) into d_out."""
    _check(lib.lyap_net_eval(ctypes.byref(net), _vp(d_xyz), n, _vp(d_out), _stream(stream)))


def net_grad(net, d_xyz, d_target, n, d_grad, d_loss=None, stream=None):
    """lyap_net_grad: d(mean squared error)/d(params) into d_grad (NET_PARAMS floats)."""
    _check(lib.lyap_net_grad(ctypes.byref(net), _vp(d_xyz), _vp(d_target), n, _vp(d_grad), _vp(d_loss),
                             _stream(stream)))


def net_save(net, path):
    _check(lib.lyap_net_save(ctypes.byref(net), os.fsencode(path)))


def net_load(path):
    net = LyapNet()
    _check(lib.lyap_net_load(ctypes.byref(net), os.fsencode(path)))
    return net


def net_from_params(params, lo, hi):
    """A LyapNet with the given FP32 parameters and input box (hash left to lyap_net_save)."""
    net = LyapNet()
    net.magic = NET_MAGIC
    net.version = NET_VERSION
    for k in range(3):
        net.lo[k] = lo[k]
        net.hi[k] = hi[k]
    p = np.asarray(params, dtype=np.float32)
    assert p.size == NET_PARAMS
    ctypes.memmove(net.params, p.ctypes.data, p.nbytes)
    return net


# ---- preset, animation path and output files --------------------------------
def params_init(double=False):
    """lyap_params_init(_d): (params, camera, lights, sequence string, (width, height))."""
    from .types import LyapCamD, LyapLightD, LyapParamsD
    prm, cam = (LyapParamsD(), LyapCamD()) if double else (LyapParams(), LyapCam())
    lights = ((LyapLightD if double else LyapLight) * 4)()
    n = c_uint32(0)
    seq = ctypes.create_string_buffer(64)
    w, h = c_uint32(0), c_uint32(0)
    fn = lib.lyap_params_init_d if double else lib.lyap_params_init
    _check(fn(ctypes.byref(prm), ctypes.byref(cam), lights, 4, ctypes.byref(n), seq, 64, ctypes.byref(w),
              ctypes.byref(h)))
    return prm, cam, list(lights)[:n.value], seq.value.decode(), (w.value, h.value)


def ease_in_out_quart(t, b=0.0, c=1.0, d=1.0):
    return lib.lyap_ease_in_out_quart(t, b, c, d)


def anim_camera(i, cam=None, double=False):
    """The camera of the animation path at eased value i (C and Q set on a copy of cam)."""
    from .types import LyapCamD
    if cam is None:
        cam = params_init(double)[1]
    c = (LyapCamD if double else LyapCam).from_buffer_copy(cam)
    _check((lib.lyap_anim_camera_d if double else lib.lyap_anim_camera)(i, ctypes.byref(c)))
    return c


def write_ppm(path, rgba, binary=False):
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = a.shape[:2]
    _check(lib.lyap_write_ppm(os.fsencode(path), _vp(a), w, h, 1 if binary else 0))


def write_points(path, points):
    a = np.ascontiguousarray(points)
    _check(lib.lyap_write_points(os.fsencode(path), _vp(a), a.size))


def write_exps(path, values):
    a = np.ascontiguousarray(values, dtype=np.float32)
    _check(lib.lyap_write_exps(os.fsencode(path), _vp(a), a.size))


def output_name(kind, stamp, width, height, seq, cam, prm, elapsed_s, ext):
    buf = ctypes.create_string_buffer(512)
    _check(lib.lyap_output_name(buf, 512, kind.encode(), stamp, width, height, seq.encode(), ctypes.byref(cam),
                                ctypes.byref(prm), elapsed_s, ext.encode()))
    return buf.value.decode()


# ---- DOUBLE_REALS render mode ---------------------------------------------
def cam_recalculate_d(cam, tw, th, td=1):
    from .types import LyapCamD
    c = LyapCamD.from_buffer_copy(cam)
    _check(lib.lyap_cam_recalculate_d(ctypes.byref(c), tw, th, td))
    return c


def lights_recalculate_d(lights):
    from .types import LyapLightD
    arr = (LyapLightD * max(1, len(lights)))(*[LyapLightD.from_buffer_copy(l) for l in lights])
    _check(lib.lyap_lights_recalculate_d(arr, len(lights)))
    return list(arr)[:len(lights)]


def render_d(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height,
             light_model=LIGHT_SPOT, d_counts=None, stream=None):
    """lyap_render_d: the DOUBLE_REALS render on device buffers (points: 72 bytes each)."""
    _check(lib.lyap_render_d(ctypes.byref(cam), ctypes.byref(prm), _vp(d_seq), seq_len, _vp(d_lights), n_lights,
                             _vp(d_rgba), _vp(d_points), width, height, light_model, _vp(d_counts),
                             _stream(stream)))
