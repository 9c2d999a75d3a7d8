"""Device-resident frames and volumes for the workloads of scenes.py.

The buffers are torch CUDA tensors (torch is used for device memory and
streams only); every computation goes through the C ABI (capi.py).
"""
import numpy as np

from . import capi
from .types import POINT_DTYPE


def _torch():
    import torch
    return torch


class DeviceFrame:
    """One RenderWorkload on the GPU: prepared camera/lights, device inputs and outputs."""

    def __init__(self, wl, device="cuda", counts=False, stats=True):
        torch = _torch()
        self.wl = wl
        self.width, self.height = wl.width, wl.height
        self.cam = capi.cam_recalculate(wl.cam, wl.width, wl.height, 1)
        self.lights = capi.lights_recalculate(wl.lights)
        self.seq = capi.seq_parse(wl.seq)
        self.prm = wl.params
        self.light_model = wl.light_model
        n = self.width * self.height
        self.d_seq = torch.from_numpy(self.seq).to(device)
        self.d_lights = torch.from_numpy(capi.lights_array(self.lights)).to(device)
        self.d_rgba = torch.empty(n * 4, dtype=torch.uint8, device=device)
        self.d_points = torch.empty(n * 9, dtype=torch.float32, device=device)
        self.d_counts = torch.zeros(n * 3, dtype=torch.int32, device=device) if counts else None
        self.d_stats = torch.zeros(capi.STAT_COUNT, dtype=torch.int64, device=device) if stats else None

    def ext(self, variant=capi.VARIANT_PLAIN, jit=False, **kw):
        """jit: hand the host copy of the sequence over so the library uses the
        kernels compiled for it at run time (identical results, faster; the
        first call per sequence pays a few seconds of compilation); False
        forces the precompiled kernels."""
        if jit:
            kw.setdefault("h_seq", self.seq.ctypes.data)
        else:
            kw["flags"] = kw.get("flags", 0) | capi.FLAG_NO_JIT
        return capi.LyapRenderExt(variant=variant, light_model=self.light_model,
                                  d_counts=self.d_counts.data_ptr() if self.d_counts is not None else None,
                                  d_stats=self.d_stats.data_ptr() if self.d_stats is not None else None, **kw)

    def run(self, variant=capi.VARIANT_PLAIN, stream=None, jit=False, **kw):
        capi.render(self.cam, self.prm, self.d_seq, self.seq.size, self.d_lights, len(self.lights), self.d_rgba,
                    self.d_points, self.width, self.height, ext=self.ext(variant, jit, **kw), stream=stream)

    def reset_stats(self):
        if self.d_stats is not None:
            self.d_stats.zero_()

    def stats(self):
        return self.d_stats.cpu().numpy().astype(np.int64) if self.d_stats is not None else None

    def iterations(self, stats=None):
        """Logistic-map iterations the plain method performs for the recorded samples."""
        s = self.stats() if stats is None else stats
        return int(s[capi.STAT_SAMPLES]) * (self.prm.settle + self.prm.accum) - int(s[capi.STAT_SKIPPED]) * self.prm.accum

    def rgba(self):
        return self.d_rgba.cpu().numpy().reshape(self.height, self.width, 4)

    def points(self):
        return self.d_points.cpu().numpy().view(POINT_DTYPE).reshape(self.height, self.width)

    def counts(self):
        return self.d_counts.cpu().numpy().reshape(self.height, self.width, 3).astype(np.uint32)


class DeviceVolume:
    """One VolumeWorkload on the GPU."""

    def __init__(self, wl, device="cuda", stats=True):
        torch = _torch()
        self.wl = wl
        self.nx, self.ny, self.nz = wl.n
        self.seq = capi.seq_parse(wl.seq)
        self.prm = wl.params
        self.d_seq = torch.from_numpy(self.seq).to(device)
        self.d_out = torch.empty(self.nx * self.ny * self.nz, dtype=torch.float32, device=device)
        self.d_stats = torch.zeros(capi.STAT_COUNT, dtype=torch.int64, device=device) if stats else None

    def ext(self, variant=capi.VARIANT_PLAIN, jit=False, **kw):
        if jit:
            kw.setdefault("h_seq", self.seq.ctypes.data)
        else:
            kw["flags"] = kw.get("flags", 0) | capi.FLAG_NO_JIT
        return capi.LyapVolumeExt(variant=variant,
                                  d_stats=self.d_stats.data_ptr() if self.d_stats is not None else None, **kw)

    def run(self, variant=capi.VARIANT_PLAIN, stream=None, jit=False, **kw):
        capi.volume(self.d_out, self.nx, self.ny, self.nz, self.wl.lo, self.wl.hi, self.prm, self.d_seq,
                    self.seq.size, ext=self.ext(variant, jit, **kw), stream=stream)

    def reset_stats(self):
        if self.d_stats is not None:
            self.d_stats.zero_()

    def stats(self):
        return self.d_stats.cpu().numpy().astype(np.int64) if self.d_stats is not None else None

    def iterations(self, stats=None):
        s = self.stats() if stats is None else stats
        return int(s[capi.STAT_SAMPLES]) * (self.prm.settle + self.prm.accum) - int(s[capi.STAT_SKIPPED]) * self.prm.accum

    def values(self):
        return self.d_out.cpu().numpy().reshape(self.nz, self.ny, self.nx)


class DeviceBatch:
    """A list of RenderWorkloads on the GPU as one lyap_batch (one graph launch)."""

    def __init__(self, workloads, device="cuda", variant=capi.VARIANT_PLAIN, autotune=True, counts=False,
                 **shape):
        torch = _torch()
        self.frames = [DeviceFrame(wl, device=device, counts=counts, stats=False) for wl in workloads]
        self.d_stats = torch.zeros(capi.STAT_COUNT, dtype=torch.int64, device=device)
        reqs = []
        for f in self.frames:
            q = capi.LyapRequest()
            q.cam = f.cam
            q.prm = f.prm
            q.d_seq = f.d_seq.data_ptr()
            q.d_lights = f.d_lights.data_ptr()
            q.d_rgba = f.d_rgba.data_ptr()
            q.d_points = f.d_points.data_ptr()
            q.d_counts = f.d_counts.data_ptr() if f.d_counts is not None else None
            q.seq_len = f.seq.size
            q.n_lights = len(f.lights)
            q.width, q.height = f.width, f.height
            q.light_model = f.light_model
            reqs.append(q)
        self.batch = capi.Batch(reqs, variant=variant, autotune=autotune, d_stats=self.d_stats, **shape)

    def run(self, stream=None):
        self.batch.run(stream)

    def stats(self):
        return self.d_stats.cpu().numpy().astype(np.int64)

    def iterations(self):
        """Plain-method logistic iterations of one run, from the per-pixel sample
        counts (requests differ in settle + accum; needs counts=True)."""
        total = 0
        for f in self.frames:
            samples = int(f.d_counts.view(-1, 3).sum(dim=1, dtype=_torch().int64).sum().item())
            total += samples * (f.prm.settle + f.prm.accum)
        return total
