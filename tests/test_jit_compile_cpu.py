"""The run-time specialisation compiles, checked without a GPU.

Given the host copy of the sequence, the library compiles the render and
volume kernels for it with NVRTC (a host library) and then loads the cubin
into the device.  On a machine without a GPU the compile runs and only the
load fails, so a call that requires the specialisation reports which step
failed: "cudaLibraryLoadData" means the kernels compiled for that sequence,
"nvrtcCompileProgram" that the embedded kernel sources do not compile.  A
compile failure on a GPU host would otherwise only show as the slower
precompiled kernels taking over.

The calls pass placeholder device pointers, so this test must never run
where a GPU is visible (the call would launch): it skips there.
"""
import glob

import pytest

from lyapunov3d_gb300 import capi, scenes


def _gpu_visible():
    if glob.glob("/dev/nvidia[0-9]*"):
        return True
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.mark.skipif(_gpu_visible(), reason="placeholder device pointers: only without a GPU")
@pytest.mark.parametrize("seqstr,settle", [("A", 20), ("AACACBACCAAB", 200), ("ABCD" * 8, 7)])
def test_specialised_kernels_compile(seqstr, settle):
    prm = scenes.make_params(settle, 100, lmin=2.0, lmax=4.0)
    seq = capi.seq_parse(seqstr)
    ext = capi.LyapVolumeExt(variant=capi.VARIANT_PRODUCT, flags=capi.FLAG_REQUIRE_JIT, h_seq=seq.ctypes.data)
    with pytest.raises(capi.LyapError) as e:
        capi.volume(0x1000, 8, 8, 8, (2.0,) * 3, (4.0,) * 3, prm, 0x2000, seq.size, ext=ext)
    msg = e.value.message
    if "NVRTC unavailable" in msg:
        pytest.skip(msg)
    assert e.value.code == capi.LYAP_ERR_JIT
    assert "nvrtcCompileProgram" not in msg, msg
    assert "cudaLibraryLoadData" in msg, msg
