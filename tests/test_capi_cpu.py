"""The C-ABI library without a GPU: it loads, exports every symbol the public
headers declare (and the reference's kernel entry points under the
reference's mangled names), its host scene helpers are bit-exact against the
reference's own host build, and argument errors come back as status codes."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

capi = pytest.importorskip("lyapunov3d_gb300.capi", reason="library not built")
from lyapunov3d_gb300.types import LyapCam, LyapLight, LyapParams, struct_from_bytes  # noqa: E402


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "lyap_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lyap_[a-z0-9_]+)\s*\(", src)))


def _exported():
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def test_every_declared_symbol_is_exported():
    decl = _declared_functions()
    assert decl, "no declarations parsed"
    exported = _exported()
    missing = [d for d in decl if d not in exported]
    assert not missing, missing
    assert sorted(decl) == sorted(capi.EXPORTED)


def test_reference_kernel_symbols_exported(golden):
    meta, _ = golden
    exported = _exported()
    for sym in meta["ref_kernel_symbols"]:
        assert sym in exported, sym


def test_version_and_status_strings():
    assert "sm_103a" in capi.version()
    assert capi.lib.lyap_abi_version() == 1
    assert capi.lib.lyap_status_string(capi.LYAP_ERR_SEQUENCE).decode() == "bad sequence"


def test_seq_parse_matches_reference(golden):
    meta, _ = golden
    for s, expect in meta["seq"].items():
        assert capi.seq_parse(s).tolist() == expect, s


@pytest.mark.parametrize("bad", ["", "0", "AX", "A0", " A", "E", "a-b"])
def test_seq_parse_rejects_what_the_reference_exits_on(bad):
    with pytest.raises(capi.LyapError) as e:
        capi.seq_parse(bad)
    assert e.value.code == capi.LYAP_ERR_SEQUENCE


def test_seq_parse_capacity():
    with pytest.raises(capi.LyapError) as e:
        capi.seq_parse("A9", cap=5)
    assert e.value.code == capi.LYAP_ERR_CAPACITY
    assert capi.seq_parse("A9", cap=11).tolist() == [0] * 10 + [-1]


def test_cam_lights_recalculate_bit_exact(golden):
    _, g = golden
    for i in range(g["cams_in"].shape[0]):
        cam = struct_from_bytes(LyapCam, g["cams_in"][i].tobytes())
        tw, th, td = (int(x) for x in g["cams_dims"][i])
        assert bytes(capi.cam_recalculate(cam, tw, th, td)) == g["cams_out"][i].tobytes(), i
    lights = [struct_from_bytes(LyapLight, r.tobytes()) for r in g["lights_in"]]
    assert [bytes(l) for l in capi.lights_recalculate(lights)] == [r.tobytes() for r in g["lights_out"]]


def test_cam_recalculate_rejects_zero_denominator():
    cam = LyapCam()
    cam.Q.w = 1.0
    with pytest.raises(capi.LyapError) as e:
        capi.cam_recalculate(cam, 64, 64, 0)
    assert e.value.code == capi.LYAP_ERR_INVALID_ARG


def _render_args(**over):
    cam, prm = LyapCam(), LyapParams()
    a = dict(cam=ctypes.byref(cam), prm=ctypes.byref(prm), seq=ctypes.c_void_p(0x1000), seq_len=3,
             lights=ctypes.c_void_p(0x2000), n_lights=1, rgba=ctypes.c_void_p(0x3000),
             points=ctypes.c_void_p(0x4000), w=8, h=8, ext=None, stream=None)
    a.update(over)
    return a, (cam, prm)


@pytest.mark.parametrize("over,code", [
    (dict(cam=None), capi.LYAP_ERR_INVALID_ARG),
    (dict(prm=None), capi.LYAP_ERR_INVALID_ARG),
    (dict(seq=None), capi.LYAP_ERR_INVALID_ARG),
    (dict(seq_len=1), capi.LYAP_ERR_SEQUENCE),
    (dict(seq_len=5000), capi.LYAP_ERR_SEQUENCE),
    (dict(lights=None), capi.LYAP_ERR_INVALID_ARG),
    (dict(n_lights=17), capi.LYAP_ERR_INVALID_ARG),
    (dict(rgba=None), capi.LYAP_ERR_INVALID_ARG),
    (dict(points=None), capi.LYAP_ERR_INVALID_ARG),
    (dict(w=0), capi.LYAP_ERR_INVALID_ARG),
    (dict(w=65536, h=65536), capi.LYAP_ERR_INVALID_ARG),
])
def test_render_argument_errors(over, code):
    a, keep = _render_args(**over)
    rc = capi.lib.lyap_render(a["cam"], a["prm"], a["seq"], a["seq_len"], a["lights"], a["n_lights"], a["rgba"],
                              a["points"], a["w"], a["h"], a["ext"], a["stream"])
    assert rc == code, capi.last_error()
    assert capi.last_error().startswith("lyap_render")


def test_render_ext_size_checked():
    ext = capi.LyapRenderExt()
    ext.size = 12
    a, keep = _render_args(ext=ctypes.byref(ext))
    rc = capi.lib.lyap_render(a["cam"], a["prm"], a["seq"], a["seq_len"], a["lights"], a["n_lights"], a["rgba"],
                              a["points"], a["w"], a["h"], a["ext"], a["stream"])
    assert rc == capi.LYAP_ERR_INVALID_ARG and "LyapRenderExt.size" in capi.last_error()
    ext = capi.LyapRenderExt(variant=7)
    a, keep = _render_args(ext=ctypes.byref(ext))
    assert capi.lib.lyap_render(a["cam"], a["prm"], a["seq"], a["seq_len"], a["lights"], a["n_lights"], a["rgba"],
                                a["points"], a["w"], a["h"], a["ext"], a["stream"]) == capi.LYAP_ERR_INVALID_ARG


@pytest.mark.parametrize("flags,ext_kw,msg", [
    (capi.FLAG_REQUIRE_JIT, {}, "precompiled"),
    (capi.FLAG_BISECT_F64, {}, "LYAP_FLAG_BISECT_F64"),
])
def test_render_noalloc_refuses_what_needs_allocation(flags, ext_kw, msg):
    """lyap_render_noalloc always runs the precompiled kernels and refuses the
    modes that need scratch memory, before touching any device."""
    ext = capi.LyapRenderExt(flags=flags, **ext_kw)
    a, keep = _render_args(ext=ctypes.byref(ext))
    rc = capi.lib.lyap_render_noalloc(a["cam"], a["prm"], a["seq"], a["seq_len"], a["lights"], a["n_lights"],
                                      a["rgba"], a["points"], a["w"], a["h"], a["ext"], a["stream"])
    assert rc == capi.LYAP_ERR_INVALID_ARG, capi.last_error()
    assert capi.last_error().startswith("lyap_render_noalloc") and msg in capi.last_error()


def test_volume_argument_errors():
    prm = LyapParams()
    L = capi.lib
    assert L.lyap_volume(None, 4, 4, 4, None, None, ctypes.byref(prm), ctypes.c_void_p(8), 3, None, None) == \
        capi.LYAP_ERR_INVALID_ARG
    assert L.lyap_volume(ctypes.c_void_p(8), 0, 4, 4, None, None, ctypes.byref(prm), ctypes.c_void_p(8), 3, None,
                         None) == capi.LYAP_ERR_INVALID_ARG
    assert L.lyap_volume(ctypes.c_void_p(8), 4, 4, 4, None, None, ctypes.byref(prm), ctypes.c_void_p(8), 1, None,
                         None) == capi.LYAP_ERR_SEQUENCE
    assert L.lyap_volume(ctypes.c_void_p(8), 1 << 20, 1 << 20, 1 << 20, None, None, ctypes.byref(prm),
                         ctypes.c_void_p(8), 3, None, None) == capi.LYAP_ERR_INVALID_ARG


def test_host_buffer_sequence_validated():
    """lyap_volume_host sees the sequence on the host and checks it before any device work."""
    prm = LyapParams()
    out = np.zeros(8, dtype=np.float32)
    for seq, code in [([0, 1, 5, -1], capi.LYAP_ERR_SEQUENCE), ([0, 1, 2], capi.LYAP_ERR_SEQUENCE),
                      ([-1], capi.LYAP_ERR_SEQUENCE)]:
        s = np.array(seq, dtype=np.int32)
        rc = capi.lib.lyap_volume_host(ctypes.c_void_p(out.ctypes.data), 2, 2, 2, None, None, ctypes.byref(prm),
                                       ctypes.c_void_p(s.ctypes.data), s.size, None, None)
        assert rc == code, capi.last_error()


def test_drop_in_launcher_argument_errors():
    cam, prm = LyapCam(), LyapParams()
    L = capi.lib
    assert L.lyap_kernel_calc_render(0, 1, 16, 16, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.byref(cam),
                                     ctypes.byref(prm), ctypes.c_void_p(8), ctypes.c_void_p(8), 1, None) == \
        capi.LYAP_ERR_INVALID_ARG
    assert L.lyap_kernel_calc_render(1, 1, 64, 64, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.byref(cam),
                                     ctypes.byref(prm), ctypes.c_void_p(8), ctypes.c_void_p(8), 1, None) == \
        capi.LYAP_ERR_INVALID_ARG
    # blocks of more than 256 threads (the kernel is compiled for two of 256 per SM)
    assert L.lyap_kernel_calc_render(1, 1, 32, 16, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.byref(cam),
                                     ctypes.byref(prm), ctypes.c_void_p(8), ctypes.c_void_p(8), 1, None) == \
        capi.LYAP_ERR_INVALID_ARG
    assert "at most 256" in capi.last_error()
    g = (ctypes.c_uint32 * 3)(1, 1, 0)
    b = (ctypes.c_uint32 * 3)(8, 8, 8)
    assert L.lyap_kernel_calc_volume(g, b, ctypes.c_void_p(8), ctypes.byref(prm), ctypes.c_void_p(8), None) == \
        capi.LYAP_ERR_INVALID_ARG


def test_abi_struct_sizes_match_c(tmp_path):
    """Every struct of include/lyap_gb300.h has the same size and field offsets
    in C (compiled here with gcc) as in the ctypes mirrors."""
    import shutil
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    checks = {
        "LyapRenderExt": (capi.LyapRenderExt, ["size", "flags", "d_counts", "d_stats", "h_seq", "bisect_halvings",
                                               "proposal", "proposal_margin", "proposal_dilate", "proposal_grid"]),
        "LyapNet": (capi.LyapNet, ["lo", "hi", "params", "train_mse", "val_mse", "seq_hash", "hash"]),
        "LyapNetTrainOptions": (capi.LyapNetTrainOptions, ["steps", "lr", "seed", "box_lo", "box_hi", "h_loss"]),
        "LyapVolumeExt": (capi.LyapVolumeExt, ["variant", "d_stats", "flags", "h_seq"]),
        "LyapRequest": (capi.LyapRequest, ["prm", "d_seq", "d_counts", "seq_len", "flags"]),
        "LyapBatchOptions": (capi.LyapBatchOptions, ["autotune", "flags", "d_stats", "jit_groups"]),
        "LyapBatchInfo": (capi.LyapBatchInfo, ["candidates", "specialised", "tuned_ms"]),
    }
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "lyap_gb300.h"', "int main(void) {"]
    for name, (_, fields) in checks.items():
        src.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        for f in fields:
            src.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    src.append("return 0; }")
    c = tmp_path / "sizes.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(c), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.splitlines())
    for name, (cls, fields) in checks.items():
        assert int(out[f"{name} size"]) == ctypes.sizeof(cls), name
        for f in fields:
            assert int(out[f"{name}.{f}"]) == getattr(cls, f).offset, (name, f)


def _net(seed=0):
    rng = np.random.default_rng(seed)
    return capi.net_from_params(rng.standard_normal(capi.NET_PARAMS) * 0.1, (2.0, 2.0, 2.0), (4.0, 4.0, 4.0))


def test_net_save_load_roundtrip(tmp_path):
    net = _net()
    path = str(tmp_path / "net.bin")
    capi.net_save(net, path)
    back = capi.net_load(path)
    assert bytes(back)[:-8] == bytes(net)[:-8]
    assert back.hash != 0
    # a flipped byte in the weights, a truncated file and a foreign file are refused
    raw = bytearray(open(path, "rb").read())
    raw[100] ^= 1
    open(path, "wb").write(bytes(raw))
    with pytest.raises(capi.LyapError, match="hash mismatch"):
        capi.net_load(path)
    open(path, "wb").write(bytes(raw[:-1]))
    with pytest.raises(capi.LyapError, match="not"):
        capi.net_load(path)
    open(path, "wb").write(b"\0" * ctypes.sizeof(capi.LyapNet))
    with pytest.raises(capi.LyapError, match="not a LyapNet"):
        capi.net_load(path)


@pytest.mark.parametrize("change,msg", [
    (dict(magic=0), "not a LyapNet"),
    (dict(segment=65), "proposal_segment"),
    (dict(dilate=2), "proposal_dilate"),
    (dict(margin=float("nan")), "proposal_margin"),
    (dict(jitter=0.5), "fixed step"),
    (dict(near_mul=2.0), "fixed step"),
])
def test_render_proposal_argument_errors(change, msg):
    net = _net()
    if "magic" in change:
        net.magic = change["magic"]
    ext = capi.LyapRenderExt(proposal=ctypes.pointer(net), proposal_margin=change.get("margin", 0.5),
                             proposal_segment=change.get("segment", 8), proposal_dilate=change.get("dilate", 0))
    a, (cam, prm) = _render_args(ext=ctypes.byref(ext))
    prm.jitter = change.get("jitter", 0.0)
    prm.nearMultiplier = change.get("near_mul", 1.0)
    rc = capi.lib.lyap_render(a["cam"], a["prm"], a["seq"], a["seq_len"], a["lights"], a["n_lights"], a["rgba"],
                              a["points"], a["w"], a["h"], a["ext"], a["stream"])
    assert rc == capi.LYAP_ERR_INVALID_ARG and msg in capi.last_error(), capi.last_error()


def test_render_ext_short_struct_accepted():
    """A caller built against the struct without the proposal fields passes
    its own (shorter) size; the size check accepts it (the call then fails
    later only for want of a device here)."""
    ext = capi.LyapRenderExt()
    ext.size = capi.LyapRenderExt.proposal.offset
    a, keep = _render_args(ext=ctypes.byref(ext))
    capi.lib.lyap_render(a["cam"], a["prm"], a["seq"], a["seq_len"], a["lights"], a["n_lights"], a["rgba"],
                         a["points"], a["w"], a["h"], a["ext"], a["stream"])
    assert "LyapRenderExt.size" not in capi.last_error()


def test_net_entry_argument_errors():
    net = _net()
    with pytest.raises(capi.LyapError, match="multiple of 128"):
        capi.net_grad(net, 8, 8, 100, 8)
    bad = _net()
    bad.hi[1] = bad.lo[1]
    with pytest.raises(capi.LyapError, match="empty input box"):
        capi.net_eval(bad, 8, 4, 8)
    prm = LyapParams()
    with pytest.raises(capi.LyapError) as e:
        capi.net_train(prm, np.array([0, 1, 7, -1], dtype=np.int32))
    assert e.value.code == capi.LYAP_ERR_SEQUENCE
    with pytest.raises(capi.LyapError, match="batch"):
        capi.net_train(prm, np.array([0, 1, -1], dtype=np.int32), batch=100)


def test_batch_options_checked():
    """LyapBatchOptions: jit_groups above LYAP_BATCH_JIT_GROUPS_MAX is refused
    before any device work; a caller built without jit_groups passes the
    shorter size, which the size check accepts (the call then fails on the
    request's null buffers instead)."""
    q = capi.LyapRequest()
    arr = (capi.LyapRequest * 1)(q)
    h = ctypes.c_void_p()
    opt = capi.LyapBatchOptions(jit_groups=capi.BATCH_JIT_GROUPS_MAX + 1)
    rc = capi.lib.lyap_batch_create(arr, 1, ctypes.byref(opt), ctypes.byref(h))
    assert rc == capi.LYAP_ERR_INVALID_ARG and "jit_groups" in capi.last_error(), capi.last_error()
    short = capi.LyapBatchOptions()
    short.size = capi.LyapBatchOptions.jit_groups.offset
    rc = capi.lib.lyap_batch_create(arr, 1, ctypes.byref(short), ctypes.byref(h))
    assert rc == capi.LYAP_ERR_INVALID_ARG and "request 0" in capi.last_error(), capi.last_error()
    bad = capi.LyapBatchOptions()
    bad.size = 12
    rc = capi.lib.lyap_batch_create(arr, 1, ctypes.byref(bad), ctypes.byref(h))
    assert rc == capi.LYAP_ERR_INVALID_ARG and "LyapBatchOptions.size" in capi.last_error()


def test_mirrored_constants_match_the_header():
    """Every numeric LYAP_* constant of include/lyap_gb300.h that the ctypes
    mirror defines (under its name without the prefix, or with it) has the
    header's value."""
    import re
    text = open(os.path.join(ROOT, "include", "lyap_gb300.h")).read()
    checked = 0
    for name, value in re.findall(r"^#define\s+LYAP_([A-Z0-9_]+)\s+\(?(-?\d+)u?\)?\s*(?:/\*.*)?$", text, re.M):
        for attr in (name, "LYAP_" + name):
            if hasattr(capi, attr) and isinstance(getattr(capi, attr), int):
                assert getattr(capi, attr) == int(value), (attr, getattr(capi, attr), value)
                checked += 1
                break
    assert checked >= 30
