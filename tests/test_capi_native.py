"""A native C++ caller of the C ABI (tests/capi_clip.cpp): compiled and linked
against the library on any host; on a GPU it synthesises a clip, directly and
as two requests served at once, and every result must equal the Python
binding's and the oracle's bit for bit."""
import ctypes
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from _harness import assert_array_equal, assert_offsets_equal, config_params
from painttween_gb300 import _abi, synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def compile_consumer(out_dir):
    from painttween_gb300 import build as B
    lib = B.build()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = os.path.join(str(out_dir), "capi_clip")
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "capi_clip.cpp"), "-L", os.path.dirname(lib), "-lpainttween_gb300",
                           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe])
    return exe


def test_native_consumer_compiles_and_links(tmp_path):
    exe = compile_consumer(tmp_path)
    assert os.access(exe, os.X_OK)


def write_input(path, p, ex, clip):
    h, w = clip[0]["rgba"].shape[:2]
    eh, ew = ex["base"].shape[:2]
    with open(path, "wb") as f:
        f.write(struct.pack("<7i", 0x4C435450, w, h, ew, eh, len(clip), ctypes.sizeof(p)))
        f.write(bytes(p))
        for k in ("base", "output", "orient_tensor", "dist_trans", "object_ids"):
            f.write(np.ascontiguousarray(ex[k]).tobytes())
        for fr in clip:
            for k in ("rgba", "orient_tensor", "dist_trans", "object_ids", "vel_fwd", "vel_bwd", "scale"):
                f.write(np.ascontiguousarray(fr[k]).tobytes())


def read_output(path, frames, w, h, requests=2):
    """(per-frame results of the callback, pt_get_frame_result's last frame,
    per request the served clip's (rgba, offsets) stacks)."""
    raw = np.fromfile(path, np.uint8)
    n = w * h
    per = n * 16 + n * _abi.PATCH_DTYPE.itemsize
    assert raw.size == (frames + 1) * per + requests * frames * per
    out = []
    for f in range(frames + 1):
        chunk = raw[f * per:(f + 1) * per]
        rgba = chunk[:n * 16].view(np.float32).reshape(h, w, 4)
        offs = chunk[n * 16:].view(_abi.PATCH_DTYPE).reshape(h, w)
        out.append((rgba, offs))
    served, off = [], (frames + 1) * per
    for _ in range(requests):
        rgba = raw[off:off + frames * n * 16].view(np.float32).reshape(frames, h, w, 4)
        off += frames * n * 16
        offs = raw[off:off + frames * n * _abi.PATCH_DTYPE.itemsize].view(_abi.PATCH_DTYPE).reshape(frames, h, w)
        off += frames * n * _abi.PATCH_DTYPE.itemsize
        served.append((rgba, offs))
    return out[:frames], out[frames], served


@pytest.mark.gpu
def test_native_consumer_matches_python_binding_and_oracle(tmp_path):
    from oracle import oracle as O
    from painttween_gb300 import Synthesizer

    p = config_params(r=2, levels=3, iterations=2)
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(64, 64, seed=71)
    clip = synthetic.make_clip(72, 56, 3, 3, seed=72)
    exe = compile_consumer(tmp_path)
    inp, outp = os.path.join(str(tmp_path), "in.bin"), os.path.join(str(tmp_path), "out.bin")
    write_input(inp, p, ex, clip)
    run = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    native, last, served = read_output(outp, 3, 72, 56)

    s = Synthesizer(device=0)
    try:
        s.setup(p, 72, 56, 64, 64, 1)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        py = s.synthesize_animation(0, 2)
    finally:
        s.close()
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 2)
    for f in range(3):
        assert_offsets_equal(native[f][1], py[f][1], 1.0, "native vs Python binding, frame %d offsets" % f)
        assert_array_equal(native[f][0], py[f][0], "native vs Python binding, frame %d output" % f)
        assert_offsets_equal(native[f][1], ref[f][0], 1.0, "native vs oracle, frame %d offsets" % f)
        assert np.abs(native[f][0] - ref[f][2]).max() <= 1e-6
    assert_offsets_equal(last[1], native[2][1], 1.0, "pt_get_frame_result offsets")
    assert_array_equal(last[0], native[2][0], "pt_get_frame_result output")
    for r, (rgba, offs) in enumerate(served):
        for f in range(3):
            assert_offsets_equal(offs[f], native[f][1], 1.0, "served request %d, frame %d offsets" % (r, f))
            assert_array_equal(rgba[f], native[f][0], "served request %d, frame %d output" % (r, f))
