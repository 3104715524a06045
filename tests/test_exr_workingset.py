"""EXR files and working sets (host side, no GPU).

The EXR codec follows the published OpenEXR file layout; these tests check
it against hand-made byte streams and by round trips through every
supported compression.  The temporary-image helpers reproduce the files
WorkingBuffers::saveTempImages writes (src/PaintTweenCUDA/
workingBuffers.cpp:242-296), and the working-set loader the XML of
GUI/nlSynthesizer.cpp:99-160.
"""
import os
import struct

import numpy as np
import pytest

from painttween_gb300 import _abi, exr, workingset


@pytest.mark.parametrize("comp", [exr.NONE, exr.RLE, exr.ZIPS, exr.ZIP])
def test_round_trip_every_compression(tmp_path, comp):
    rng = np.random.default_rng(comp)
    h, w = 37, 19  # more lines than one ZIP chunk, odd sizes
    chans = {"R": rng.random((h, w)).astype(np.float16), "G": np.zeros((h, w), np.float16),
             "layer.x": rng.normal(size=(h, w)).astype(np.float32), "n": rng.integers(0, 2**32, (h, w), np.uint32)}
    chans["G"][:, 3:9] = 1.5  # runs for RLE
    p = str(tmp_path / "a.exr")
    exr.write(p, chans, comp)
    img = exr.read(p)
    assert (img["width"], img["height"], img["compression"]) == (w, h, comp)
    for k, v in chans.items():
        assert img["channels"][k].dtype == v.dtype
        assert img["channels"][k].tobytes() == v.tobytes(), k


def test_file_layout_bytes(tmp_path):
    p = str(tmp_path / "b.exr")
    exr.write(p, {"Y": np.ones((20, 3), np.float32)}, exr.ZIP)
    data = open(p, "rb").read()
    assert data[:4] == bytes([0x76, 0x2F, 0x31, 0x01]) and data[4:8] == bytes([2, 0, 0, 0])
    assert b"channels\0chlist\0" in data and b"compression\0compression\0\x01\0\0\0\x03" in data
    attrs, pos = exr._parse_header(data)
    offs = struct.unpack_from("<2Q", data, pos)  # ceil(20 / 16) chunks
    assert offs[0] == pos + 16 and struct.unpack_from("<i", data, offs[1])[0] == 16


def test_byte_transforms_and_rle_stream():
    rng = np.random.default_rng(3)
    for n in (0, 1, 2, 7, 64, 1001):
        raw = rng.integers(0, 256, n, np.uint8).tobytes()
        assert exr._unpredict_join(exr._split_predict(raw)) == raw
        enc = exr._rle_encode(raw)
        assert exr._rle_decode(enc, n) == raw
    # run of three 7s, then two literals
    assert exr._rle_decode(bytes([2, 7, 0xFE, 1, 2]), 5) == bytes([7, 7, 7, 1, 2])


def test_unsupported_compression_raises(tmp_path):
    p = str(tmp_path / "c.exr")
    exr.write(p, {"Y": np.zeros((4, 4), np.float32)}, exr.NONE)
    data = bytearray(open(p, "rb").read())
    i = data.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    data[i] = exr.PIZ
    open(p, "wb").write(bytes(data))
    with pytest.raises(exr.ExrError):
        exr.read(p)


def test_temporary_images_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    h, w = 12, 17
    offs = np.zeros((h, w), _abi.PATCH_DTYPE)
    for f in ("x", "y", "theta", "hysteresis", "lumShiftY", "lumShiftA", "scaleU", "scaleV"):
        offs[f] = rng.normal(size=(h, w))
    offs["layer"] = rng.integers(0, 3, (h, w))
    out = rng.random((h, w, 4)).astype(np.float32)
    res = (rng.random((h, w)) * 50).astype(np.float32)
    exr.save_temp_images(str(tmp_path), 2, 7, 1, offs, out, res)
    assert os.path.exists(os.path.join(str(tmp_path), "offsetsraw_2_1_0.0007.exr"))
    o2, out2, res2 = exr.load_temp_images(str(tmp_path), 2, 7, 1)
    assert o2.tobytes() == offs.tobytes()  # offsets round-trip exactly (FLOAT)
    assert np.array_equal(out2, out.astype(np.float16).astype(np.float32))
    assert np.array_equal(res2, res.astype(np.float16).astype(np.float32))  # loadResidual's half .b


def _write_set(root, keyed=False):
    rng = np.random.default_rng(9)
    os.makedirs(os.path.join(root, "shots"), exist_ok=True)
    h, w, sh, sw = 10, 14, 8, 8
    style = {"style_input": rng.random((sh, sw, 4)), "style_output": rng.random((sh, sw, 4))}
    for name, a in style.items():
        exr.write(os.path.join(root, name + ".exr"),
                  {"%s.%s" % (name, c): a[..., i].astype(np.float32) for i, c in enumerate(("red", "green", "blue", "alpha"))})
    ids = np.zeros((sh, sw, 3), np.float32)
    ids[..., 0], ids[..., 1] = 3 / 255.0, 1 / 255.0
    exr.write(os.path.join(root, "ids.exr"), {"id.%s" % c: ids[..., i] for i, c in enumerate(("red", "green", "blue"))})
    frames = {}
    for f in (1, 2):
        rgba = rng.random((h, w, 4)).astype(np.float16)
        exr.write(os.path.join(root, "shots", "sh1.rgba.%d.exr" % f), {c: rgba[..., i] for i, c in enumerate("RGBA")})
        vb = rng.normal(size=(h, w, 2)).astype(np.float32)
        exr.write(os.path.join(root, "shots", "sh1.velB.%d.exr" % f), {"vel_b_1.x": vb[..., 0], "vel_b_1.y": vb[..., 1]})
        frames[f] = (rgba, vb)
    xml = """<doc creator="t">
  <styles>
    <style%s><styleInput path="style_input.exr"/><styleOutput path="style_output.exr"/>
           <styleObjectIDs path="ids.exr"/></style>
  </styles>
  <params><levels value="3"/><maxLevel value="1"/><coherenceWeight value="0.5"/>
          <transparencyAllowed value="1"/><synthesisScheme value="0"/><firstFrame value="1"/>
          <lastFrame value="2"/><offsetsHistogramSlope value0="0.25"/><keyFrameInterpolation value="%d"/></params>
  <anim><unit name="u"/><shot name="sh1"/><shotDir path="shots"/><workingDir path="."/>
        <fileAccess checkFarm="0"/><elements inputElem=".rgba." velBElem="velB"/></anim>
</doc>""" % (' frame="1"' if keyed else "", 1 if keyed else 0)
    p = os.path.join(root, "set.xml")
    open(p, "w").write(xml)
    return p, style, frames


def test_working_set_loader(tmp_path):
    p, style, frames = _write_set(str(tmp_path))
    ws = workingset.load(p)
    q = ws.params
    assert (q.levels, q.finalLevel, q.scheme, q.transparencyOk, q.numStyles) == (3, 1, 0, 1, 1)
    assert q.coherenceWeight == 0.5 and abs(q.offsetsHistogramSlope[0] - 0.25) < 1e-7
    assert q.residualWindowSize == 4 and (ws.first_frame, ws.last_frame) == (1, 2)
    s = ws.styles[0]
    assert np.array_equal(s["base"], style["style_input"].astype(np.float32))
    assert (s["object_ids"] == 3 + 1 * 255).all()
    fr = ws.frame(2)
    assert np.array_equal(fr["rgba"], frames[2][0].astype(np.float32))
    assert np.array_equal(fr["vel_bwd"], frames[2][1])
    assert (fr["scale"] == 1).all() and (fr["vel_fwd"] == 0).all()  # absent elements


def test_keyed_working_set_feeds_keyframes(tmp_path):
    p, _, _ = _write_set(str(tmp_path), keyed=True)
    ws = workingset.load(p)
    assert ws.keyframes == [1] and ws.params.interpolateKeyFrame == 1

    class Recorder:
        def __init__(self):
            self.calls = []

        def __getattr__(self, name):
            return lambda *a, **k: self.calls.append((name,) + a[:1])

    r = Recorder()
    assert ws.setup(r) == (1, 2)
    names = [c[0] for c in r.calls]
    assert names[:3] == ["setup", "set_style", "set_keyframes"] and names.count("set_frame_dict") == 2


def test_ribbon_elements(tmp_path, monkeypatch):
    """Ribbon files per step (vel_b_01, vel_b_02 ...), relative to the
    working directory as in the reference; steps stop at the first missing."""
    p, _, _ = _write_set(str(tmp_path))
    xml = open(p).read().replace('velBElem="velB"', 'velBElem="velB" ribbonBElem="rb_[NN]" ribbonFElem="rf_[NN]"')
    open(p, "w").write(xml)
    monkeypatch.chdir(str(tmp_path))
    rng = np.random.default_rng(4)
    vals = {}
    for st in (1, 2, 4):
        for f in (1, 2):
            for key, elem, layer in (("vel_bwd", "rb", "vel_b"), ("vel_fwd", "rf", "vel_f")):
                if st == 4 and f == 2 and key == "vel_fwd":
                    continue  # step 4 incomplete
                v = rng.normal(size=(10, 14, 2)).astype(np.float32)
                vals[(key, st, f)] = v
                exr.write("%s_%02d.%d.exr" % (elem, st, f), {"%s_%d.x" % (layer, st): v[..., 0],
                                                            "%s_%d.y" % (layer, st): v[..., 1]})
    ws = workingset.load(p)
    assert ws.ribbon_steps(1, 2) == [1, 2]
    vf, vb = ws.ribbons(2, 2)
    assert np.array_equal(vf, vals[("vel_fwd", 2, 2)]) and np.array_equal(vb, vals[("vel_bwd", 2, 2)])
