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


@pytest.mark.parametrize("comp", [exr.NONE, exr.RLE, exr.ZIPS, exr.ZIP, exr.PIZ])
def test_round_trip_every_compression(tmp_path, comp):
    rng = np.random.default_rng(comp)
    h, w = 37, 19  # more lines than one ZIP / PIZ chunk, odd sizes
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
    data[i] = 5  # PXR24
    open(p, "wb").write(bytes(data))
    with pytest.raises(exr.ExrError):
        exr.read(p)


# --- PIZ, against chunks assembled by hand from the format's layout ---------

def _bits(*fields):
    """Bytes of (value, bit count) fields, most significant bit first, the
    last byte padded with zeros."""
    s = "".join(format(v, "0%db" % n) for v, n in fields)
    s += "0" * (-len(s) % 8)
    return bytes(int(s[i:i + 8], 2) for i in range(0, len(s), 8))


def _huf(im, iM, table, nbits, data):
    return struct.pack("<5I", im, iM, len(table), nbits, 0) + table + data


def _piz(lo, hi, bitmap, huf):
    return struct.pack("<HH", lo, hi) + bytes(bitmap) + struct.pack("<i", len(huf)) + huf


def test_piz_hand_built_two_equal_words():
    """One HALF line of two words 0x0005: bit map byte 0 = bit 5; ranks
    0 -> 0, 5 -> 1; no wavelet level (one line); Huffman symbols 1 and the
    run symbol 2, both 1 bit long (codes 0 and 1); data "00"."""
    huf = _huf(1, 2, bytes([0x04, 0x10]), 2, bytes([0x00]))
    assert _bits((1, 6), (1, 6)) == bytes([0x04, 0x10])
    chunk = _piz(0, 0, [0x20], huf)
    out = exr._piz_decompress(chunk, [("Y", exr.HALF)], 2, 1)
    assert out == bytes([5, 0, 5, 0])


def test_piz_hand_built_run_code():
    """Ten equal words 0x0007 sent as the word, the run symbol and 9 in 8
    bits: "0" "1" "00001001"."""
    huf = _huf(1, 2, _bits((1, 6), (1, 6)), 10, _bits((0, 1), (1, 1), (9, 8)))
    chunk = _piz(0, 0, [0x80], huf)
    out = exr._piz_decompress(chunk, [("Y", exr.HALF)], 10, 1)
    assert out == bytes([7, 0]) * 10


def test_piz_hand_built_wavelet_block():
    """A 2x2 HALF block of words 1, 2 / 3, 4.  Ranks are the words (map
    byte 0 = bits 1-4, largest rank 4 < 2^14: the 14-bit pair transform).
    Encoding the block: rows (1, 2) -> (1, -1), (3, 4) -> (3, -1), then
    columns (1, 3) -> (2, -2), (-1, -1) -> (-1, 0): words 2, 0xFFFF, 0xFFFE, 0.
    Code lengths chosen by hand: 0, 2 and 0xFFFE 2 bits, 0xFFFF and the run
    symbol 0x10000 3 bits; canonical codes 01, 10, 11, 000, 001.  The table
    runs from symbol 0 to 0x10000: 2, 0, 2, 65531 zeros (251 long runs of
    261 and one of 20), 2, 3, 3."""
    table = [(2, 6), (0, 6), (2, 6)] + [(63, 6), (255, 8)] * 251 + [(63, 6), (14, 8)] + [(2, 6), (3, 6), (3, 6)]
    data = [(0b10, 2), (0b000, 3), (0b11, 2), (0b01, 2)]
    huf = _huf(0, 0x10000, _bits(*table), 9, _bits(*data))
    assert _bits(*data) == bytes([0x86, 0x80])
    chunk = _piz(0, 0, [0x1E], huf)
    out = exr._piz_decompress(chunk, [("Y", exr.HALF)], 2, 2)
    assert np.frombuffer(out, "<u2").tolist() == [1, 2, 3, 4]


def test_piz_hand_built_float_channel():
    """One FLOAT sample 1.0 (0x3F800000): words 0x0000, 0x3F80; map byte
    2032 = bit 0 (0x3F80 = 16256); ranks 0, 1; lengths 1, 2 and 2 for the
    run symbol: codes 1, 00, 01; data "1" "00"."""
    huf = _huf(0, 2, _bits((1, 6), (2, 6), (2, 6)), 3, _bits((1, 1), (0, 2)))
    chunk = _piz(2032, 2032, [0x01], huf)
    out = exr._piz_decompress(chunk, [("Z", exr.FLOAT)], 1, 1)
    assert struct.unpack("<f", out)[0] == 1.0


def test_piz_pair_transforms():
    """The 16-bit modular pair transform (largest rank >= 2^14), values
    worked by hand, and both transforms invert on every word pair class."""
    a, b = np.array([1, 40000]), np.array([3, 50000])
    l, h = exr._enc16(a, b)
    assert l.tolist() == [16386, 61384] and h.tolist() == [32766, 22768]
    ra, rb = exr._dec16(l, h)
    assert ra.tolist() == [1, 40000] and rb.tolist() == [3, 50000]
    rng = np.random.default_rng(9)
    x, y = rng.integers(0, 1 << 16, 5000), rng.integers(0, 1 << 16, 5000)
    assert [v.tolist() for v in exr._dec16(*exr._enc16(x, y))] == [x.tolist(), y.tolist()]
    x, y = rng.integers(0, 1 << 14, 5000), rng.integers(0, 1 << 14, 5000)
    assert [v.tolist() for v in exr._dec14(*exr._enc14(x, y))] == [x.tolist(), y.tolist()]


@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (32, 17), (7, 64), (32, 700)])
def test_piz_round_trip_chunks(shape):
    """The encoder's chunks decode back, odd sizes (odd rows and columns at
    several wavelet levels), FLOAT / UINT channels (two word planes) and
    more than 2^14 distinct words (the 16-bit transform)."""
    rng = np.random.default_rng(shape[1])
    h, w = shape
    chans = [("A", exr.HALF), ("B", exr.FLOAT), ("C", exr.UINT)]
    arrs = [rng.random((h, w)).astype(np.float16), rng.normal(size=(h, w)).astype(np.float32),
            rng.integers(0, 2**32, (h, w), dtype=np.uint64).astype(np.uint32)]
    raw = b"".join(a[r].tobytes() for r in range(h) for a in arrs)
    assert exr._piz_decompress(exr._piz_compress(raw, chans, w, h), chans, w, h) == raw


def test_piz_malformed_blocks_raise():
    huf = _huf(1, 2, _bits((1, 6), (1, 6)), 10, _bits((0, 1), (1, 1), (9, 8)))
    chunk = _piz(0, 0, [0x80], huf)
    with pytest.raises(exr.ExrError):  # one word more than the run gives
        exr._piz_decompress(chunk, [("Y", exr.HALF)], 11, 1)
    with pytest.raises(exr.ExrError):  # truncated bits
        exr._piz_decompress(chunk[:-1], [("Y", exr.HALF)], 10, 1)
    bad = _huf(1, 2, _bits((1, 6), (1, 6)), 10, _bits((1, 1), (1, 1), (9, 8)))  # a run before any word
    with pytest.raises(exr.ExrError):
        exr._piz_decompress(_piz(0, 0, [0x80], bad), [("Y", exr.HALF)], 10, 1)


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
