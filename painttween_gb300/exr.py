"""OpenEXR scanline files, and the reference's temporary images.

A reader and writer of single-part scanline OpenEXR files, written from the
published file layout (magic 20000630, version 2; attribute header; chunk
offset table; chunks of whole scanlines, channels sorted by name, each
channel's samples of a line stored together).  Compression NONE, RLE, ZIPS
and ZIP is read and written (ZIP and RLE apply the format's byte split and
delta predictor before deflate / run-length coding); PIZ, PXR24, B44 and DWA
files raise ExrError.  Pixel types UINT, HALF and FLOAT.

On top of it, the files the reference keeps between levels and passes
(src/PaintTweenCUDA/workingBuffers.cpp:166-207,242-296, imageIO.cpp:45,
118-122,159-186,340-390): `offsetsraw` holds PatchXF records as nine FLOAT
channels of layer "PatchXF", `output` the canvas and `residual` the residual
as half RGBA (residual in .b, scaled copies in .r and .g); names follow
ImageIO::temporaryOutputPath, `<dir>/<element>_<level>_<pass>_<version>.<frame
as 4 digits>.exr`.  The reference writes its RGBA files with PIZ; these are
written with ZIP, which every OpenEXR reader reads.
"""
import os
import struct
import zlib

import numpy as np

from . import _abi

MAGIC = 20000630
NONE, RLE, ZIPS, ZIP, PIZ = 0, 1, 2, 3, 4
_LINES = {NONE: 1, RLE: 1, ZIPS: 1, ZIP: 16}
UINT, HALF, FLOAT = 0, 1, 2
_DTYPES = {UINT: np.dtype("<u4"), HALF: np.dtype("<f2"), FLOAT: np.dtype("<f4")}
_PTYPE = {np.dtype("uint32"): UINT, np.dtype("float16"): HALF, np.dtype("float32"): FLOAT}


class ExrError(ValueError):
    pass


# --- byte transforms of the ZIP and RLE codecs ------------------------------

def _split_predict(raw):
    """Even bytes then odd bytes, then each byte as the difference to the
    previous one plus 128 (mod 256)."""
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]])
    if t.size > 1:
        d = t.astype(np.int16)
        d[1:] = (t[1:].astype(np.int16) - t[:-1].astype(np.int16) + 128) & 0xFF
        t = d.astype(np.uint8)
    return t.tobytes()


def _unpredict_join(buf):
    t = np.frombuffer(buf, np.uint8).astype(np.int64)
    if t.size > 1:
        t[1:] = t[1:] - 128
        t = np.cumsum(t) & 0xFF
    t = t.astype(np.uint8)
    n = t.size
    h = (n + 1) // 2
    out = np.empty(n, np.uint8)
    out[0::2] = t[:h]
    out[1::2] = t[h:]
    return out.tobytes()


def _rle_encode(data):
    out = bytearray()
    n, i = len(data), 0
    while i < n:
        j = i + 1
        while j < n and j - i < 128 and data[j] == data[i]:
            j += 1
        if j - i >= 3:  # a run
            out.append(j - i - 1)
            out.append(data[i])
            i = j
            continue
        j = i  # literals up to the next run of three
        while j < n and j - i < 127:
            if j + 2 < n and data[j] == data[j + 1] == data[j + 2]:
                break
            j += 1
        out.append((-(j - i)) & 0xFF)
        out += data[i:j]
        i = j
    return bytes(out)


def _rle_decode(data, size):
    out = bytearray()
    i = 0
    while i < len(data) and len(out) < size:
        c = struct.unpack_from("b", data, i)[0]
        i += 1
        if c < 0:
            out += data[i:i - c]
            i -= c
        else:
            out += bytes([data[i]]) * (c + 1)
            i += 1
    if len(out) != size:
        raise ExrError("RLE chunk decodes to %d bytes, expected %d" % (len(out), size))
    return bytes(out)


def _compress(raw, comp):
    if comp == NONE:
        return raw
    if comp in (ZIP, ZIPS):
        c = zlib.compress(_split_predict(raw))
    elif comp == RLE:
        c = _rle_encode(_split_predict(raw))
    else:
        raise ExrError("cannot write compression %d" % comp)
    return c if len(c) < len(raw) else raw  # stored raw when it does not shrink


def _decompress(data, comp, size):
    if comp == NONE or len(data) == size:
        return data
    if comp in (ZIP, ZIPS):
        return _unpredict_join(zlib.decompress(data))
    if comp == RLE:
        return _unpredict_join(_rle_decode(data, size))
    raise ExrError("compression %d is not supported (NONE, RLE, ZIPS and ZIP are)" % comp)


# --- header -------------------------------------------------------------------

def _cstr(data, i):
    j = data.index(b"\0", i)
    return data[i:j].decode("latin-1"), j + 1


def _parse_header(data):
    if len(data) < 8 or struct.unpack_from("<i", data, 0)[0] != MAGIC:
        raise ExrError("not an OpenEXR file")
    version = struct.unpack_from("<I", data, 4)[0]
    if version & 0xFF != 2:
        raise ExrError("OpenEXR version %d" % (version & 0xFF))
    if version & (0x200 | 0x800 | 0x1000):
        raise ExrError("only single-part scanline files are read")
    i, attrs = 8, {}
    while data[i] != 0:
        name, i = _cstr(data, i)
        typ, i = _cstr(data, i)
        size = struct.unpack_from("<i", data, i)[0]
        i += 4
        attrs[name] = (typ, data[i:i + size])
        i += size
    return attrs, i + 1


def _channels(raw):
    chans, i = [], 0
    while raw[i] != 0:
        name, i = _cstr(raw, i)
        ptype, _lin, xs, ys = struct.unpack_from("<iB3xii", raw, i)
        i += 16
        if xs != 1 or ys != 1:
            raise ExrError("subsampled channel %s" % name)
        chans.append((name, ptype))
    return chans


def read(path):
    """{'width', 'height', 'channels': {name: (h, w) array}, 'compression'}."""
    with open(path, "rb") as f:
        data = f.read()
    attrs, pos = _parse_header(data)
    for req in ("channels", "compression", "dataWindow"):
        if req not in attrs:
            raise ExrError("missing %s attribute" % req)
    chans = _channels(attrs["channels"][1])
    comp = attrs["compression"][1][0]
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = _LINES.get(comp)
    if lines is None:
        raise ExrError("compression %d is not supported (NONE, RLE, ZIPS and ZIP are)" % comp)
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack_from("<%dQ" % nchunks, data, pos)
    out = {name: np.empty((h, w), _DTYPES[pt]) for name, pt in chans}
    line_bytes = sum(w * _DTYPES[pt].itemsize for _, pt in chans)
    for off in offsets:
        y, size = struct.unpack_from("<ii", data, off)
        ly = y - y0
        n = min(lines, h - ly)
        raw = _decompress(data[off + 8:off + 8 + size], comp, n * line_bytes)
        k = 0
        for r in range(n):
            for name, pt in chans:
                nb = w * _DTYPES[pt].itemsize
                out[name][ly + r] = np.frombuffer(raw, _DTYPES[pt], w, k)
                k += nb
    return dict(width=w, height=h, channels=out, compression=comp)


def _attr(name, typ, value):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def write(path, channels, compression=ZIP):
    """Channels: {name: (h, w) array of float16, float32 or uint32}."""
    names = sorted(channels)
    if not names:
        raise ExrError("no channels")
    arrs = [np.ascontiguousarray(channels[n]) for n in names]
    h, w = arrs[0].shape
    types = []
    for n, a in zip(names, arrs):
        if a.shape != (h, w) or a.dtype not in _PTYPE:
            raise ExrError("channel %s: shape %s dtype %s" % (n, a.shape, a.dtype))
        types.append(_PTYPE[a.dtype])
    chl = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", t, 0, 1, 1) for n, t in zip(names, types)) + b"\0"
    box = struct.pack("<4i", 0, 0, w - 1, h - 1)
    header = (struct.pack("<iI", MAGIC, 2) + _attr("channels", "chlist", chl) +
              _attr("compression", "compression", bytes([compression])) + _attr("dataWindow", "box2i", box) +
              _attr("displayWindow", "box2i", box) + _attr("lineOrder", "lineOrder", bytes([0])) +
              _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              _attr("screenWindowCenter", "v2f", struct.pack("<2f", 0.0, 0.0)) +
              _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    lines = _LINES[compression]
    chunks = []
    for y in range(0, h, lines):
        raw = b"".join(a[r].astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
                       for r in range(y, min(y + lines, h)) for a in arrs)
        c = _compress(raw, compression)
        chunks.append(struct.pack("<ii", y, len(c)) + c)
    table_at = len(header)
    pos = table_at + 8 * len(chunks)
    table = []
    for c in chunks:
        table.append(pos)
        pos += len(c)
    with open(path, "wb") as f:
        f.write(header + struct.pack("<%dQ" % len(table), *table) + b"".join(chunks))


# --- the reference's temporary images ------------------------------------------

PATCHXF_CHANNELS = ("x", "y", "theta", "hyst", "layer", "lumShift_y", "lumShift_a", "scale_u", "scale_v")
_PATCHXF_FIELDS = ("x", "y", "theta", "hysteresis", "layer", "lumShiftY", "lumShiftA", "scaleU", "scaleV")


def temporary_path(directory, element, level, frame, pass_, version=0):
    """ImageIO::temporaryOutputPath over NLDataAccess::getOutPath
    (imageIO.h:118-122, nlDataAccess.cpp:427-433)."""
    return os.path.join(directory, "%s_%d_%d_%d.%04d.exr" % (element, level, pass_, version, frame))


def write_offsets(path, offsets):
    """offsetsraw: PatchXF as nine FLOAT channels (imageIO.cpp:373-390); the
    header's default compression is ZIP."""
    o = np.asarray(offsets)
    chans = {"PatchXF." + c: o[f].astype(np.float32) for c, f in zip(PATCHXF_CHANNELS, _PATCHXF_FIELDS)}
    write(path, chans, ZIP)


def read_offsets(path):
    """ImageIO::readImage for PatchXF (imageIO.cpp:159-186): the layer
    channel converted to int by truncation."""
    img = read(path)
    ch = img["channels"]
    out = np.zeros((img["height"], img["width"]), _abi.PATCH_DTYPE)
    for c, f in zip(PATCHXF_CHANNELS, _PATCHXF_FIELDS):
        v = ch["PatchXF." + c].astype(np.float32)
        out[f] = np.trunc(v).astype(np.int32) if f == "layer" else v
    return out


def write_rgba(path, rgba, compression=ZIP):
    """Half RGBA (RgbaOutputFile, WRITE_RGBA; imageIO.cpp:340-371)."""
    a = np.asarray(rgba, np.float32)
    write(path, {c: a[..., i].astype(np.float16) for i, c in enumerate("RGBA")}, compression)


def read_rgba(path):
    """RGBA as float32 (R, G, B, A; a missing A reads 1, missing colours 0)."""
    img = read(path)
    ch = img["channels"]
    out = np.zeros((img["height"], img["width"], 4), np.float32)
    out[..., 3] = 1.0
    for i, c in enumerate("RGBA"):
        if c in ch:
            out[..., i] = ch[c].astype(np.float32)
    return out


def write_residual(path, residual):
    """saveTempImages' residual image (workingBuffers.cpp:264-269): r =
    0.0001 res, g = 0.01 res, b = res, a = 1, as half."""
    r = np.asarray(residual, np.float32)
    rgba = np.stack([r * np.float32(0.0001), r * np.float32(0.01), r, np.ones_like(r)], axis=-1)
    write_rgba(path, rgba)


def read_residual(path):
    """WorkingBuffers::loadResidual (workingBuffers.cpp:166-188): the .b
    channel."""
    return read_rgba(path)[..., 2].copy()


def save_temp_images(directory, level, frame, pass_, offsets, output, residual, version=0):
    """The offsetsraw, output and residual files of WorkingBuffers::
    saveTempImages (the display-only offsets colour map is not written)."""
    write_offsets(temporary_path(directory, "offsetsraw", level, frame, pass_, version), offsets)
    write_rgba(temporary_path(directory, "output", level, frame, pass_, version), output)
    write_residual(temporary_path(directory, "residual", level, frame, pass_, version), residual)


def load_temp_images(directory, level, frame, pass_, version=0):
    """(offsets, output, residual) of one saved pass."""
    return (read_offsets(temporary_path(directory, "offsetsraw", level, frame, pass_, version)),
            read_rgba(temporary_path(directory, "output", level, frame, pass_, version)),
            read_residual(temporary_path(directory, "residual", level, frame, pass_, version)))
