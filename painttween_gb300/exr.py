"""OpenEXR scanline files, and the reference's temporary images.

A reader and writer of single-part scanline OpenEXR files, written from the
published file layout (magic 20000630, version 2; attribute header; chunk
offset table; chunks of whole scanlines, channels sorted by name, each
channel's samples of a line stored together).  Compression NONE, RLE, ZIPS,
ZIP and PIZ is read and written (ZIP and RLE apply the format's byte split
and delta predictor before deflate / run-length coding; PIZ is the format's
wavelet + Huffman codec, restated below); PXR24, B44 and DWA files raise
ExrError.  Pixel types UINT, HALF and FLOAT.

The codecs belong to OpenEXR's IlmImf library, which the reference links
without pinning a version (src/PaintTweenCUDA/CMakeLists.txt:94); the PIZ
layout has not changed across OpenEXR's releases.

On top of it, the files the reference keeps between levels and passes
(src/PaintTweenCUDA/workingBuffers.cpp:166-207,242-296, imageIO.cpp:45,
118-122,159-186,340-390): `offsetsraw` holds PatchXF records as nine FLOAT
channels of layer "PatchXF", `output` the canvas and `residual` the residual
as half RGBA (residual in .b, scaled copies in .r and .g); names follow
ImageIO::temporaryOutputPath, `<dir>/<element>_<level>_<pass>_<version>.<frame
as 4 digits>.exr`.  The reference writes its RGBA files with PIZ
(imageIO.h:131-133), and so does write_rgba by default.
"""
import os
import struct
import zlib

import numpy as np

from . import _abi

MAGIC = 20000630
NONE, RLE, ZIPS, ZIP, PIZ = 0, 1, 2, 3, 4
_LINES = {NONE: 1, RLE: 1, ZIPS: 1, ZIP: 16, PIZ: 32}
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


# --- PIZ: value map, 2-D wavelet and Huffman coding of 16-bit words ----------
#
# A PIZ chunk (32 scanlines) is coded as 16-bit words: each channel's samples
# of all the chunk's lines in turn (channels in file order), a HALF sample one
# word, a FLOAT or UINT sample two (its low and high halves, little-endian).
# 1. The words that occur, except 0, are marked in a 65536-bit map; every
#    word is replaced by its rank among the marked values and 0 (0 -> 0).
# 2. Each channel's plane of words (for 32-bit types each half separately,
#    x stride 2) gets a 2-D Haar-like lifting wavelet: levels p = 1, 2, 4, ...
#    while 2p <= min(nx, ny), on the 2x2 blocks at multiples of 2p, then an
#    odd column (when nx & p) and an odd row (when ny & p).  The pair
#    transform is the 14-bit one (mean and difference in 16-bit signed
#    arithmetic) when the largest rank is below 2^14, else a 16-bit modular one.
# 3. The words are Huffman coded: code lengths of the symbols im..iM (iM is a
#    run symbol one above the largest word) packed in 6 bits each, runs of
#    zero lengths as 59..62 (2-5 zeros) or 63 + 8 bits (6-261 zeros); the
#    canonical codes give the longest lengths the numerically lowest codes;
#    a run of r + 1 equal words may be sent as the word, the run symbol and
#    r in 8 bits.  Bits are packed most significant first.
# Chunk layout: u16 first and u16 last non-zero byte of the bit map, those
# bytes of the map, i32 length of the Huffman block; the Huffman block holds
# u32 im, iM, table bytes, bit count, 0, then the table and the bits.

_BITMAP_BYTES = 8192
_SHORT_ZERO_RUN, _LONG_ZERO_RUN = 59, 63
_SHORTEST_LONG_RUN = 2 + _LONG_ZERO_RUN - _SHORT_ZERO_RUN  # 6
_LONGEST_LONG_RUN = 255 + _SHORTEST_LONG_RUN                # 261
_MAX_CODE_LEN = 58


def _as_i16(a):
    return a.astype(np.uint16).view(np.int16).astype(np.int32)


def _enc14(a, b):
    sa, sb = _as_i16(a), _as_i16(b)
    return ((sa + sb) >> 1) & 0xFFFF, (sa - sb) & 0xFFFF


def _dec14(l, h):
    sl, sh = _as_i16(l), _as_i16(h)
    ai = sl + (sh & 1) + (sh >> 1)
    return ai & 0xFFFF, (ai - sh) & 0xFFFF


def _enc16(a, b):
    ao = (a.astype(np.int32) + 0x8000) & 0xFFFF
    b = b.astype(np.int32)
    m = (ao + b) >> 1
    d = ao - b
    m = np.where(d < 0, (m + 0x8000) & 0xFFFF, m)
    return m, d & 0xFFFF


def _dec16(l, h):
    m, d = l.astype(np.int32), h.astype(np.int32)
    b = (m - (d >> 1)) & 0xFFFF
    return (d + b - 0x8000) & 0xFFFF, b


def _wavelet_levels(nx, ny):
    n, p, out = min(nx, ny), 1, []
    while 2 * p <= n:
        out.append(p)
        p *= 2
    return out


def _wavelet(z, mx, inverse):
    """The PIZ wavelet of one plane z (ny, nx) of words, in place."""
    ny, nx = z.shape
    enc, dec = (_enc14, _dec14) if mx < (1 << 14) else (_enc16, _dec16)
    levels = _wavelet_levels(nx, ny)
    for p in (levels[::-1] if inverse else levels):
        p2 = 2 * p
        rb, cb = (ny // p2) * p2, (nx // p2) * p2  # the blocks' extent; the odd row / column start there
        a = z[0:rb:p2, 0:cb:p2]
        a01 = z[0:rb:p2, p:cb:p2]
        a10 = z[p:rb:p2, 0:cb:p2]
        a11 = z[p:rb:p2, p:cb:p2]
        if not inverse:
            i00, i01 = enc(a, a01)
            i10, i11 = enc(a10, a11)
            a[...], a10[...] = enc(i00, i10)
            a01[...], a11[...] = enc(i01, i11)
        else:
            i00, i10 = dec(a, a10)
            i01, i11 = dec(a01, a11)
            a[...], a01[...] = dec(i00, i01)
            a10[...], a11[...] = dec(i10, i11)
        f = dec if inverse else enc
        if nx & p:  # odd column, beside the block rows
            c, c10 = z[0:rb:p2, cb], z[p:rb:p2, cb]
            c[...], c10[...] = f(c, c10)
        if ny & p:  # odd row, below the block rows
            r, r01 = z[rb, 0:cb:p2], z[rb, p:cb:p2]
            r[...], r01[...] = f(r, r01)


def _canonical_codes(lengths):
    """Codes of the canonical table for code lengths (0: no code): the
    lowest code of each length counts down from the longest length, and the
    codes of one length rise with the symbol."""
    lengths = np.asarray(lengths, np.int64)
    counts = np.bincount(lengths, minlength=_MAX_CODE_LEN + 1)
    first = np.zeros(_MAX_CODE_LEN + 1, np.int64)
    c = 0
    for ln in range(_MAX_CODE_LEN, 0, -1):
        first[ln] = c
        c = (c + int(counts[ln])) >> 1
    syms = np.nonzero(lengths)[0]
    lens = lengths[syms]
    order = np.lexsort((syms, lens))  # by length, then symbol
    rank = np.empty(syms.size, np.int64)
    group_start = np.concatenate([[0], np.cumsum(counts[1:])])[lens[order] - 1]
    rank[order] = np.arange(syms.size) - group_start
    codes = np.zeros(lengths.size, np.int64)
    codes[syms] = first[lens] + rank
    return codes


def _pack_bits(vals, lens):
    """The values, each in its number of bits, most significant bit first,
    packed into bytes (the last byte padded with zeros); and the bit count."""
    vals = np.asarray(vals, np.int64)
    lens = np.asarray(lens, np.int64)
    nbits = int(lens.sum())
    owner = np.repeat(np.arange(vals.size), lens)
    pos = np.arange(nbits) - np.repeat(np.cumsum(lens) - lens, lens)
    bits = (vals[owner] >> (lens[owner] - 1 - pos)) & 1
    return np.packbits(bits.astype(np.uint8)).tobytes(), nbits


def _huf_lengths(freq):
    """Huffman code lengths of the symbols with nonzero frequency (merging
    the two least frequent nodes until one is left; a node's depth is its
    code length)."""
    import heapq
    syms = np.nonzero(freq)[0]
    lengths = np.zeros(len(freq), np.int64)
    if len(syms) == 1:
        lengths[syms[0]] = 1
        return lengths
    heap = [(int(freq[s]), k) for k, s in enumerate(syms)]
    heapq.heapify(heap)
    parent = [0] * (2 * len(syms) - 1)
    nxt = len(syms)
    while len(heap) > 1:
        f0, a = heapq.heappop(heap)
        f1, b = heapq.heappop(heap)
        parent[a] = parent[b] = nxt
        heapq.heappush(heap, (f0 + f1, nxt))
        nxt += 1
    depth = [0] * nxt
    for k in range(nxt - 2, -1, -1):  # parents are made after their children
        depth[k] = depth[parent[k]] + 1
    lengths[syms] = depth[:len(syms)]
    if lengths.max() > _MAX_CODE_LEN:
        raise ExrError("Huffman code longer than %d bits" % _MAX_CODE_LEN)
    return lengths


def _pack_table(lengths, im, iM):
    """The code lengths of symbols im..iM in 6 bits each, zero runs of 2-5
    as 59-62 and of 6-261 as 63 plus 8 bits."""
    seg = lengths[im:iM + 1]
    vals, lens = [], []
    i, n = 0, seg.size
    nz = np.nonzero(seg)[0].tolist() + [n]
    k = 0
    while i < n:
        if seg[i]:
            vals.append(int(seg[i]))
            lens.append(6)
            i += 1
            continue
        while nz[k] < i:
            k += 1
        zr = nz[k] - i  # zeros from i on
        while zr > 0:
            run = min(zr, _LONGEST_LONG_RUN)
            if run >= _SHORTEST_LONG_RUN:
                vals += [_LONG_ZERO_RUN, run - _SHORTEST_LONG_RUN]
                lens += [6, 8]
            elif run >= 2:
                vals.append(_SHORT_ZERO_RUN + run - 2)
                lens.append(6)
            else:
                vals.append(0)
                lens.append(6)
            zr -= run
            i += run
    return _pack_bits(vals, lens)[0]


def _huf_compress(words):
    """The Huffman block of a sequence of 16-bit words."""
    words = np.asarray(words, np.int64)
    if words.size == 0:
        return b""
    freq = np.bincount(words, minlength=65537)
    im = int(np.nonzero(freq)[0][0])
    rlc = int(np.nonzero(freq)[0][-1]) + 1  # the run symbol
    freq[rlc] = 1
    lengths = _huf_lengths(freq)
    codes = _canonical_codes(lengths)
    table = _pack_table(lengths, im, rlc)
    # runs of equal words, cut into pieces of at most 256: a piece is sent
    # as its word and the run symbol with the repeat count when that is
    # shorter, else as its words
    starts = np.concatenate([[0], np.nonzero(words[1:] != words[:-1])[0] + 1])
    ends = np.concatenate([starts[1:], [words.size]])
    runlen = ends - starts
    pieces = (runlen + 255) // 256
    psym = np.repeat(words[starts], pieces)
    first_piece = np.repeat(np.cumsum(pieces) - pieces, pieces)
    pidx = np.arange(psym.size) - first_piece
    plen = np.minimum(np.repeat(runlen, pieces) - 256 * pidx, 256)
    ls = lengths[psym]
    lr = int(lengths[rlc])
    coded = ls + lr + 8 < ls * (plen - 1)
    # the emitted (code, length) pairs, piece by piece
    n_emit = np.where(coded, 3, plen)
    em_piece = np.repeat(np.arange(psym.size), n_emit)
    em_k = np.arange(em_piece.size) - np.repeat(np.cumsum(n_emit) - n_emit, n_emit)
    em_coded = coded[em_piece]
    em_sym = psym[em_piece]
    em_val = np.where(em_coded & (em_k == 1), codes[rlc], codes[em_sym])
    em_len = np.where(em_coded & (em_k == 1), lr, lengths[em_sym])
    cnt = em_coded & (em_k == 2)
    em_val = np.where(cnt, plen[em_piece] - 1, em_val)
    em_len = np.where(cnt, 8, em_len)
    data, nbits = _pack_bits(em_val, em_len)
    return struct.pack("<5I", im, rlc, len(table), nbits, 0) + table + data


def _huf_decompress(buf, n_words):
    """n_words 16-bit words from a Huffman block (pt_piz_huffman_decode in
    the native library)."""
    from ._lib import lib
    out = np.empty(max(n_words, 1), np.uint16)
    b = np.frombuffer(bytes(buf), np.uint8) if len(buf) else np.zeros(1, np.uint8)
    st = lib().pt_piz_huffman_decode(b.ctypes.data, len(buf), out.ctypes.data, n_words)
    if st != _abi.PT_OK:
        raise ExrError("PIZ: malformed Huffman block (%d bytes, %d words expected)" % (len(buf), n_words))
    return out[:n_words]


def _piz_planes(words, chans, w, n):
    """The wavelet planes of a chunk's words: (plane view (ny, nx) with x
    stride `size`) per channel half."""
    out, k = [], 0
    for _, pt in chans:
        size = _DTYPES[pt].itemsize // 2
        blk = words[k:k + n * w * size].reshape(n, w, size)
        for j in range(size):
            out.append(blk[:, :, j])
        k += n * w * size
    return out


def _chunk_words(raw, chans, w, n):
    """The chunk's bytes (line by line, channel by channel) as PIZ words
    (channel by channel, line by line)."""
    b = np.frombuffer(raw, np.uint8)
    per_line = [w * _DTYPES[pt].itemsize for _, pt in chans]
    lines = b.reshape(n, sum(per_line))
    parts, k = [], 0
    for nb in per_line:
        parts.append(lines[:, k:k + nb].reshape(-1))
        k += nb
    return np.concatenate(parts).view("<u2").astype(np.int64)


def _chunk_bytes(words, chans, w, n):
    per_line = [w * _DTYPES[pt].itemsize for _, pt in chans]
    wb = words.astype("<u2").view(np.uint8)
    out = np.empty((n, sum(per_line)), np.uint8)
    k = kb = 0
    for nb in per_line:
        out[:, kb:kb + nb] = wb[k:k + n * nb].reshape(n, nb)
        k += n * nb
        kb += nb
    return out.tobytes()


def _piz_compress(raw, chans, w, n):
    words = _chunk_words(raw, chans, w, n)
    present = np.zeros(65536, bool)
    present[words] = True
    present[0] = False
    bitmap = np.packbits(present, bitorder="little")
    nz = np.nonzero(bitmap)[0]
    lo, hi = (int(nz[0]), int(nz[-1])) if nz.size else (_BITMAP_BYTES - 1, 0)
    present[0] = True
    rank = np.cumsum(present) - 1  # word -> its rank among the present values
    mx = int(rank[-1])
    mapped = rank[words].astype(np.int64)
    for z in _piz_planes(mapped, chans, w, n):
        _wavelet(z, mx, inverse=False)
    huf = _huf_compress(mapped)
    head = struct.pack("<HH", lo, hi) + (bitmap[lo:hi + 1].tobytes() if lo <= hi else b"")
    return head + struct.pack("<i", len(huf)) + huf


def _piz_decompress(data, chans, w, n):
    if len(data) < 4:
        raise ExrError("PIZ: truncated chunk")
    lo, hi = struct.unpack_from("<HH", data, 0)
    if hi >= _BITMAP_BYTES:
        raise ExrError("PIZ: bit map ends at byte %d" % hi)
    bitmap = np.zeros(_BITMAP_BYTES, np.uint8)
    k = 4
    if lo <= hi:
        bitmap[lo:hi + 1] = np.frombuffer(data, np.uint8, hi - lo + 1, k)
        k += hi - lo + 1
    present = np.unpackbits(bitmap, bitorder="little").astype(bool)
    present[0] = True
    values = np.nonzero(present)[0]  # rank -> word
    mx = values.size - 1
    (length,) = struct.unpack_from("<i", data, k)
    k += 4
    n_words = sum(n * w * (_DTYPES[pt].itemsize // 2) for _, pt in chans)
    words = _huf_decompress(data[k:k + length], n_words).astype(np.int64)
    for z in _piz_planes(words, chans, w, n):
        _wavelet(z, mx, inverse=True)
    if words.size and words.max() > mx:
        raise ExrError("PIZ: decoded rank %d above the map's %d" % (words.max(), mx))
    return _chunk_bytes(values[words], chans, w, n)


def _compress(raw, comp, layout=None):
    if comp == NONE:
        return raw
    if comp in (ZIP, ZIPS):
        c = zlib.compress(_split_predict(raw))
    elif comp == RLE:
        c = _rle_encode(_split_predict(raw))
    elif comp == PIZ:
        c = _piz_compress(raw, *layout)
    else:
        raise ExrError("cannot write compression %d" % comp)
    return c if len(c) < len(raw) else raw  # stored raw when it does not shrink


def _decompress(data, comp, size, layout=None):
    if comp == NONE or len(data) == size:
        return data
    if comp in (ZIP, ZIPS):
        return _unpredict_join(zlib.decompress(data))
    if comp == RLE:
        return _unpredict_join(_rle_decode(data, size))
    if comp == PIZ:
        return _piz_decompress(data, *layout)
    raise ExrError("compression %d is not supported (NONE, RLE, ZIPS, ZIP and PIZ are)" % comp)


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
        raise ExrError("compression %d is not supported (NONE, RLE, ZIPS, ZIP and PIZ are)" % comp)
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack_from("<%dQ" % nchunks, data, pos)
    out = {name: np.empty((h, w), _DTYPES[pt]) for name, pt in chans}
    line_bytes = sum(w * _DTYPES[pt].itemsize for _, pt in chans)
    for off in offsets:
        y, size = struct.unpack_from("<ii", data, off)
        ly = y - y0
        n = min(lines, h - ly)
        raw = _decompress(data[off + 8:off + 8 + size], comp, n * line_bytes, (chans, w, n))
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
    chans = list(zip(names, types))
    chunks = []
    for y in range(0, h, lines):
        raw = b"".join(a[r].astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
                       for r in range(y, min(y + lines, h)) for a in arrs)
        c = _compress(raw, compression, (chans, w, min(lines, h - y)))
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


def write_rgba(path, rgba, compression=PIZ):
    """Half RGBA (RgbaOutputFile, WRITE_RGBA; imageIO.cpp:340-371), PIZ
    compressed as the reference's (imageIO.h:131-133)."""
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
