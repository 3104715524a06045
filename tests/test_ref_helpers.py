"""The oracle's restated helpers against the reference's own code.

src/PaintTweenCUDA/texSynth_util.h (colour conversion, exemplar basis and
coordinates, clamping, squared differences, ribbon unpacking) and
src/PaintTweenCUDA/cudaImageBuffer.h (pixelWrap and inBounds: the level-0
wrap that coarse levels read through) and src/PaintTweenCUDA/downsample.cpp
(host pyramids: 2x2 averages, velocity scaling, majority vote of object
ids) compile for the host; oracle/build.py builds them through
oracle/ref_helpers.cpp and oracle/ref_downsample.cpp
(downsample.cpp over the QtCore container shim oracle/qt_shim) into
oracle/_ref/libref_helpers.so where the reference tree is present.  These
tests are skipped where it is not (the library is built from the reference's
sources and never committed).

Exactness: the shim is compiled with FP contraction on, as nvcc compiles the
reference's device code (--fmad=true), so its sums of products become fused
multiply-adds: gcc fuses the first product of a sum of two products with
the second (nvcc mostly does the same, depending on the surrounding code).
The oracle and the kernels write their fused multiply-adds out by their own
fixed specification: exemplar coordinates fuse the first product, as gcc
does here, and agree bit for bit;
squared differences fuse the running sum with each next product, so they
agree bit for bit on most inputs and within 2 ulp on all.  Clamping and
ribbon unpacking agree bit for bit.  The basis calls cos/sin
(host libm here, CUDA's device functions in the reference) where the oracle
and the kernels share their own sincos polynomial: within 2 ulp.  RGBtoLAB
calls pow: within 1e-6.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import build as ob
from oracle import oracle as O
from painttween_gb300 import _abi

pytestmark = pytest.mark.skipif(
    not os.path.exists(os.path.join(ob.REF_SRC, "texSynth_util.h")),
    reason="reference tree absent: oracle/_ref/libref_helpers.so cannot be built")

_REF = None


def ref():
    global _REF
    if _REF is None:
        L = ctypes.CDLL(ob.build_ref())
        vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        for name, (res, args) in {
            "ref_rgb_to_lab": (None, [vp, vp]),
            "ref_basis": (None, [f, f, f, vp]),
            "ref_new_coord": (None, [f, f, f, f, vp, vp]),
            "ref_clamp_to_exemplar": (None, [vp, vp, i, i]),
            "ref_ssd": (f, [vp, vp, f]),
            "ref_ssd_plain": (f, [vp, vp]),
            "ref_ribbon_of": (None, [vp, vp, vp]),
            "ref_pyramid_rgba": (i, [vp, i, i, i, vp]),
            "ref_pyramid_float": (i, [vp, i, i, i, vp]),
            "ref_pyramid_float2": (i, [vp, i, i, i, vp]),
            "ref_pyramid_int": (i, [vp, i, i, vp]),
            "ref_pixel_wrap": (i, [vp, i, i, i, i]),
            "ref_in_bounds": (i, [i, i, i, i, i, i]),
            "ref_to_patchxf": (i, [vp, vp]),
            "ref_param_field": (i, [i, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_long),
                                    ctypes.POINTER(ctypes.c_long)]),
            "ref_layer": (i, [i, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_long)]),
            "ref_param_constants": (None, [vp]),
            "ref_flags": (None, [vp]),
            "ref_record_layouts": (None, [vp]),
        }.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _REF = L
    return _REF


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def test_shim_builds_and_exports():
    L = ref()
    for name in ("ref_rgb_to_lab", "ref_basis", "ref_new_coord", "ref_clamp_to_exemplar",
                 "ref_ssd", "ref_ssd_plain", "ref_ribbon_of"):
        assert hasattr(L, name)


def test_squared_differences_within_2ulp():
    rng = np.random.default_rng(5)
    R, OL = ref(), O.lib()
    exact, n = 0, 4000
    for k in range(n):
        a = rng.random(4, dtype=np.float32) * np.float32(rng.choice([1, 100]))
        b = rng.random(4, dtype=np.float32)
        alpha = np.float32(rng.random() * 4)
        if k % 2:
            r, o = R.ref_ssd(_p(a), _p(b), alpha), OL.pto_ssd(_p(a), _p(b), alpha)
        else:
            r, o = R.ref_ssd_plain(_p(a), _p(b)), OL.pto_ssd_plain(_p(a), _p(b))
        assert _ulp_diff(r, o) <= 2, (a, b, alpha, r, o)
        exact += np.float32(r).tobytes() == np.float32(o).tobytes()
    assert exact >= 0.8 * n


def test_exemplar_coordinates_bit_exact():
    rng = np.random.default_rng(6)
    R, OL = ref(), O.lib()
    ro, oo = np.empty(2, np.float32), np.empty(2, np.float32)
    for _ in range(2000):
        i, j = (np.float32(v) for v in rng.integers(-8, 9, 2))
        ex, ey = (np.float32(v) for v in rng.random(2) * 512)
        b = (rng.random(4) * 2 - 1).astype(np.float32)
        R.ref_new_coord(i, j, ex, ey, _p(b), _p(ro))
        OL.pto_new_coord(i, j, ex, ey, _p(b), _p(oo))
        assert ro.tobytes() == oo.tobytes(), (i, j, ex, ey, b, ro, oo)


def test_clamp_to_exemplar_bit_exact():
    R, OL = ref(), O.lib()
    for x0 in (-3.5, -0.0, 0.0, 0.25, 63.0, 63.99, 64.0, 1e9, float("-inf")):
        for y0 in (-1.0, 10.5, 47.0, 48.0):
            rx, ry = ctypes.c_float(x0), ctypes.c_float(y0)
            ox, oy = ctypes.c_float(x0), ctypes.c_float(y0)
            R.ref_clamp_to_exemplar(ctypes.byref(rx), ctypes.byref(ry), 64, 48)
            OL.pto_clamp_to_exemplar(ctypes.byref(ox), ctypes.byref(oy), 64, 48)
            assert (rx.value, ry.value) == (ox.value, oy.value), (x0, y0)


def test_ribbon_unpacking_bit_exact():
    rng = np.random.default_rng(7)
    R, OL = ref(), O.lib()
    rxy, oxy = np.empty(2, np.float32), np.empty(2, np.float32)
    rtl, otl = np.empty(2, np.int32), np.empty(2, np.int32)
    cases = [np.array([1, 2.5, 3.5, 0], np.float32), np.array([-1, 0, 0, -1], np.float32),
             np.array([-1.5, 7.25, -3.0, 2.9], np.float32), np.array([4.99, 0.5, 0.5, -0.5], np.float32)]
    cases += [((rng.random(4) * 200) - 50).astype(np.float32) for _ in range(500)]
    for c in cases:
        R.ref_ribbon_of(_p(c), _p(rxy), _p(rtl))
        OL.pto_ribbon_of(_p(c), _p(oxy), _p(otl))
        assert rxy.tobytes() == oxy.tobytes() and (rtl == otl).all(), (c, rxy, rtl, oxy, otl)


def test_exemplar_basis_within_2ulp():
    rng = np.random.default_rng(8)
    R, OL = ref(), O.lib()
    ro, oo = np.empty(4, np.float32), np.empty(4, np.float32)
    angles = np.concatenate([np.float32([0, np.pi / 2, -np.pi / 2, np.pi, 1e-8]),
                             (rng.random(3000) * 2 * np.pi - np.pi).astype(np.float32)])
    worst = 0
    for a in angles:
        su, sv = (np.float32(v) for v in rng.random(2) * 2 + 0.25)
        R.ref_basis(a, su, sv, _p(ro))
        OL.pto_basis(a, su, sv, _p(oo))
        d = _ulp_diff(ro, oo)
        # near zeros of sin/cos an ulp of the result is tiny: the bound there
        # is absolute, one ulp of the scale
        small = np.abs(ro) < 1e-3
        assert (d[~small] <= 2).all(), (a, su, sv, ro, oo)
        assert (np.abs(ro - oo)[small] <= 2.5e-7 * max(su, sv)).all(), (a, su, sv, ro, oo)
        worst = max(worst, int(d[~small].max(initial=0)))
    assert worst <= 2


def test_rgb_to_lab_against_reference():
    rng = np.random.default_rng(9)
    R = ref()
    ro = np.empty(4, np.float32)
    cols = [np.float32([0, 0, 0, 1]), np.float32([1, 1, 1, 0.5]), np.float32([0.2, 0.5, 0.9, 1]),
            np.float32([0.04045, 0.0031308, 0.008856, 1])]
    cols += [rng.random(4, dtype=np.float32) for _ in range(3000)]
    for c in cols:
        R.ref_rgb_to_lab(_p(c), _p(ro))
        oo = O.rgb_to_lab(c)
        assert np.abs(ro - oo).max() <= 1e-6, (c, ro, oo)


def _ref_levels(fn, img, w, h, ch, dtype, *mode):
    n = sum((w >> l) * (h >> l) for l in range(O.num_levels(w, h))) * ch
    out = np.empty(n, dtype)
    nl = fn(_p(np.ascontiguousarray(img)), w, h, *mode, _p(out))
    assert nl == O.num_levels(w, h)
    levels, off = [], 0
    for l in range(nl):
        k = (w >> l) * (h >> l) * ch
        levels.append(out[off:off + k])
        off += k
    return levels


@pytest.mark.parametrize("w,h", [(64, 48), (37, 20), (128, 128), (9, 300)])
def test_pyramids_bit_exact_with_reference_downsample(w, h):
    """downsamplePyramid<Color4/float/float2> (2x2 averages, with and without
    the per-level halving of velocities) against the oracle's pyramids."""
    rng = np.random.default_rng(w * 1000 + h)
    R = ref()
    for ch, fn in ((4, R.ref_pyramid_rgba), (1, R.ref_pyramid_float), (2, R.ref_pyramid_float2)):
        img = (rng.standard_normal((h, w, ch)) * 3).astype(np.float32)
        for scale_with_levels in (0, 1):
            ref_levels = _ref_levels(fn, img, w, h, ch, np.float32, scale_with_levels)
            ours = O.pyramid_avg(img if ch > 1 else img[..., 0], vel=bool(scale_with_levels))
            assert len(ours) == len(ref_levels)
            for a, b in zip(ours, ref_levels):
                assert a.reshape(-1).tobytes() == b.tobytes(), (ch, scale_with_levels)


@pytest.mark.parametrize("w,h,k", [(64, 48, 3), (37, 20, 2), (128, 64, 6), (16, 16, 1)])
def test_object_id_vote_bit_exact_with_reference_downsample(w, h, k):
    """downsamplePyramid<int> (majority vote of the 2x2 ids through QHash and
    QMap) against the oracle's vote.  Ties follow the container shim's hash
    order (descending ids, one of the orders Qt may give): the smallest id."""
    rng = np.random.default_rng(w + h + k)
    ids = rng.integers(-1, k, (h, w)).astype(np.int32)
    ref_levels = _ref_levels(ref().ref_pyramid_int, ids, w, h, 1, np.int32)
    ours = O.pyramid_vote(ids)
    assert len(ours) == len(ref_levels)
    for a, b in zip(ours, ref_levels):
        assert (a.reshape(-1) == b).all()


@pytest.mark.parametrize("w,h", [(64, 48), (37, 20), (1920, 1080), (5, 3)])
def test_pixel_wrap_and_bounds_bit_exact(w, h):
    """CudaImageBufferDevice::pixelWrap (floorf-based wrap by the buffer's
    level-0 size, which coarse levels read through) and inBounds (the level
    rectangle with a border) against the oracle's restatements, over
    coordinates from several periods below zero to several above."""
    R, OL = ref(), O.lib()
    index_image = np.arange(w * h, dtype=np.int32)
    xs = list(range(-3 * w - 2, -3 * w + 3)) + list(range(-w - 2, w + 3)) + list(range(3 * w - 2, 3 * w + 3))
    ys = list(range(-2 * h - 2, -2 * h + 3)) + list(range(-h - 2, h + 3)) + list(range(2 * h - 2, 2 * h + 3))
    for y in ys[:: max(1, len(ys) // 40)] + [ys[0], ys[-1], 0, -1, h - 1, h]:
        for x in xs[:: max(1, len(xs) // 60)] + [xs[0], xs[-1], 0, -1, w - 1, w]:
            assert R.ref_pixel_wrap(_p(index_image), w, h, x, y) == OL.pto_pixel_wrap(w, h, x, y), (x, y)
    for level in range(4):
        for border in (0, 1, 3):
            for y in (-1, 0, 1, 2, (h >> level) - 4, (h >> level) - 1, h >> level, h):
                for x in (-1, 0, 1, 2, (w >> level) - 4, (w >> level) - 1, w >> level, w):
                    assert R.ref_in_bounds(w, h, x, y, level, border) == OL.pto_in_bounds(w, h, x, y, level, border)


def test_random_texel_to_patchxf_bit_exact():
    """toPatchXF (the random layer's packed texel as a PatchXF: zero
    hysteresis, unit scale, layer truncated) against the oracle, all 36
    bytes of the record."""
    R, OL = ref(), O.lib()
    rng = np.random.default_rng(17)
    cases = [np.float32([3.25, 7.5, 0.3, 0.0]), np.float32([0.0, 0.0, -1.2, 2.9]),
             np.float32([5.5, 1.0, 3.0, -0.5]), np.float32([1.0, 2.0, 0.0, -1.5])]
    cases += [np.float32([rng.random() * 500, rng.random() * 500, rng.random() * 6 - 3, rng.integers(0, 8)])
              for _ in range(300)]
    for c in cases:
        r = np.zeros(36, np.uint8)
        o = np.zeros(1, _abi.PATCH_DTYPE)
        assert R.ref_to_patchxf(_p(c), _p(r)) == 36
        OL.pto_to_patchxf(_p(c), _p(o))
        assert r.tobytes() == o.tobytes(), (c, r, o)


def test_params_mirror_tsparameters_field_for_field():
    """pt_params lists TsParameters' fields (texSynth_interface.h) by name and
    in order, each the same size except the reference's bools, which are
    int32 here; the fields after them are this library's own.  The style
    limit and PassDirection's values are the reference's."""
    R = ref()
    name, off, size = ctypes.c_char_p(), ctypes.c_long(), ctypes.c_long()
    n = R.ref_param_field(0, ctypes.byref(name), ctypes.byref(off), ctypes.byref(size))
    ref_fields = []
    for k in range(n):
        R.ref_param_field(k, ctypes.byref(name), ctypes.byref(off), ctypes.byref(size))
        ref_fields.append((name.value.decode(), off.value, size.value))
    ours = [(f[0], ctypes.sizeof(f[1])) for f in _abi.Params._fields_]
    assert [f[0] for f in ref_fields] == [f[0] for f in ours[:n]]
    offsets = [f[1] for f in ref_fields]
    assert offsets == sorted(offsets) and len(set(offsets)) == n  # declaration order in the reference
    bools = {"lumShiftEnable", "transparencyOk", "orientationEnabled", "interpolateKeyFrame", "useGuide"}
    for (nm, _, rsize), (_, osize) in zip(ref_fields, ours):
        assert rsize == (1 if nm in bools else osize), (nm, rsize, osize)
    consts = (ctypes.c_long * 5)()
    R.ref_param_constants(consts)
    assert consts[0] == _abi.PT_MAX_STYLES
    assert (consts[2], consts[3], consts[4]) == (0, 1, 2)  # PT_FORWARD, PT_BACKWARD, PT_BIDIRECTIONAL


def test_layer_numbers_are_tsimagelayer_values():
    """Every PT_LAYER_<name> of include/painttween.h has the value of the
    reference's TS_LAYER_<name> (texSynth_interface.h)."""
    import re
    header = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                               "painttween.h")).read()
    ours = {m.group(1): int(m.group(2)) for m in re.finditer(r"PT_LAYER_([A-Z0-9_]+)\s*=\s*(\d+)", header)}
    R = ref()
    name, value = ctypes.c_char_p(), ctypes.c_long()
    n = R.ref_layer(0, ctypes.byref(name), ctypes.byref(value))
    theirs = {}
    for k in range(n):
        R.ref_layer(k, ctypes.byref(name), ctypes.byref(value))
        theirs[name.value.decode()] = value.value
    assert set(ours) == set(theirs)
    assert ours == theirs


def test_sync_advect_merge_flags_are_the_references():
    """PT_DONT_COPY_OFFSETS ... PT_ADVECT_UPDATE_RESIDUAL have the values of
    TexSynth's flags (texSynth_kernel.h), so callers pass the same constants."""
    import re
    header = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                               "painttween.h")).read()
    ours = {m.group(1): int(m.group(2), 16) for m in re.finditer(r"PT_([A-Z_]+)\s*=\s*(0x[0-9a-fA-F]+)", header)}
    names = ["DONT_COPY_OFFSETS", "DONT_UPDATE_RESIDUAL", "MERGE_FALLBACK_RANDOM", "MERGE_FALLBACK_LAST_PASS",
             "ADVECT_IGNORE_RANDOM", "ADVECT_DO_NOT_CHECK_PREVIOUS", "ADVECT_CHECK_FRAME_TO_KEY",
             "ADVECT_UPDATE_RESIDUAL"]
    vals = (ctypes.c_long * 8)()
    ref().ref_flags(vals)
    assert {n: ours[n] for n in names} == dict(zip(names, vals))


def test_patchxf_and_ribbon_records_have_the_references_layout():
    """pt_patchxf is PatchXF byte for byte (36 bytes, same field offsets) and
    pt_ribbon is RibbonP (types.h), so the reference's QVector<PatchXF> and
    QVector<RibbonP> buffers pass through the C ABI as they are."""
    v = (ctypes.c_long * 15)()
    ref().ref_record_layouts(v)
    pf = _abi.PATCH_DTYPE.fields
    assert v[0] == _abi.PATCH_DTYPE.itemsize == 36
    names = ["x", "y", "theta", "hysteresis", "layer", "scaleU", "scaleV", "lumShiftY", "lumShiftA"]
    assert [v[1 + k] for k in range(9)] == [pf[n][1] for n in names]
    rf = _abi.RIBBON_DTYPE.fields
    assert v[10] == _abi.RIBBON_DTYPE.itemsize == 16
    assert [v[11 + k] for k in range(4)] == [rf[n][1] for n in ("x", "y", "time_step", "layer")]


def test_gaussian_weights_bit_exact_with_reference_allocate_gaussian_kernel(gpu_lib):
    """allocateGaussianKernel (convolution.cu:37-60), compiled from the
    reference's own source for the host, against the oracle's weights and the
    library's (pt_gaussian_kernel), unnormalised (the patch window) and
    normalised (the histogram smoothing), for every radius the library
    takes."""
    path = ob.build_ref_gauss()
    assert path is not None
    R = ctypes.CDLL(path)
    R.ref_gaussian_kernel.restype = ctypes.c_int
    R.ref_gaussian_kernel.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    L = O.lib()
    L.pto_gauss_weights.restype = None
    L.pto_gauss_weights.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    for r in range(1, 16):
        for norm in (0, 1):
            ref = np.zeros(64, np.float32)
            n = R.ref_gaussian_kernel(r, norm, _p(ref))
            assert n == 2 * r + 1
            orc = np.zeros(2 * r + 1, np.float32)
            L.pto_gauss_weights(r, norm, _p(orc))
            lib = np.zeros(2 * r + 1, np.float32)
            assert gpu_lib.pt_gaussian_kernel(r, norm, _p(lib)) == 0
            assert np.array_equal(ref[:n].view(np.uint32), orc.view(np.uint32)), (r, norm)
            assert np.array_equal(ref[:n].view(np.uint32), lib.view(np.uint32)), (r, norm)
