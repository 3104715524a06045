"""The oracle's restated helpers against the reference's own device code on the GPU.

oracle/_ref/ref_helpers.cubin is src/PaintTweenCUDA/texSynth_util.h compiled by
nvcc for sm_103a with nvcc's default arithmetic (oracle/ref_helpers_dev.cu,
built by oracle/build.py where the reference tree is present; the cubin itself
needs only the driver).  It is loaded here through the driver API and run on
seeded inputs; the oracle's restatements are checked against its outputs:

  squared differences (sumSquaredDiff, with and without the alpha weight):
      nvcc fuses the first product of the sum with the second, the oracle's
      specification the running sum with each next product: identical on
      most inputs, within 2 ulp on all;
  exemplar coordinates (calculateNewExemplarCoord on the reference's basis):
      the oracle fuses the first product, which is what nvcc does in most
      contexts, but nvcc's choice depends on the surrounding code: identical
      on most inputs, within 2 ulp of the largest term on all;
  exemplar clamping and ribbon unpacking: bit for bit;
  exemplar basis (screenToExemplarBasis: CUDA's cos/sin against the shared
      sincos polynomial): within 2 ulp;
  RGBtoLAB (CUDA's pow and fused double sums against the shared double pow,
      unfused): within 1e-6 of the colour's largest channel.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import build as ob
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = 1 << 14


def _check(res, what):
    if res != 0:
        raise RuntimeError("%s failed with CUresult %d" % (what, res))


def run_reference_cubin(inp):
    """Run ref_helpers_batch over the arrays in `inp`; returns its outputs."""
    import torch

    if not os.path.exists(ob.REF_CUBIN):
        pytest.skip("oracle/_ref/ref_helpers.cubin absent (built only where the reference tree is present)")
    torch.cuda.init()
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in inp.items()}
    n = inp["alpha"].shape[0]
    out = {
        "ssd_alpha": torch.empty(n, dtype=torch.float32, device=dev),
        "ssd_plain": torch.empty(n, dtype=torch.float32, device=dev),
        "basis": torch.empty((n, 4), dtype=torch.float32, device=dev),
        "coord": torch.empty((n, 2), dtype=torch.float32, device=dev),
        "lab": torch.empty((n, 4), dtype=torch.float32, device=dev),
        "clamped": torch.empty((n, 2), dtype=torch.float32, device=dev),
        "ribbon": torch.empty((n, 4), dtype=torch.float32, device=dev),
    }
    torch.cuda.synchronize()
    cu = ctypes.CDLL("libcuda.so.1")
    with open(ob.REF_CUBIN, "rb") as fh:
        image = ctypes.create_string_buffer(fh.read())
    mod, fn = ctypes.c_void_p(), ctypes.c_void_p()
    _check(cu.cuModuleLoadData(ctypes.byref(mod), image), "cuModuleLoadData")
    try:
        _check(cu.cuModuleGetFunction(ctypes.byref(fn), mod, b"ref_helpers_batch"), "cuModuleGetFunction")
        order = ["a", "b", "alpha", "angle", "su", "sv", "ij", "e", "ssd_alpha", "ssd_plain", "basis",
                 "coord", "lab", "clamped", "packed", "ribbon"]
        vals = [ctypes.c_void_p((t[k] if k in t else out[k]).data_ptr()) for k in order]
        vals.append(ctypes.c_int(n))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.addressof(v) for v in vals])
        block = 128
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _check(cu.cuLaunchKernel(fn, ctypes.c_uint((n + block - 1) // block), ctypes.c_uint(1), ctypes.c_uint(1),
                                 ctypes.c_uint(block), ctypes.c_uint(1), ctypes.c_uint(1), ctypes.c_uint(0),
                                 stream, params, None), "cuLaunchKernel")
        torch.cuda.synchronize()
    finally:
        cu.cuModuleUnload(mod)
    return {k: v.cpu().numpy() for k, v in out.items()}


def make_inputs(n=N, seed=21):
    rng = np.random.default_rng(seed)
    scale = rng.choice(np.float32([1, 100]), n)[:, None]
    packed = ((rng.random((n, 4)) * 200) - 50).astype(np.float32)
    packed[:4] = [[1, 2.5, 3.5, 0], [-1, 0, 0, -1], [-1.5, 7.25, -3.0, 2.9], [4.99, 0.5, 0.5, -0.5]]
    return {
        "a": (rng.random((n, 4), dtype=np.float32) * scale).astype(np.float32),
        "b": rng.random((n, 4), dtype=np.float32),
        "alpha": (rng.random(n) * 4).astype(np.float32),
        "angle": (rng.random(n) * 2 * np.pi - np.pi).astype(np.float32),
        "su": (rng.random(n) * 2 + 0.25).astype(np.float32),
        "sv": (rng.random(n) * 2 + 0.25).astype(np.float32),
        "ij": rng.integers(-8, 9, (n, 2)).astype(np.float32),
        "e": (rng.random((n, 2)) * 512).astype(np.float32),
        "packed": packed,
    }


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def oracle_outputs(inp, ref_basis):
    """The oracle's helpers on the same inputs (coordinates on the
    reference's own basis, so that they test the coordinate arithmetic)."""
    L = O.lib()
    n = inp["alpha"].shape[0]
    o = {k: np.empty_like(v) for k, v in (("ssd_alpha", inp["alpha"]), ("ssd_plain", inp["alpha"]),
                                           ("basis", inp["a"]), ("coord", inp["e"]), ("lab", inp["a"]),
                                           ("clamped", inp["e"]), ("ribbon", inp["packed"]))}
    xy, tl = np.empty(2, np.float32), np.empty(2, np.int32)
    for i in range(n):
        a, b = inp["a"][i], inp["b"][i]
        o["ssd_alpha"][i] = L.pto_ssd(_p(a), _p(b), inp["alpha"][i])
        o["ssd_plain"][i] = L.pto_ssd_plain(_p(a), _p(b))
        bs = np.empty(4, np.float32)
        L.pto_basis(inp["angle"][i], inp["su"][i], inp["sv"][i], _p(bs))
        o["basis"][i] = bs
        rb = np.ascontiguousarray(ref_basis[i])
        c = np.empty(2, np.float32)
        L.pto_new_coord(inp["ij"][i, 0], inp["ij"][i, 1], inp["e"][i, 0], inp["e"][i, 1], _p(rb), _p(c))
        o["coord"][i] = c
        o["lab"][i] = O.rgb_to_lab(a)
        cx = ctypes.c_float(np.float32(inp["e"][i, 0] - np.float32(40)))
        cy = ctypes.c_float(np.float32(inp["e"][i, 1] - np.float32(40)))
        L.pto_clamp_to_exemplar(ctypes.byref(cx), ctypes.byref(cy), 64, 48)
        o["clamped"][i] = (cx.value, cy.value)
        L.pto_ribbon_of(_p(np.ascontiguousarray(inp["packed"][i])), _p(xy), _p(tl))
        o["ribbon"][i] = (xy[0], xy[1], tl[0], tl[1])
    return o


@pytest.fixture(scope="module")
def both():
    inp = make_inputs()
    r = run_reference_cubin(inp)
    return inp, r, oracle_outputs(inp, r["basis"])


def test_squared_differences(both):
    _, r, o = both
    for k in ("ssd_alpha", "ssd_plain"):
        d = _ulp_diff(r[k], o[k])
        assert d.max() <= 2, (k, int(d.max()))
        assert (d == 0).mean() >= 0.8, (k, float((d == 0).mean()))


def test_exemplar_coordinates(both):
    inp, r, o = both
    b = r["basis"]
    big = np.stack([np.maximum(np.abs(inp["e"][:, 0]), np.maximum(np.abs(inp["ij"][:, 0] * b[:, 0]),
                                                                   np.abs(inp["ij"][:, 1] * b[:, 2]))),
                    np.maximum(np.abs(inp["e"][:, 1]), np.maximum(np.abs(inp["ij"][:, 0] * b[:, 1]),
                                                                   np.abs(inp["ij"][:, 1] * b[:, 3])))], 1)
    assert (np.abs(r["coord"] - o["coord"]) <= 2 * np.spacing(big.astype(np.float32))).all()
    assert (r["coord"] == o["coord"]).mean() >= 0.9, float((r["coord"] == o["coord"]).mean())


def test_clamp_and_ribbon_bit_exact(both):
    _, r, o = both
    assert r["clamped"].tobytes() == o["clamped"].tobytes()
    assert r["ribbon"].tobytes() == o["ribbon"].tobytes()


def test_exemplar_basis_within_2ulp(both):
    inp, r, o = both
    small = np.abs(r["basis"]) < 1e-3
    d = _ulp_diff(r["basis"], o["basis"])
    assert d[~small].max() <= 2, int(d[~small].max())
    scale = np.maximum(inp["su"], inp["sv"])[:, None] * np.ones((1, 4), np.float32)
    assert (np.abs(r["basis"] - o["basis"])[small] <= 2.5e-7 * scale[small]).all()


def test_rgb_to_lab_within_1e6_of_scale(both):
    _, r, o = both
    # the a and b channels are differences of cube roots: the bound is
    # relative to the colour's largest channel, not to each result
    scale = np.maximum(1.0, np.abs(r["lab"]).max(1, keepdims=True))
    rel = np.abs(r["lab"] - o["lab"]) / scale
    assert rel.max() <= 1e-6, float(rel.max())
