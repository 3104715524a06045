"""CPU tests of the oracle: pinned pieces (glibc rand, IEEE half), accuracy of
the polynomial elementary functions, pyramid construction, and the
committed golden fixtures."""
import ctypes
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from painttween_gb300 import _abi, synthetic

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_glibc_stream_matches_libc_rand():
    """The restated TYPE_3 generator reproduces the C library's rand()."""
    libc = ctypes.CDLL("libc.so.6")
    for seed in (0, 1, 2, 3, 17, 96, 1 << 20):
        libc.srand(seed)
        ref = np.array([libc.rand() for _ in range(2000)], np.int32)
        assert (O.glibc_stream(seed, 2000) == ref).all(), seed


def test_glibc_stream_matches_committed_vectors():
    g = np.load(os.path.join(GOLDEN, "glibc_rand.npz"))
    for key in g.files:
        seed = int(key.split("_")[1])
        assert (O.glibc_stream(seed, g[key].size) == g[key]).all(), key


def test_half_roundtrip_matches_numpy():
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.normal(0, 1, 20000) * 10.0 ** rng.integers(-9, 6, 20000),
                        [0.0, -0.0, 65504.0, 65519.9, 65520.0, 1e31, 6.1e-5, 5.96e-8, 2.98e-8, 1e-9]]).astype(np.float32)
    lib = O.lib()
    got = np.array([lib.pto_half_roundtrip(float(x)) for x in v], np.float32)
    with np.errstate(over="ignore"):
        ref = v.astype(np.float16).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_polynomial_functions_accuracy():
    lib = O.lib()
    t = np.linspace(-9.0, 9.0, 4001).astype(np.float32)
    s = np.array([lib.pto_sinf(float(x)) for x in t])
    c = np.array([lib.pto_cosf(float(x)) for x in t])
    assert np.abs(s - np.sin(t.astype(np.float64))).max() < 2.5e-7
    assert np.abs(c - np.cos(t.astype(np.float64))).max() < 2.5e-7
    assert lib.pto_sinf(0.0) == 0.0 and lib.pto_cosf(0.0) == 1.0
    rng = np.random.default_rng(1)
    ys, xs = rng.normal(size=2000).astype(np.float32), rng.normal(size=2000).astype(np.float32)
    a = np.array([lib.pto_atan2f(float(y), float(x)) for y, x in zip(ys, xs)])
    assert np.abs(a - np.arctan2(ys.astype(np.float64), xs.astype(np.float64))).max() < 5e-7
    assert lib.pto_atan2f(0.0, 0.0) == 0.0
    xl = np.exp(rng.uniform(-20, 20, 2000)).astype(np.float32)
    lg = np.array([lib.pto_logf(float(x)) for x in xl])
    assert np.abs(lg - np.log(xl.astype(np.float64))).max() < 5e-6
    xc = rng.uniform(-1, 1, 2000).astype(np.float32)
    ac = np.array([lib.pto_acosf(float(x)) for x in xc])
    assert np.abs(ac - np.arccos(xc.astype(np.float64))).max() < 1e-6
    assert math.isnan(lib.pto_acosf(1.5))


def test_pyramids():
    rng = np.random.default_rng(2)
    img = rng.random((37, 50, 4), dtype=np.float32)
    pyr = O.pyramid_avg(img)
    assert len(pyr) == 5 and pyr[1].shape == (18, 25, 4)
    a = img[0:36:2, 0:50:2] + img[0:36:2, 1:50:2]
    b = a + img[1:36:2, 0:50:2]
    ref = ((b + img[1:36:2, 1:50:2]) * np.float32(0.25)).astype(np.float32)
    assert np.array_equal(pyr[1], ref)
    vel = O.pyramid_avg(img[..., :2], vel=True)
    assert np.array_equal(vel[1], ref[..., :2] * np.float32(0.5))
    ids = np.array([[1, 2, 3, 3], [2, 1, 3, 4]], np.int32)
    v = O.pyramid_vote(np.tile(ids, (2, 2)))
    assert v[1][0, 0] == 1 and v[1][0, 1] == 3  # 2-2 tie -> smaller id; 3 wins
    ang = O.tensor_to_angle(np.array([[[1.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.5, 0.5, 0.5]]], np.float32))
    assert np.allclose(ang, [[-np.pi / 2, 0.0, -np.pi / 4]], atol=1e-6)


def test_random_level_uses_rand_sequence():
    """createRandomPyramid draws (x, y, fx, fy) per pixel in scan order."""
    h, w = 3, 5
    img = np.ones((h, w, 4), np.float32)
    orient = np.zeros((h, w), np.float32)
    ex_out = np.ones((16, 16, 4), np.float32)
    ex_or = np.zeros((16, 16), np.float32)
    rnd = O.random_level(7 * 2, 2, 64, 64, img, orient, ex_out, ex_or)
    s = O.glibc_stream(14, 4 * w * h).reshape(h, w, 4)
    assert np.array_equal(rnd[..., 0], (s[..., 0] % 15).astype(np.float32) + s[..., 2].astype(np.float32) / np.float32(2147483647))
    assert np.array_equal(rnd[..., 1], (s[..., 1] % 15).astype(np.float32) + s[..., 3].astype(np.float32) / np.float32(2147483647))


def test_oracle_still_matches_golden_fixture():
    """Regression lock of the oracle on a small still (fixture written by
    tests/golden/make_golden.py)."""
    g = np.load(os.path.join(GOLDEN, "still48.npz"))
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 3, 2
    p.filterMode = _abi.FILTER_EXACT
    ex = synthetic.make_exemplar(48, 48, seed=int(g["ex_seed"]))
    fr = synthetic.make_still(48, 48, 3, seed=int(g["fr_seed"]))
    d = O.OracleDriver(p, [ex], [fr], threads=4)
    offs, res, out = d.render(0, 0)[0]
    assert np.array_equal(offs.view(np.uint8), g["offsets"].view(np.uint8))
    assert np.array_equal(res, g["residual"])
    assert np.array_equal(out, g["output"])


def test_oracle_clip_schemes_match_golden_fixture():
    """Regression lock of the oracle's temporal paths: a 40x32 three-frame
    clip under FMBM_RM, FBMO and TCTF (fixture written by
    tests/golden/make_golden.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(os.path.join(GOLDEN, "clip40.npz"))
    for name, scheme in mg.CLIP_SCHEMES:
        results = mg.render_clip(scheme)
        for f in range(3):
            offs, _, out = results[f]
            assert np.array_equal(offs.view(np.uint8), g["%s_offsets_%d" % (name, f)].view(np.uint8)), (name, f)
            assert np.array_equal(out, g["%s_output_%d" % (name, f)]), (name, f)


def test_oracle_keyframe_path_matches_golden_fixture():
    """Regression lock of the oracle's keyframe path: a 32x24 four-frame clip
    interpolating keys 1 and 3 (fixture written by tests/golden/make_golden.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(os.path.join(GOLDEN, "keys32.npz"))
    results = mg.render_keyed()
    for f in range(4):
        offs, _, out = results[f]
        assert np.array_equal(offs.view(np.uint8), g["offsets_%d" % f].view(np.uint8)), f
        assert np.array_equal(out, g["output_%d" % f]), f


def test_energy_fp32_close_to_fp64():
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 3, 2, 2
    ex = synthetic.make_exemplar(48, 48, seed=4)
    fr = synthetic.make_still(48, 48, 3, seed=5)
    d = O.OracleDriver(p, [ex], [fr], threads=4)
    offs = d.render(0, 0)[0][0]
    e32, e64 = d.o.energy_map(0, offs)
    m = e64 > 0
    rel = np.abs(e32[m] - e64[m]) / np.maximum(e64[m], 1e-3)
    assert rel.max() < 1e-5


def test_oracle_openmp_threads_agree():
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 2, 2
    ex = synthetic.make_exemplar(32, 32, seed=8)
    fr = synthetic.make_still(40, 32, 2, seed=9)
    a = O.OracleDriver(p, [ex], [fr], threads=1).render(0, 0)[0][0]
    b = O.OracleDriver(p, [ex], [fr], threads=4).render(0, 0)[0][0]
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_animation_oracle_runs():
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 2, 1
    ex = synthetic.make_exemplar(32, 32, seed=1)
    clip = synthetic.make_clip(32, 32, 2, 3, seed=2)
    res = O.OracleDriver(p, [ex], clip, threads=4).render(0, 2)
    assert sorted(res) == [0, 1, 2]
    for f in res:
        assert np.isfinite(res[f][2]).all()


def test_ind_scheme_equals_fmbm_on_a_still():
    """For one frame and no fix-up passes renderAnimationIND and
    renderAnimationFMBM run the same steps (one forward pass of a first frame
    per level), so they agree on every byte.  (Across frames IND's frames are not independent: as in the
    reference, propagate's level-0 wrap reads offsets that earlier frames left
    outside a coarse level's rectangle.)"""
    ex = synthetic.make_exemplar(48, 48, seed=61)
    fr = synthetic.make_still(56, 40, 3, seed=62)
    out = []
    for scheme in (_abi.S_IND, _abi.S_FMBM_RM):
        p = _abi.default_params()
        p.residualWindowSize, p.levels, p.iterations = 2, 2, 2
        p.scheme, p.fixupPasses = scheme, 0
        out.append(O.OracleDriver(p, [ex], [fr], threads=4).render(0, 0)[0])
    assert (out[0][0].view(np.uint8) == out[1][0].view(np.uint8)).all()
    assert np.array_equal(out[0][2], out[1][2])


def test_fbmo_merge_pass_takes_each_record_from_a_directional_pass():
    """renderAnimationFBMO's pass 2 merges the forward (pass 0) and backward
    (pass 1) offsets at random: every record of pass 2 is one of the two."""
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 2, 2
    p.scheme, p.fixupPasses = _abi.S_FBMO, 1
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(48, 48, seed=65)
    clip = synthetic.make_clip(56, 40, 3, 3, seed=66)
    drv = O.OracleDriver(p, [ex], clip, threads=4)
    out = drv.render(0, 2)
    assert sorted(out) == [0, 1, 2]
    for f in range(3):
        rec = lambda pass_: drv.store[(0, f, pass_)][0].view(np.uint8).reshape(40, 56, -1)
        fw, bw, mg = rec(0), rec(1), rec(2)
        from_fw = (mg == fw).all(-1)
        from_bw = (mg == bw).all(-1)
        assert (from_fw | from_bw).all()
        assert from_fw.any() and from_bw.any() and not (from_fw & from_bw).all()
        assert drv.last_saved[(f, 0)] == 3  # the fix-up pass, not the merge


@pytest.mark.parametrize("scheme,final_level,full", [(_abi.S_FMBM_RM, 1, True), (_abi.S_TCTF, 1, True),
                                                     (_abi.S_TCTF, 0, True), (_abi.S_IND, 1, False)])
def test_output_level_of_each_scheme(scheme, final_level, full):
    """FMBM and TCTF upsample a final level > 0 down to level 0 (the level
    copyOutputToFinal hands out); IND hands out its final level."""
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 3, 1
    p.scheme, p.finalLevel, p.fixupPasses = scheme, final_level, 1
    ex = synthetic.make_exemplar(48, 48, seed=71)
    clip = synthetic.make_clip(64, 48, 3, 3, seed=72)
    out = O.OracleDriver(p, [ex], clip, threads=4).render(0, 2)
    lv = _abi.output_level(p)
    assert lv == (0 if full else final_level)
    for f in range(3):
        offs, res, rgba = out[f]
        assert offs.shape == (48 >> lv, 64 >> lv) and rgba.shape == (48 >> lv, 64 >> lv, 4)
        assert np.isfinite(rgba).all()


def test_lab_conversion_against_float64_formula():
    """RGBtoLAB (texSynth_util.h:175-246) with the shared double pow, against
    the same formula in numpy float64: within 2e-6 absolute."""
    rng = np.random.default_rng(21)
    for x, y in zip(rng.uniform(1e-3, 4.0, 200), rng.uniform(0.1, 3.0, 200)):
        got = O.lib().pto_powd(float(x), float(y))
        assert abs(got - x ** y) <= 1e-13 * x ** y
    cols = np.concatenate([rng.random((300, 4)), [[0, 0, 0, 1], [1, 1, 1, 0.5], [0.04, 0.5, 0.9, 1]]])
    for c in cols.astype(np.float32):
        lin = np.where(c[:3] > 0.04045, ((c[:3].astype(np.float64) + 0.055) / 1.055) ** 2.4, c[:3] / 12.92) * 100
        X = 0.4124 * lin[0] + 0.3576 * lin[1] + 0.1805 * lin[2]
        Y = 0.2126 * lin[0] + 0.7152 * lin[1] + 0.0722 * lin[2]
        Z = 0.0193 * lin[0] + 0.1192 * lin[1] + 0.9505 * lin[2]
        f = lambda t: t ** (1 / 3) if t > (6 / 29) ** 3 else t / 3 * (29 / 6) ** 2 + 4 / 29
        ref = [(116 * f(Y / 100) - 16) / 100, (500 * (f(X / 95.047) - f(Y / 100)) + 100) / 200,
               (200 * (f(Y / 100) - f(Z / 108.883)) + 100) / 200, c[3]]
        assert np.allclose(O.rgb_to_lab(c), ref, atol=2e-6, rtol=0), c


def test_texture_filter_emulation_matches_recorded_gb300_fetches(oracle_mod):
    """PT_FILTER_TEXTURE: the oracle's restatement of the texture unit's
    bilinear filtering against fetches recorded on a GB300
    (tests/golden/texfilter_gb300.npz, written by make_texfilter.py from
    texfilter_probe.cu): 1-, 2- and 4-channel float textures, layered arrays
    and pitched memory, unit weights, coordinates beyond the edges, fraction
    ties, large coordinates, zeros, signed zeros, subnormals and values over
    twelve decades -- every fetched bit."""
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "texfilter_gb300.npz"))
    cases = sorted({k.split("/")[0] for k in d.files if not k.startswith("meta")})
    assert len(cases) >= 7
    total = 0
    for name in cases:
        tex, q, out = d[name + "/tex"], d[name + "/q"], d[name + "/out"]
        got = oracle_mod.tex_fetch(tex, q, hw=True)
        same = got.view(np.uint32) == out.view(np.uint32)
        assert same.all(), "%s: %d of %d channels differ" % (name, (~same).sum(), same.size)
        total += same.size
        if name != "weights":  # exact FP32 bilinear is a different arithmetic
            assert (oracle_mod.tex_fetch(tex, q, hw=False).view(np.uint32) != out.view(np.uint32)).any()
    assert total > 100000

