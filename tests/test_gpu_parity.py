"""Parity of the CUDA kernels (through the C ABI) with the CPU oracle.

Integer and index work (random levels, offsets' layers, the pyramid
indexing) and, by the shared FP32 arithmetic contract, the floating-point
offsets, residuals and outputs are compared bit for bit.  The energy is also
checked against the FP64 oracle within 1e-5 relative.  Tests run with the
default sampling (the texture unit's bilinear filtering, which the tiled
kernels take from the texture unit itself and the oracle emulates); those
parametrised by `fm` also run with exact FP32 bilinear filtering.
"""
import numpy as np
import pytest

from painttween_gb300 import Synthesizer, _abi, synthetic
from oracle import oracle as O

from _harness import FILTER_MODES, Pair, assert_array_equal, assert_offsets_equal, config_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def _still_steps(pair, level, frame=0):
    pair.load_style(level)
    pair.load_frame(frame, level)
    pair.random_level(frame, level)


def test_random_level_and_randomize_bit_exact():
    pair = Pair(64, 48, 64, 64, config_params())
    try:
        for level in (2, 1, 0):
            _still_steps(pair, level, 0)
            pair.both("randomize_offsets", level)
            pair.compare(level, "randomize L%d" % level)
    finally:
        pair.close()


@pytest.mark.parametrize("fm", FILTER_MODES)
@pytest.mark.parametrize("jump", [1, 2, 8, 128])
def test_propagate_bit_exact(jump, fm):
    pair = Pair(64, 64, 64, 64, config_params(filter_mode=fm))
    try:
        _still_steps(pair, 1)
        pair.both("randomize_offsets", 1)
        for _ in range(2):
            pair.both("propagate", 1, jump)
            pair.compare(1, "propagate jump %d" % jump)
    finally:
        pair.close()


@pytest.mark.parametrize("fm", FILTER_MODES)
def test_scatter_bit_exact(fm):
    pair = Pair(64, 64, 64, 64, config_params(filter_mode=fm))
    try:
        _still_steps(pair, 0)
        pair.both("randomize_offsets", 0)
        pair.both("propagate", 0, 4)
        pair.both("scatter", 0)
        pair.compare(0, "scatter")
        pair.both("scatter", 0)
        pair.compare(0, "scatter 2")
    finally:
        pair.close()


def test_upsample_bit_exact_odd_sizes():
    # odd sizes: the upsample reads one coarse row/column past the coarse
    # rectangle (texSynth_kernel.cu:1468-1474)
    pair = Pair(67, 45, 64, 64, config_params())
    try:
        _still_steps(pair, 1)
        pair.both("randomize_offsets", 1)
        pair.both("propagate", 1, 2)
        _still_steps(pair, 0)
        pair.both("upsample", 0)
        pair.compare(0, "upsample", residual=True, output=False)
        pair.both("sync", 0, 0)
        pair.compare(0, "upsample+sync")
    finally:
        pair.close()


@pytest.mark.parametrize("fm", FILTER_MODES)
@pytest.mark.parametrize("forwards", [True, False])
def test_advect_and_merge_bit_exact(forwards, fm):
    p = config_params(filter_mode=fm)
    pair = Pair(64, 64, 64, 64, p, frames=3)
    try:
        level = 0
        pair.load_style(level)
        pair.both("reset_advected")
        f0, f1 = (0, 1) if forwards else (2, 1)
        pair.load_frame(f0, level)
        pair.random_level(f0, level)
        pair.both("randomize_offsets", level)
        pair.both("propagate", level, 2)
        pair.flip()
        pair.load_frame(f1, level)
        pair.random_level(f1, level)
        pair.both("advect", level, 1, forwards, 0)
        pair.compare(level, "advect")
        pair.both("merge_randomly", level, forwards, 0.5, False)
        pair.compare(level, "merge randomly")
        pair.both("advect", level, 1, forwards, _abi.ADVECT_UPDATE_RESIDUAL)
        pair.both("merge_using_residual", level, forwards)
        pair.compare(level, "merge using residual")
        # temporal terms active now (advected hysteresis > 0)
        q = p.copy()
        q.direction = _abi.FORWARD if forwards else _abi.BACKWARD
        q.hysteresisWeight = 0.5
        pair.set_params(q)
        pair.both("propagate", level, 1)
        pair.compare(level, "propagate with temporal terms")
        pair.both("scatter", level)
        pair.compare(level, "scatter with temporal terms")
    finally:
        pair.close()


def test_all_energy_terms_bit_exact():
    p = config_params(r=3)
    p.distTransWeight = 1.0
    p.styleObjIdWeight = 1.0
    p.coherenceWeight = 0.5
    p.offsetsHistogramSlope[0] = 1.0
    p.offsetsHistogramThreshold[0] = -0.25  # makes the (always-empty) histogram term non-zero
    ex = synthetic.make_exemplar(64, 64, seed=5)
    ex["dist_trans"] = np.random.default_rng(3).uniform(0, 80, (64, 64)).astype(np.float32)
    pair = Pair(64, 64, 64, 64, p, style=ex)
    try:
        _still_steps(pair, 0)
        pair.both("randomize_offsets", 0)
        pair.compare(0, "randomize (all terms)")
        pair.both("propagate", 0, 4)
        pair.compare(0, "propagate (all terms)")
        pair.both("scatter", 0)
        pair.compare(0, "scatter (all terms)")
    finally:
        pair.close()


def test_transparent_exemplar_serial_random_level():
    # transparent exemplar texels force the reference's retry loop; the GPU
    # then draws the glibc sequence serially
    ex = synthetic.make_exemplar(64, 64, seed=9)
    ex["output"][:, :20, 3] = 0.2
    ex["base"][:, :20, 3] = 0.2
    pair = Pair(48, 48, 64, 64, config_params(), style=ex)
    try:
        for level in (1, 0):
            _still_steps(pair, level)
            pair.both("randomize_offsets", level)
            pair.compare(level, "randomize transparent L%d" % level)
    finally:
        pair.close()


def test_load_offsets_residual_half_roundtrip():
    pair = Pair(32, 32, 32, 32, config_params())
    try:
        _still_steps(pair, 0)
        pair.both("randomize_offsets", 0)
        offs = pair.o.get_offsets(0)
        offs["lumShiftA"] = 0.125
        offs["lumShiftY"] = -0.25
        res = np.random.default_rng(0).uniform(0, 70000, (32, 32)).astype(np.float32)
        for side in (pair.o, pair.g):
            side.load_offsets(0, offs)
            side.load_residual(0, res)
        assert_array_equal(pair.g.get_residual(0), pair.o.get_residual(0), "half residual")
        with np.errstate(over="ignore"):
            half = res.astype(np.float16).astype(np.float32)
        assert_array_equal(pair.g.get_residual(0), half, "half vs numpy")
        pair.both("sync", 0, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
        pair.compare(0, "loaded offsets")
    finally:
        pair.close()


def test_energy_matches_fp64_oracle():
    """Per-pixel patch distance of the CUDA residual vs the FP64 oracle."""
    pair = Pair(64, 64, 64, 64, config_params(r=3))
    try:
        _still_steps(pair, 0)
        pair.both("randomize_offsets", 0)
        pair.both("propagate", 0, 8)
        offs = pair.g.get_offsets(0)
        g = pair.g.get_residual(0).astype(np.float64)
        _, e64 = pair.o.energy_map(0, offs, f32=False, f64=True)
        mask = e64 > 0
        rel = np.abs(g[mask] - e64[mask]) / np.maximum(np.abs(e64[mask]), 1e-3)
        assert rel.max() <= 1e-5, rel.max()
    finally:
        pair.close()


def _driver_pair(W, H, EW, EH, p, frames, seed):
    ex = synthetic.make_exemplar(EW, EH, seed=seed)
    clip = synthetic.make_clip(W, H, 3, frames, seed=seed + 1)
    s = Synthesizer(device=0)
    s.setup(p, W, H, EW, EH, 1)
    s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
    for i, fr in enumerate(clip):
        s.set_frame_dict(i, fr)
    d = O.OracleDriver(p, [ex], clip, threads=8)
    return s, d


@pytest.mark.parametrize("fm", FILTER_MODES)
def test_still_synthesis_driver_bit_exact(fm):
    p = config_params(r=2, levels=3, iterations=3, filter_mode=fm)
    s, d = _driver_pair(96, 80, 64, 64, p, 1, seed=21)
    try:
        rgba, offs = s.synthesize_frame(0)
        ref = d.render(0, 0)[0]
        assert_offsets_equal(offs, ref[0], 1.0, "still offsets")
        assert np.abs(rgba - ref[2]).max() <= 1e-6
        psnr = 10 * np.log10(1.0 / max(np.mean((rgba - ref[2]) ** 2), 1e-20))
        assert psnr >= 40
    finally:
        s.close()


@pytest.mark.parametrize("fm", FILTER_MODES)
def test_animation_driver_bit_exact(fm):
    p = config_params(r=2, levels=3, iterations=2, filter_mode=fm)
    p.temporalCoherenceWeight = 0.5
    s, d = _driver_pair(64, 64, 64, 64, p, 4, seed=31)
    try:
        got = s.synthesize_animation(0, 3)
        ref = d.render(0, 3)
        for f in range(4):
            assert_offsets_equal(got[f][1], ref[f][0], 1.0, "frame %d offsets" % f)
            assert np.abs(got[f][0] - ref[f][2]).max() <= 1e-6
    finally:
        s.close()


def test_animation_scheme_fmbm_residual_merge():
    p = config_params(r=2, levels=2, iterations=2)
    p.scheme = _abi.S_FMBM
    s, d = _driver_pair(48, 48, 64, 64, p, 3, seed=41)
    try:
        got = s.synthesize_animation(0, 2)
        ref = d.render(0, 2)
        for f in range(3):
            assert_offsets_equal(got[f][1], ref[f][0], 1.0, "FMBM frame %d" % f)
    finally:
        s.close()


def test_still_config_256_full_size():
    """The 256x256 still configuration at full size (r2, 3 levels, 4
    iterations) against the oracle."""
    cfg = synthetic.config("still256")
    p = cfg["params"]
    s, d = _driver_pair(cfg["w"], cfg["h"], cfg["ew"], cfg["eh"], p, 1, seed=7)
    try:
        rgba, offs = s.synthesize_frame(0)
        ref = d.render(0, 0)[0]
        assert_offsets_equal(offs, ref[0], 1.0, "still256 offsets")
        psnr = 10 * np.log10(1.0 / max(np.mean((rgba - ref[2]) ** 2), 1e-20))
        assert psnr >= 40
    finally:
        s.close()


def test_determinism_and_residual_consistency_large():
    """Size-independent properties on a larger frame: two runs are identical,
    offsets stay inside the exemplar, and the stored residual equals a fresh
    recomputation."""
    p = config_params(r=3, levels=4, iterations=2)
    ex = synthetic.make_exemplar(256, 256, seed=3)
    fr = synthetic.make_still(640, 360, 6, seed=4)
    outs = []
    for _ in range(2):
        s = Synthesizer(device=0)
        s.setup(p, 640, 360, 256, 256, 1)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        s.set_frame_dict(0, fr)
        outs.append(s.synthesize_frame(0))
        res_before = s.get_residual(0)
        s.update_residual_cache(0)
        assert_array_equal(s.get_residual(0), res_before, "residual recomputation")
        s.close()
    assert_offsets_equal(outs[0][1], outs[1][1], 1.0, "repeat run")
    o = outs[0][1]
    assert np.isfinite(o["x"]).all() and np.isfinite(o["y"]).all()
    # offsetUpsampleNearest clamps in coarse coordinates to the fine exemplar
    # size before doubling (texSynth_kernel.cu:1411-1414), so coordinates can
    # reach 2 * (w - 1) + 0.5
    assert (o["x"] >= 0).all() and (o["x"] <= 2 * 255 + 0.5).all()
    assert (o["y"] >= 0).all() and (o["y"] <= 2 * 255 + 0.5).all()


def test_counter_rng_mode_matches_oracle():
    """Opt-in counter-based RNG (hashed random levels and a real random
    search): GPU and oracle agree bit for bit."""
    p = config_params(r=2, levels=3, iterations=3)
    p.rngMode = _abi.RNG_COUNTER
    p.rngSeed = 77
    s, d = _driver_pair(64, 64, 64, 64, p, 2, seed=81)
    try:
        got = s.synthesize_animation(0, 1)
        ref = d.render(0, 1)
        for f in range(2):
            assert_offsets_equal(got[f][1], ref[f][0], 1.0, "counter mode frame %d" % f)
    finally:
        s.close()


def test_counter_rng_mode_runs_and_is_deterministic():
    p = config_params(r=2, levels=3, iterations=2)
    p.rngMode = _abi.RNG_COUNTER
    p.rngSeed = 1234
    ex = synthetic.make_exemplar(64, 64, seed=2)
    fr = synthetic.make_still(64, 64, 3, seed=3)
    res = []
    for _ in range(2):
        s = Synthesizer(device=0)
        s.setup(p, 64, 64, 64, 64, 1)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        s.set_frame_dict(0, fr)
        res.append(s.synthesize_frame(0)[1])
        s.close()
    assert_offsets_equal(res[0], res[1], 1.0, "counter mode repeat")


def test_errors_are_status_codes():
    from painttween_gb300 import PaintTweenError, TexSynth
    t = TexSynth(device=0)
    with pytest.raises(PaintTweenError):
        t.propagate(0, 1)  # before initialize
    for sizes in ((0, 32, 32, 32, 1), (32, 1, 32, 32, 1), (32, 32, 32, 32, 0), (70000, 70000, 32, 32, 1),
                  (32, 32, 40000, 40000, 2)):
        with pytest.raises(PaintTweenError) as e:
            t.initialize(*sizes)  # empty, degenerate and oversized images are refused before any allocation
        assert e.value.status == 1, sizes  # PT_ERR_INVALID
    t.initialize(32, 32, 32, 32, 1)
    with pytest.raises(PaintTweenError):
        t.upload_image_color4(0, _abi.LAYER_INPUT_COLOR, np.zeros((10, 10, 4), np.float32))
    p = config_params()
    p.colorspace = 2  # neither RGB nor Lab
    with pytest.raises(PaintTweenError):
        t.set_params(p)
    t.close()
    tb = TexSynth(device=0, hbm_budget=1 << 20)
    with pytest.raises(PaintTweenError) as e:
        tb.initialize(1024, 1024, 256, 256, 1)
    assert e.value.status == 7  # PT_ERR_BUDGET
    tb.close()


@pytest.mark.parametrize("fm", FILTER_MODES)
@pytest.mark.parametrize("r", [1, 2, 3, 4])
def test_tiled_and_generic_kernels_identical(r, fm):
    """The tiled shared-memory kernels (patch radius 2-4) and the generic
    kernels give bit-identical animations, including the temporal terms of
    both pass directions; radius 1 runs the generic kernels in both cases.
    With the texture unit's filtering the tiled kernels fetch through the
    texture unit and the generic kernels emulate it."""
    p = config_params(r=r, levels=2, iterations=2, filter_mode=fm)
    p.temporalCoherenceWeight = 0.5
    p.hysteresisWeight = 0.25
    p.distTransWeight = 0.5
    ex = synthetic.make_exemplar(64, 64, seed=50 + r)
    clip = synthetic.make_clip(72, 56, 3, 3, seed=60 + r)
    outs = []
    for tiled in (True, False):
        s = Synthesizer(device=0)
        s.setup(p, 72, 56, 64, 64, 1)
        s.set_tiled_kernels(tiled)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        outs.append(s.synthesize_animation(0, 2))
        s.close()
    for f in range(3):
        assert_offsets_equal(outs[0][f][1], outs[1][f][1], 1.0, "tiled vs generic frame %d" % f)
        assert_array_equal(outs[0][f][0], outs[1][f][0], "tiled vs generic output frame %d" % f)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 2)
    for f in range(3):
        assert_offsets_equal(outs[0][f][1], ref[f][0], 1.0, "tiled vs oracle frame %d" % f)


@pytest.mark.parametrize("fm", FILTER_MODES)
@pytest.mark.parametrize("r", [2, 3, 4])
def test_tensor_copy_staging_identical_to_plain_loads(r, fm):
    """Tiles whose halo lies inside the level rectangle are staged by tensor
    copies (pt_set_tma_staging, the default); plain loads everywhere give
    the same bits, for every radius, temporal direction and filter mode.
    Some input colours are subnormal: the texture mode flushes them to zero
    in shared memory after the copies, as the loads do."""
    p = config_params(r=r, levels=2, iterations=2, filter_mode=fm)
    p.temporalCoherenceWeight = 0.5
    p.hysteresisWeight = 0.25
    p.distTransWeight = 0.5
    W, H = 200, 120  # level 0 and 1 both have interior tiles
    ex = synthetic.make_exemplar(96, 96, seed=70 + r)
    clip = synthetic.make_clip(W, H, 3, 3, seed=80 + r)
    for fr in clip:
        fr["rgba"][30:50, 60:120, 0] = np.float32(1e-40)
    outs = []
    for tma in (True, False):
        s = Synthesizer(device=0)
        s.setup(p, W, H, 96, 96, 1)
        s.set_tma_staging(tma)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        outs.append(s.synthesize_animation(0, 2))
        s.close()
    for f in range(3):
        assert_offsets_equal(outs[0][f][1], outs[1][f][1], 1.0, "tensor copies vs loads frame %d" % f)
        assert_array_equal(outs[0][f][0], outs[1][f][0], "tensor copies vs loads output frame %d" % f)


@pytest.mark.parametrize("fm", FILTER_MODES)
@pytest.mark.parametrize("r", [2, 3, 4])
def test_propagate_warps_per_row_identical(r, fm):
    """Propagate with one warp per tile row, with two (the second only
    evaluating queued candidates), and with the autotuner's choice per
    launch shape give the same bits, and equal the oracle."""
    p = config_params(r=r, levels=3, iterations=2, filter_mode=fm)
    p.temporalCoherenceWeight = 0.5
    p.hysteresisWeight = 0.25
    W, H = 160, 96
    ex = synthetic.make_exemplar(80, 80, seed=90 + r)
    clip = synthetic.make_clip(W, H, 3, 3, seed=95 + r)
    outs = []
    for lanes in (1, 2, 0):
        s = Synthesizer(device=0)
        s.setup(p, W, H, 80, 80, 1)
        s.set_propagate_lanes(lanes)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        outs.append(s.synthesize_animation(0, 2))
        s.close()
    for o, name in ((outs[1], "two warps"), (outs[2], "autotuned")):
        for f in range(3):
            assert_offsets_equal(o[f][1], outs[0][f][1], 1.0, "%s vs one warp, frame %d" % (name, f))
            assert_array_equal(o[f][0], outs[0][f][0], "%s vs one warp output, frame %d" % (name, f))
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 2)
    for f in range(3):
        assert_offsets_equal(outs[1][f][1], ref[f][0], 1.0, "two warps vs oracle frame %d" % f)


@pytest.mark.parametrize("radius", [1, 3, 7])
def test_convolve_separable_matches_oracle(radius):
    """Separable Gaussian (convolutionRowsGPU + convolutionColumnsGPU) on a
    device image, against the oracle bit for bit."""
    torch = pytest.importorskip("torch")
    from painttween_gb300 import TexSynth
    rng = np.random.default_rng(radius)
    img = rng.uniform(0, 5, (70, 93)).astype(np.float32)
    ref = O.convolve_separable(img, radius)
    src = torch.from_numpy(img).cuda()
    dst = torch.zeros_like(src)
    t = TexSynth(device=0)
    t.convolve_separable(src.data_ptr(), dst.data_ptr(), 93, 70, 93, radius)
    t.synchronize()
    t.close()
    assert_array_equal(dst.cpu().numpy(), ref, "separable Gaussian r=%d" % radius)


def _animate(p, ex, clip, W, H, incremental=True, tiled=True):
    s = Synthesizer(device=0)
    try:
        s.setup(p, W, H, ex["w"], ex["h"], 1)
        s.set_tiled_kernels(tiled)
        s.set_incremental(incremental)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        return s.synthesize_animation(0, len(clip) - 1)
    finally:
        s.close()


@pytest.mark.parametrize("r", [2, 3, 4])
def test_change_tracking_identical_and_matches_oracle(r):
    """The propagate/scatter loop with change tracking (skipped candidates,
    incremental canvas and residual) gives the same bytes as the loop that
    evaluates everything, and as the oracle, over an animation with temporal,
    hysteresis and distance-transform terms in both pass directions."""
    p = config_params(r=r, levels=3, iterations=3)
    p.temporalCoherenceWeight = 0.5
    p.hysteresisWeight = 0.25
    p.distTransWeight = 0.5
    ex = synthetic.make_exemplar(64, 64, seed=70 + r)
    clip = synthetic.make_clip(96, 72, 3, 3, seed=80 + r)
    on = _animate(p, ex, clip, 96, 72, incremental=True)
    off = _animate(p, ex, clip, 96, 72, incremental=False)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 2)
    for f in range(3):
        assert_offsets_equal(on[f][1], off[f][1], 1.0, "tracked vs full frame %d" % f)
        assert_array_equal(on[f][0], off[f][0], "tracked vs full output frame %d" % f)
        assert_offsets_equal(on[f][1], ref[f][0], 1.0, "tracked vs oracle frame %d" % f)
        assert_array_equal(on[f][0], ref[f][2], "tracked vs oracle output frame %d" % f)


def test_change_tracking_identical_large_still():
    """A 640x360 still at patch radius 3: the tracked loop and the full loop
    agree on every byte of the offsets and the output."""
    p = config_params(r=3, levels=4, iterations=4)
    ex = synthetic.make_exemplar(256, 256, seed=5)
    fr = synthetic.make_still(640, 360, 6, seed=6)
    on = _animate(p, ex, [fr], 640, 360, incremental=True)
    off = _animate(p, ex, [fr], 640, 360, incremental=False)
    assert_offsets_equal(on[0][1], off[0][1], 1.0, "tracked vs full offsets")
    assert_array_equal(on[0][0], off[0][0], "tracked vs full output")


def test_negative_weight_disables_early_exit():
    """A negative term weight makes partial patch sums non-monotone, so the
    early exit must stay off; the result still matches the oracle."""
    p = config_params(r=3, levels=2, iterations=2)
    p.canvasOutputWeight = -0.25
    ex = synthetic.make_exemplar(64, 64, seed=90)
    clip = synthetic.make_clip(80, 64, 3, 2, seed=91)
    got = _animate(p, ex, clip, 80, 64)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 1)
    for f in range(2):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "negative weight frame %d" % f)


def test_frame_results_into_page_locked_memory():
    """pt_get_frame_result into page-locked arrays (pt_host_alloc) returns
    the same bytes as the animation callback; inputs may live in page-locked
    memory too."""
    from painttween_gb300 import host_array
    p = config_params(r=3, levels=2, iterations=2)
    ex = synthetic.make_exemplar(64, 64, seed=95)
    clip = synthetic.make_clip(80, 64, 3, 2, seed=96)
    ref = _animate(p, ex, clip, 80, 64)
    s = Synthesizer(device=0)
    try:
        s.setup(p, 80, 64, 64, 64, 1)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            pinned = {}
            for key in ("rgba", "orient_tensor", "dist_trans", "object_ids", "vel_fwd", "vel_bwd", "scale"):
                pinned[key] = host_array(fr[key].shape, fr[key].dtype)
                pinned[key][...] = fr[key]
            s.set_frame_dict(i, pinned)
        lib = __import__("painttween_gb300._lib", fromlist=["lib"]).lib()
        s._check(lib.pt_synthesize_animation(s.h, 0, 1, None, None), "pt_synthesize_animation")
        for f in range(2):
            a = host_array((64, 80, 4), np.float32)
            o = host_array((64, 80), _abi.PATCH_DTYPE)
            s.get_frame_result(f, a, o)
            assert_offsets_equal(o, ref[f][1], 1.0, "pinned offsets frame %d" % f)
            assert_array_equal(a, ref[f][0], "pinned output frame %d" % f)
    finally:
        s.close()


def test_near_ties_match_oracle():
    """An exemplar whose colours differ by ~1e-5 makes many candidates tie or
    nearly tie with the best: scatter's bound pass must leave every such
    candidate to the exact reference-order sum (checked against the oracle
    on every byte)."""
    p = config_params(r=3, levels=2, iterations=3)
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(64, 64, seed=97)
    rng = np.random.default_rng(98)
    for key in ("base", "output"):
        a = ex[key].copy()
        a[..., :3] = 0.5 + 1e-5 * np.round(rng.standard_normal(a[..., :3].shape), 1)
        ex[key] = a.astype(np.float32)
    clip = synthetic.make_clip(80, 64, 3, 2, seed=99)
    got = _animate(p, ex, clip, 80, 64)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 1)
    for f in range(2):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "near ties frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "near ties output frame %d" % f)


def test_ind_scheme_matches_oracle():
    """The IND scheme (every frame on its own) against the oracle.  Coarse
    levels of later frames read texels that earlier frames' finer levels left
    outside the level rectangle (hysteresis velocities at the right and
    bottom edges, propagate's wrap)."""
    p = config_params(r=3, levels=2, iterations=2)
    p.scheme = _abi.S_IND
    p.temporalCoherenceWeight = 0.5
    p.hysteresisWeight = 0.25
    ex = synthetic.make_exemplar(64, 64, seed=63)
    clip = synthetic.make_clip(80, 64, 3, 3, seed=64)
    got = _animate(p, ex, clip, 80, 64)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 2)
    for f in range(3):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "IND frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "IND output frame %d" % f)


@pytest.mark.parametrize("r,fixups", [(2, 1), (3, 2)])
def test_fbmo_scheme_matches_oracle(r, fixups):
    """The FBMO scheme (forward and backward passes, random merge, fix-up
    passes between advected neighbours with both temporal terms) against the
    oracle."""
    p = config_params(r=r, levels=2, iterations=2)
    p.scheme, p.fixupPasses = _abi.S_FBMO, fixups
    p.temporalCoherenceWeight = 0.5
    p.timeDerivativeInputWeight = 0.25
    ex = synthetic.make_exemplar(64, 64, seed=67 + r)
    clip = synthetic.make_clip(80, 64, 3, 4, seed=68 + r)
    got = _animate(p, ex, clip, 80, 64)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 3)
    for f in range(4):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "FBMO frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "FBMO output frame %d" % f)


@pytest.mark.parametrize("frames,levels,final_level", [(3, 2, 0), (4, 3, 1), (2, 2, 0)])
def test_tctf_scheme_matches_oracle(frames, levels, final_level):
    """The TCTF scheme without ribbon inputs (a consecutive pass at the
    coarsest level, refine passes between advected neighbours at every level,
    spatial upsampling below the final level) against the oracle."""
    p = config_params(r=2, levels=levels, iterations=2)
    p.scheme, p.finalLevel = _abi.S_TCTF, final_level
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(64, 64, seed=73 + frames)
    clip = synthetic.make_clip(80, 64, 3, frames, seed=74 + frames)
    got = _animate(p, ex, clip, 80, 64)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, frames - 1)
    for f in range(frames):
        assert got[f][0].shape == (64, 80, 4)
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "TCTF frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "TCTF output frame %d" % f)


def test_final_level_upsampled_to_full_size_matches_oracle():
    """FMBM with a final level above 0: the final level's offsets upsampled
    level by level to the full image (renderSpatialUpsample)."""
    p = config_params(r=2, levels=3, iterations=2)
    p.finalLevel = 1
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(64, 64, seed=79)
    clip = synthetic.make_clip(80, 64, 3, 3, seed=80)
    got = _animate(p, ex, clip, 80, 64)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 2)
    for f in range(3):
        assert got[f][0].shape == (64, 80, 4)
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "output frame %d" % f)


@pytest.mark.parametrize("scheme", [_abi.S_FMBM_RM, _abi.S_FMBM])
def test_lab_colour_space_matches_oracle(scheme):
    """colorspace 1: every colour the energy compares converted by RGBtoLAB
    (texSynth_kernel.cu:454-459,575-578,603-606) with the shared double pow,
    over an animation with temporal terms."""
    p = config_params(r=2, levels=2, iterations=2)
    p.colorspace = 1
    p.scheme = scheme
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(32, 32, seed=91)
    clip = synthetic.make_clip(40, 32, 3, 2, seed=92)
    got = _animate(p, ex, clip, 40, 32)
    ref = O.OracleDriver(p, [ex], clip, threads=8).render(0, 1)
    for f in range(2):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "Lab frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "Lab output frame %d" % f)


@pytest.mark.parametrize("w,h,scheme", [(17, 13, _abi.S_FMBM_RM), (31, 7, _abi.S_FBMO), (23, 19, _abi.S_TCTF),
                                        (9, 9, _abi.S_IND)])
def test_small_odd_sizes_match_oracle(w, h, scheme):
    """Odd, tiny images (a coarse level a few pixels across, narrower than
    the patch window) through each scheme, against the oracle."""
    p = config_params(r=2, levels=2, iterations=2)
    p.scheme = scheme
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(24, 20, seed=95)
    clip = synthetic.make_clip(w, h, 2, 3, seed=96)
    got = _animate(p, ex, clip, w, h)
    ref = O.OracleDriver(p, [ex], clip, threads=4).render(0, 2)
    lv = _abi.output_level(p)
    for f in range(3):
        assert got[f][0].shape == (h >> lv, w >> lv, 4)
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "%dx%d frame %d" % (w, h, f))
        assert_array_equal(got[f][0], ref[f][2], "%dx%d output frame %d" % (w, h, f))
