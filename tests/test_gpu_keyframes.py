"""Keyframe interpolation kernels against the oracle, bit for bit.

Keys are exemplar layers of the frame's size (the reference loads keyframes
as style layers).  Covered: the key mask of propagate_kernel / scatter_kernel
(key_index >= 0), propagate_kernel_keys / scatter_kernel_keys walking the
key-to-key cumulative fields, accumulateAdvectionKernel with its output
(accumulateRibbonField) and copyFrameToKeyRibbonKernel
(offsetsFromFrameToKeyRibbon), src/PaintTweenCUDA/texSynth_kernel.cu:
290-304,723-1110,1728-1853,2061-2118.
"""
import numpy as np
import pytest

from painttween_gb300 import TexSynth, _abi, synthetic
from oracle import oracle as O

from _harness import assert_array_equal, assert_offsets_equal, config_params

pytestmark = pytest.mark.gpu

W, H = 64, 48
NK = 3  # key layers


@pytest.fixture(scope="module", autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def _keys():
    keys = [synthetic.make_exemplar(W, H, seed=90 + i) for i in range(NK)]
    yy, xx = np.mgrid[0:H, 0:W]
    mask = ((xx - 40) ** 2 + (yy - 20) ** 2) < 12 ** 2
    out = keys[1]["output"].copy()
    out[..., 3] = np.where(mask, 1.0, 0.0)
    keys[1]["output"] = out
    return keys


def _ribbon_image(rng, valid=0.7):
    """A ribbon field as an RGBA image (time_step, y, x, layer)."""
    img = np.zeros((H, W, 4), np.float32)
    img[..., 0] = rng.integers(1, 4, (H, W))
    img[..., 1] = rng.normal(0.0, 2.0, (H, W))
    img[..., 2] = rng.normal(0.0, 2.0, (H, W))
    layer = rng.integers(0, NK, (H, W)).astype(np.float32)
    bad = rng.random((H, W)) > valid
    layer[bad] = -1.0
    img[..., 0][bad] = -1.0
    img[..., 3] = layer
    return img


def _ribbons(rng, valid=0.7):
    r = np.zeros((H, W), _abi.RIBBON_DTYPE)
    r["x"] = rng.normal(0.0, 3.0, (H, W))
    r["y"] = rng.normal(0.0, 3.0, (H, W))
    r["time_step"] = rng.integers(-3, 4, (H, W))
    r["layer"] = np.where(rng.random((H, W)) < valid, rng.integers(0, NK, (H, W)), -1)
    return r


class KeyPair:
    """The oracle and the GPU library with NK key layers at level 0."""

    def __init__(self, p, frames=2, seed=5):
        self.keys = _keys()
        self.sps = [O.style_pyramids(k) for k in self.keys]
        clip = synthetic.make_clip(W, H, 3, frames, seed=seed)
        rgba = clip[-1]["rgba"].copy()
        rgba[30:40, 5:25, 3] = 0.0  # masked-out pixels for the ribbon accumulation
        clip[-1]["rgba"] = rgba
        self.fps = [O.frame_pyramids(f) for f in clip]
        self.o = O.Oracle(W, H, W, H, NK, threads=8)
        self.g = TexSynth(device=0)
        self.g.initialize(W, H, W, H, NK)
        self.set_params(p)
        self.o.load_style_level(self.sps, 0)
        g = self.g
        g.initialize_exemplars(W, H, NK)
        for k, s in enumerate(self.sps):
            g.upload_image_color4(0, _abi.LAYER_EXEMPLAR_BASE, s["base"][0], k)
            g.upload_image_color4(0, _abi.LAYER_EXEMPLAR_OUTPUT, s["output"][0], k)
            g.upload_image_float(0, _abi.LAYER_EXEMPLAR_ORIENTATION, s["orient"][0], k)
            g.upload_image_float(0, _abi.LAYER_EXEMPLAR_DIST_TRANS, s["dt"][0], k)
            g.upload_image_int(0, _abi.LAYER_EXEMPLAR_OBJECT_IDS, s["ids"][0], k)

    def close(self):
        self.g.close()
        self.o.close()

    def set_params(self, p):
        self.o.set_params(p)
        self.g.set_params(p)

    def load_frame(self, f):
        fp = self.fps[f]
        self.o.load_frame_level(fp, 0)
        g = self.g
        g.upload_image_color4(0, _abi.LAYER_INPUT_COLOR, fp["rgba"][0])
        g.upload_image_float(0, _abi.LAYER_INPUT_ORIENTATION, fp["orient"][0])
        g.upload_image_int(0, _abi.LAYER_INPUT_ID, fp["ids"][0])
        g.upload_image_float2(0, _abi.LAYER_INPUT_VEL_B, fp["velb"][0])
        g.upload_image_float2(0, _abi.LAYER_INPUT_VEL_F, fp["velf"][0])
        g.upload_image_float(0, _abi.LAYER_INPUT_DIST_TRANS, fp["dt"][0])
        g.upload_image_float2(0, _abi.LAYER_INPUT_SCALE, fp["scale"][0])

    def random(self, f, seed=7):
        fp = self.fps[f]
        rnd = O.random_level(seed, 0, W, H, fp["rgba"][0], fp["orient"][0], self.sps[0]["output"][0],
                             self.sps[0]["orient"][0], False, True)
        self.o.upload_random(rnd)
        self.g.upload_image_color4(0, _abi.LAYER_RANDOM, rnd)

    def flip(self):
        self.o.flip()
        self.g.flip_anim_buffers()

    def both(self, name, *args):
        getattr(self.o, name)(*args)
        getattr(self.g, name)(*args)

    def compare(self, what):
        assert_offsets_equal(self.g.get_offsets(0), self.o.get_offsets(0), 1.0, "offsets " + what)
        assert_array_equal(self.g.get_residual(0), self.o.get_residual(0), "residual " + what)
        assert_array_equal(self.g.get_output(0), self.o.get_output(0), "output " + what)


def _params(keys=False):
    p = config_params(r=2)
    p.numStyles = NK
    if keys:
        p.interpolateKeyFrame = 1
        p.firstKeyIndex, p.lastKeyIndex = 0, NK - 1
    return p


def test_key_mask_in_propagate_and_scatter():
    kp = KeyPair(_params())
    try:
        kp.load_frame(0)
        kp.random(0)
        kp.both("randomize_offsets", 0)
        for jump in (8, 1):
            kp.both("propagate", 0, jump, 1)
            kp.compare("propagate, key 1, jump %d" % jump)
        kp.both("scatter", 0, 1)
        kp.compare("scatter, key 1")
        # under the mask the key's own positions on layer 1
        offs = kp.g.get_offsets(0)
        yy, xx = np.mgrid[0:H, 0:W]
        inside = ((xx - 40) ** 2 + (yy - 20) ** 2) < 10 ** 2
        assert (offs["layer"][inside] == 1).all()
        assert (offs["x"][inside] == xx[inside]).all() and (offs["y"][inside] == yy[inside]).all()
        kp.both("scatter", 0, -1)
        kp.compare("scatter, no key")
    finally:
        kp.close()


def _upload_cumulative(kp, rng):
    kp.o.init_cumulative_fields(W, H, NK)
    kp.g.initialize_cumulative_fields(W, H, NK)
    for fwd, layer_id in ((False, _abi.LAYER_CUMUL_FIELD_B), (True, _abi.LAYER_CUMUL_FIELD_F)):
        for j in range(NK):
            img = _ribbon_image(rng)
            kp.o.upload_cumulative_field(fwd, j, img)
            kp.g.upload_image_color4(0, layer_id, img, j)


def test_keyframe_propagate_and_scatter_through_cumulative_fields():
    kp = KeyPair(_params(keys=True))
    try:
        _upload_cumulative(kp, np.random.default_rng(11))
        kp.load_frame(0)
        kp.random(0)
        kp.both("randomize_offsets", 0)
        for jump in (16, 4, 1):
            kp.both("propagate", 0, jump, -1)
            kp.compare("propagate_kernel_keys jump %d" % jump)
        kp.both("scatter", 0, -1)
        kp.compare("scatter_kernel_keys")
        kp.both("propagate", 0, 0, 1)
        kp.compare("propagate_kernel_keys jump 0, key 1")
        kp.both("scatter", 0, 2)
        kp.compare("scatter_kernel_keys, key 2")
    finally:
        kp.close()


def test_accumulate_ribbon_field():
    kp = KeyPair(_params())
    rng = np.random.default_rng(12)
    try:
        kp.load_frame(0)
        kp.flip()
        kp.load_frame(1)
        canvas = rng.random((H, W, 4)).astype(np.float32)
        kp.o.load_canvas(0, canvas)
        kp.g.load_canvas(0, canvas)
        for fwd, ts, overwrite in ((True, 1, True), (True, 2, False), (False, -1, True), (False, -4, False)):
            rib = _ribbons(rng)
            kp.o.load_ribbon_field(0, rib)
            kp.g.load_ribbon_field(0, rib)
            kp.both("accumulate_ribbon_field", 0, fwd, ts, overwrite)
            what = "forwards %s, step %d, overwrite %s" % (fwd, ts, overwrite)
            got, ref = kp.g.get_ribbon_field(0), kp.o.get_ribbon_field(0)
            assert got.tobytes() == ref.tobytes(), "ribbon field " + what
            assert_array_equal(kp.g.get_advected_output(True, 0), kp.o.get_advected_output(True, 0),
                               "key colours " + what)
            assert (ref["layer"] >= 0).any() and (ref["layer"] < 0).any()
    finally:
        kp.close()


@pytest.mark.parametrize("look_forwards", [True, False])
def test_offsets_from_frame_to_key_ribbon(look_forwards):
    kp = KeyPair(_params())
    rng = np.random.default_rng(13)
    try:
        kp.load_frame(0)
        kp.random(0)
        for fwd, layer_id in ((False, _abi.LAYER_FRAME_TO_KEY_RIBBON_B), (True, _abi.LAYER_FRAME_TO_KEY_RIBBON_F)):
            img = _ribbon_image(rng, valid=0.6)
            kp.o.upload_frame_to_key_ribbon(fwd, img)
            kp.g.upload_image_color4(0, layer_id, img)
        kp.both("offsets_from_frame_to_key_ribbon", 0, look_forwards)
        kp.compare("frame-to-key ribbon offsets")
    finally:
        kp.close()


@pytest.mark.parametrize("fallback", [_abi.MERGE_FALLBACK_RANDOM, _abi.MERGE_FALLBACK_LAST_PASS])
def test_advect_with_frame_to_key_ribbons_and_merge_advected(fallback):
    """advectKernel with ADVECT_CHECK_FRAME_TO_KEY (long steps and pixels
    without an advection take the frame-to-key ribbon) in both directions,
    then mergeAdvectedKernel with either fallback."""
    kp = KeyPair(_params(), frames=3)
    rng = np.random.default_rng(14)
    try:
        for fwd, layer_id in ((False, _abi.LAYER_FRAME_TO_KEY_RIBBON_B), (True, _abi.LAYER_FRAME_TO_KEY_RIBBON_F)):
            img = _ribbon_image(rng, valid=0.6)
            kp.o.upload_frame_to_key_ribbon(fwd, img)
            kp.g.upload_image_color4(0, layer_id, img)
        kp.o.reset_advected()
        kp.g.reset_advected_buffers()
        kp.load_frame(0)
        kp.random(0)
        kp.both("randomize_offsets", 0)
        kp.both("propagate", 0, 2, -1)
        kp.flip()
        kp.load_frame(1)
        kp.random(1, seed=8)
        flags = _abi.ADVECT_CHECK_FRAME_TO_KEY
        kp.o.advect(0, 2, True, flags)
        kp.g.advect_offsets(0, 2, True, flags)
        kp.compare("advect forwards, step 2, frame-to-key")
        kp.o.advect(0, 1, False, flags | _abi.ADVECT_DO_NOT_CHECK_PREVIOUS)
        kp.g.advect_offsets(0, 1, False, flags | _abi.ADVECT_DO_NOT_CHECK_PREVIOUS)
        kp.compare("advect backwards, step 1, frame-to-key")
        kp.both("merge_advected_buffers", 0, fallback)
        kp.compare("merge advected")
    finally:
        kp.close()


@pytest.mark.parametrize("keys,first,last,scheme", [([2, 4], 0, 4, _abi.S_FMBM_RM), ([0, 2, 5], 1, 4, _abi.S_FMBM),
                                                    ([1, 3], 0, 4, _abi.S_FMBM_RM), ([1, 4], 0, 4, _abi.S_FBMO),
                                                    ([1, 4], 0, 4, _abi.S_TCTF), ([0, 3], 0, 3, _abi.S_IND)])
def test_keyframe_interpolation_driver_matches_oracle(keys, first, last, scheme):
    """keyFramesPreprocess (ribbons accumulated frame by frame in both
    directions, key-to-key and frame-to-key pyramids) and each scheme's
    schedule with SynthesisFrame's keyframe paths (TCTF starting with its
    initialisation pass), frames before the first key and keys outside the
    range included."""
    from painttween_gb300 import Synthesizer
    p = config_params(r=2, levels=2, iterations=2)
    p.scheme = scheme
    p.interpolateKeyFrame = 1
    p.numStyles = len(keys)
    styles = [synthetic.make_exemplar(W, H, seed=100 + i) for i in range(len(keys))]
    out = styles[0]["output"].copy()
    out[:, : W // 3, 3] = 0.0  # part of the first key left unpainted
    styles[0]["output"] = out
    nf = max(last, keys[-1]) + 1
    clip = synthetic.make_clip(W, H, 3, nf, seed=101)
    s = Synthesizer(device=0)
    try:
        s.setup(p, W, H, W, H, len(keys))
        for i, ex in enumerate(styles):
            s.set_style(i, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        s.set_keyframes(keys)
        got = s.synthesize_animation(first, last)
    finally:
        s.close()
    drv = O.OracleDriver(p, styles, clip, threads=8)
    drv.set_keyframes(keys)
    ref = drv.render(first, last)
    for f in range(first, last + 1):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "keyed frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "keyed output frame %d" % f)


@pytest.mark.parametrize("keyed", [False, True])
def test_tctf_with_ribbon_steps_matches_oracle(keyed):
    """TCTF over ribbon inputs of steps 2 and 4: a consecutive pass (or the
    keyframe initialisation) every 4th frame, refine passes at step 4, odd
    frames refined at steps 2 and 1 with the skipped frames linked to each
    new pass; with keys, the ribbons also carry the preprocessing's
    accumulation over 2 and 4 frames."""
    from painttween_gb300 import Synthesizer
    w, h, n = 48, 40, 6
    p = config_params(r=2, levels=2, iterations=2)
    p.scheme = _abi.S_TCTF
    if keyed:
        p.interpolateKeyFrame = 1
        p.numStyles = 2
        styles = [synthetic.make_exemplar(w, h, seed=100 + i) for i in range(2)]
    else:
        styles = [synthetic.make_exemplar(32, 32, seed=100)]
    clip = synthetic.make_clip(w, h, 3, n, seed=101)
    rng = np.random.default_rng(5)
    rib = {(f, st): (rng.normal(0, 1, (h, w, 2)).astype(np.float32), rng.normal(0, 1, (h, w, 2)).astype(np.float32))
           for f in range(n) for st in (2, 4)}
    s = Synthesizer(device=0)
    try:
        sh, sw = styles[0]["base"].shape[:2]
        s.setup(p, w, h, sw, sh, len(styles))
        for i, ex in enumerate(styles):
            s.set_style(i, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        for (f, st), (vf, vb) in rib.items():
            s.set_frame_ribbons(f, st, vf, vb)
        if keyed:
            s.set_keyframes([0, 5])
        got = s.synthesize_animation(0, n - 1)
    finally:
        s.close()
    drv = O.OracleDriver(p, styles, clip, threads=8)
    for (f, st), (vf, vb) in rib.items():
        drv.set_frame_ribbons(f, st, vf, vb)
    if keyed:
        drv.set_keyframes([0, 5])
    ref = drv.render(0, n - 1)
    for f in range(n):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "TCTF ribbons frame %d" % f)
        assert_array_equal(got[f][0], ref[f][2], "TCTF ribbons output frame %d" % f)
