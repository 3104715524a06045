"""Python side of the CPU oracle (test infrastructure only).

Loads oracle/libpt_oracle.so (the C restatement of the reference's kernels)
and drives it in the reference's call sequence:

* SynthesisProcessor::renderAnimationFMBM / renderConsecutivePass
  (src/PaintTweenCUDA/synthesisProcessor.cpp:703-753,846-878)
* SynthesisFrame::synthesizeConsecutive / propagateAndScatter
  (src/PaintTweenCUDA/synthesisFrame.cpp:214-323,483-508)
* renderAnimationIND, renderAnimationFBMO and renderAnimationTCTF with
  synthesizeInterpolated / advectNeighbors / refine / spatialUpsample
  (synthesisProcessor.cpp:807-1312, synthesisFrame.cpp:325-481)
* the EXR temp-file round trip between levels and passes becomes an
  in-memory store (offsets exact, residual rounded through half precision as
  WorkingBuffers::loadResidual reads the half .b channel).

Only tests, __graft_entry__.smoke() and bench.py's CPU baseline may use this
module, and only to check the library's results or as the timed CPU
baseline.
"""
import ctypes
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from painttween_gb300 import _abi  # noqa: E402  (ABI layout only)

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        from oracle import build as _build
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i, f, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint32
        sig = {
            "pto_create": (vp, [i, i, i, i, i]),
            "pto_destroy": (None, [vp]),
            "pto_set_threads": (None, [vp, i]),
            "pto_set_params": (None, [vp, ctypes.POINTER(_abi.Params)]),
            "pto_init_exemplars": (None, [vp, i, i, i]),
            "pto_upload_exemplar": (None, [vp, i, vp, vp, vp, vp, vp]),
            "pto_upload_layered": (None, [vp, i, vp, i, i]),
            "pto_upload_plain": (None, [vp, i, vp, i, i]),
            "pto_flip": (None, [vp]),
            "pto_copy_base_to_working": (None, [vp]),
            "pto_reset_advected": (None, [vp]),
            "pto_copy_base_to_advected": (None, [vp, i]),
            "pto_randomize": (None, [vp, i]),
            "pto_propagate": (None, [vp, i, i]),
            "pto_scatter": (None, [vp, i]),
            "pto_scatter_pass": (None, [vp, i, u32]),
            "pto_counter_random_level": (None, [u32, i, i, i, i, i, vp, vp, vp, vp, i, i, i, vp]),
            "pto_update_residual": (None, [vp, i]),
            "pto_sync": (None, [vp, i, i]),
            "pto_upsample": (None, [vp, i]),
            "pto_advect": (None, [vp, i, i, i, i]),
            "pto_merge_randomly": (None, [vp, i, i, f, i]),
            "pto_merge_using_residual": (None, [vp, i, i]),
            "pto_load_offsets": (None, [vp, i, vp]),
            "pto_load_residual": (None, [vp, i, vp]),
            "pto_get_offsets": (None, [vp, i, vp]),
            "pto_get_residual": (None, [vp, i, vp]),
            "pto_get_output": (None, [vp, i, vp]),
            "pto_energy_map": (None, [vp, i, vp, vp, vp]),
            "pto_sinf": (f, [f]), "pto_cosf": (f, [f]),
            "pto_atan2f": (f, [f, f]), "pto_logf": (f, [f]), "pto_acosf": (f, [f]),
            "pto_half_roundtrip": (f, [f]),
            "pto_glibc_stream": (None, [u32, i, vp]),
            "pto_random_level": (i, [u32, i, i, i, i, i, vp, vp, vp, vp, i, i, i, vp]),
            "pto_downsample_avg": (None, [vp, i, i, i, f, vp]),
            "pto_downsample_vote": (None, [vp, i, i, vp]),
            "pto_tensor_to_angle": (None, [vp, i, vp]),
            "pto_convolve_separable": (None, [vp, vp, i, i, i]),
            "pto_propagate_k": (None, [vp, i, i, i]),
            "pto_scatter_k": (None, [vp, i, u32, i]),
            "pto_propagate_keys": (None, [vp, i, i, i]),
            "pto_scatter_keys": (None, [vp, i, i]),
            "pto_init_cumulative_fields": (None, [vp, i, i, i]),
            "pto_upload_cumul": (None, [vp, i, i, vp, i, i]),
            "pto_upload_f2k": (None, [vp, i, vp, i, i]),
            "pto_accumulate_ribbon": (None, [vp, i, i, i, i]),
            "pto_frame_to_key_ribbon": (None, [vp, i, i]),
            "pto_load_ribbon": (None, [vp, i, vp]),
            "pto_get_ribbon": (None, [vp, i, vp]),
            "pto_load_canvas": (None, [vp, i, vp]),
            "pto_get_advected_output": (None, [vp, i, i, vp]),
            "pto_merge_advected": (None, [vp, i, i]),
            "pto_rgb_to_lab": (f, [vp, vp]),
            "pto_powd": (ctypes.c_double, [ctypes.c_double, ctypes.c_double]),
            "pto_basis": (None, [f, f, f, vp]),
            "pto_new_coord": (None, [f, f, f, f, vp, vp]),
            "pto_clamp_to_exemplar": (None, [vp, vp, i, i]),
            "pto_ssd": (f, [vp, vp, f]),
            "pto_ssd_plain": (f, [vp, vp]),
            "pto_ribbon_of": (None, [vp, vp, vp]),
            "pto_in_bounds": (i, [i, i, i, i, i, i]),
            "pto_pixel_wrap": (ctypes.c_longlong, [i, i, i, i]),
            "pto_to_patchxf": (None, [vp, vp]),
            "pto_random_level_keys": (i, [u32, i, i, i, i, i, vp, vp, vp, vp, i, i, i, i, i, i, i, vp]),
            "pto_tex_fetch": (None, [vp, i, i, i, i, vp, i, i, vp]),
            "pto_gauss_weights": (None, [i, i, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ---------------------------------------------------------------------------
# pyramids (downsample.cpp:41-209, GUI/nlDataAccess.cpp:82-93)
# ---------------------------------------------------------------------------

def num_levels(w, h):
    """ImagePyramid level count, imagePyramid.cpp:86 / downsample.cpp:47."""
    return int(min(math.floor(math.log2(w)), math.floor(math.log2(h))))


def pyramid_avg(img, vel=False):
    img = _c(img, np.float32)
    h, w = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    out = [img]
    for _ in range(1, num_levels(w, h)):
        cur = out[-1]
        ch_, cw = cur.shape[:2]
        dst = np.empty((ch_ >> 1, cw >> 1) + cur.shape[2:], np.float32)
        lib().pto_downsample_avg(_p(cur), cw, ch_, ch, 1.0 if vel else 0.0, _p(dst))
        out.append(dst)
    return out


def pyramid_vote(ids):
    ids = _c(ids, np.int32)
    h, w = ids.shape
    out = [ids]
    for _ in range(1, num_levels(w, h)):
        cur = out[-1]
        dst = np.empty((cur.shape[0] >> 1, cur.shape[1] >> 1), np.int32)
        lib().pto_downsample_vote(_p(cur), cur.shape[1], cur.shape[0], _p(dst))
        out.append(dst)
    return out


def convolve_separable(img, radius):
    """convolutionRowsGPU + convolutionColumnsGPU (normalised Gaussian)."""
    img = _c(img, np.float32)
    out = np.empty_like(img)
    lib().pto_convolve_separable(_p(img), _p(out), img.shape[1], img.shape[0], radius)
    return out


def tensor_to_angle(t3):
    t3 = _c(t3, np.float32)
    out = np.empty(t3.shape[:2], np.float32)
    lib().pto_tensor_to_angle(_p(t3), out.size, _p(out))
    return out


def pyramid_orientation(tensor):
    return [tensor_to_angle(t) for t in pyramid_avg(tensor)]


def style_pyramids(ex):
    w, h = ex["w"], ex["h"]
    z = np.zeros((h, w), np.float32)
    return dict(
        base=pyramid_avg(ex["base"]), output=pyramid_avg(ex["output"]),
        orient=pyramid_orientation(ex.get("orient_tensor", np.zeros((h, w, 3), np.float32))),
        dt=pyramid_avg(ex.get("dist_trans", z)),
        ids=pyramid_vote(ex.get("object_ids", np.zeros((h, w), np.int32))),
        w=w, h=h)


def frame_pyramids(fr):
    w, h = fr["w"], fr["h"]
    return dict(
        rgba=pyramid_avg(fr["rgba"]),
        orient=pyramid_orientation(fr["orient_tensor"]),
        dt=pyramid_avg(fr["dist_trans"]),
        ids=pyramid_vote(fr["object_ids"]),
        velf=pyramid_avg(fr.get("vel_fwd", np.zeros((h, w, 2), np.float32)), vel=True),
        velb=pyramid_avg(fr.get("vel_bwd", np.zeros((h, w, 2), np.float32)), vel=True),
        scale=pyramid_avg(fr.get("scale", np.ones((h, w, 2), np.float32))),
        w=w, h=h)


def counter_random_level(seed, level, style_w0, style_h0, img_rgba, img_orient, ex_out, ex_orient,
                         transparency_ok=False, orientation_enabled=True):
    """The PT_RNG_COUNTER random level (hashed draws, reference retry rule)."""
    h, w = img_orient.shape
    ew = ex_orient.shape[1]
    out = np.empty((h, w, 4), np.float32)
    lib().pto_counter_random_level(seed & 0xFFFFFFFF, w, h, level, style_w0, style_h0,
                                   _p(_c(img_rgba, np.float32)), _p(_c(img_orient, np.float32)),
                                   _p(_c(ex_out, np.float32)), _p(_c(ex_orient, np.float32)), ew,
                                   int(transparency_ok), int(orientation_enabled), _p(out))
    return out


def counter_seed(rng_seed, frame, level):
    """Seed of one random level in PT_RNG_COUNTER mode."""
    return (rng_seed ^ ((0x9E3779B9 * (frame + 1)) & 0xFFFFFFFF) ^ ((0x85EBCA6B * (level + 1)) & 0xFFFFFFFF)) & 0xFFFFFFFF


def tex_fetch(tex, q, hw=True):
    """Bilinear fetches of a (L, H, W, C) float texture at texture coordinates
    q[:, 0:2] (texel centres at +0.5) of layers q[:, 2]: the texture unit's
    arithmetic (hw) or exact FP32 bilinear."""
    tex = _c(tex, np.float32)
    q = _c(q, np.float32)
    L, H, W, C = tex.shape
    out = np.empty((q.shape[0], C), np.float32)
    lib().pto_tex_fetch(_p(tex), W, H, L, C, _p(q), q.shape[0], int(hw), _p(out))
    return out


def rgb_to_lab(rgba):
    """RGBtoLAB of one colour (the oracle's double pow)."""
    a = np.ascontiguousarray(rgba, np.float32)
    out = np.empty(4, np.float32)
    lib().pto_rgb_to_lab(_p(a), _p(out))
    return out


def glibc_stream(seed, n):
    out = np.empty(n, np.int32)
    lib().pto_glibc_stream(seed & 0xFFFFFFFF, n, _p(out))
    return out


def random_level(seed, level, style_w0, style_h0, img_rgba, img_orient, ex_out, ex_orient,
                 transparency_ok=False, orientation_enabled=True):
    """SynthesisFrame::createRandomPyramid for one level (synthesisFrame.cpp:66-150)."""
    h, w = img_orient.shape
    ew = ex_orient.shape[1]
    out = np.empty((h, w, 4), np.float32)
    lib().pto_random_level(seed & 0xFFFFFFFF, w, h, level, style_w0, style_h0,
                           _p(_c(img_rgba, np.float32)), _p(_c(img_orient, np.float32)),
                           _p(_c(ex_out, np.float32)), _p(_c(ex_orient, np.float32)), ew,
                           int(transparency_ok), int(orientation_enabled), _p(out))
    return out


# ---------------------------------------------------------------------------
# step-wise oracle with the TexSynth call surface
# ---------------------------------------------------------------------------

class Oracle:
    """CPU restatement of TexSynth::* over the reference's buffer model."""

    def __init__(self, W, H, SW, SH, NS=1, threads=1):
        self.W, self.H, self.SW, self.SH, self.NS = W, H, SW, SH, NS
        self.h = lib().pto_create(W, H, SW, SH, NS)
        lib().pto_set_threads(self.h, threads)
        self.params = _abi.default_params()
        self.pass_counter = 0

    def close(self):
        if self.h:
            lib().pto_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n):
        lib().pto_set_threads(self.h, n)

    def set_params(self, p):
        self.params = p.copy()
        lib().pto_set_params(self.h, ctypes.byref(self.params))

    def lw(self, level):
        return self.W >> level

    def lh(self, level):
        return self.H >> level

    # --- uploads -----------------------------------------------------------
    def load_style_level(self, styles, level):
        """Style::load(level), style.cpp:62-140."""
        s0 = styles[0]
        ew, eh = s0["w"] >> level, s0["h"] >> level
        lib().pto_init_exemplars(self.h, ew, eh, len(styles))
        self._ex = []
        for k, s in enumerate(styles):
            arrs = [_c(s["base"][level], np.float32), _c(s["output"][level], np.float32),
                    _c(s["orient"][level], np.float32), _c(s["dt"][level], np.float32),
                    _c(s["ids"][level], np.int32)]
            lib().pto_upload_exemplar(self.h, k, *[_p(a) for a in arrs])
            self._ex.append(arrs)

    def load_frame_level(self, fp, level):
        """SynthesisFrame::loadImages + loadAnimImages, synthesisFrame.cpp:562-656."""
        self.load_images(fp, level)
        self.load_anim_images(fp, level)

    def load_images(self, fp, level):
        """SynthesisFrame::loadImages, synthesisFrame.cpp:562-580."""
        L = lib()
        w, h = self.lw(level), self.lh(level)
        L.pto_upload_layered(self.h, _abi.LAYER_INPUT_COLOR, _p(_c(fp["rgba"][level], np.float32)), w, h)
        L.pto_upload_plain(self.h, _abi.LAYER_INPUT_ORIENTATION, _p(_c(fp["orient"][level], np.float32)), w, h)
        L.pto_upload_plain(self.h, _abi.LAYER_INPUT_ID, _p(_c(fp["ids"][level], np.int32)), w, h)

    def load_anim_images(self, fp, level):
        """SynthesisFrame::loadAnimImages, synthesisFrame.cpp:583-656."""
        L = lib()
        w, h = self.lw(level), self.lh(level)
        L.pto_upload_layered(self.h, _abi.LAYER_INPUT_VEL_B, _p(_c(fp["velb"][level], np.float32)), w, h)
        L.pto_upload_layered(self.h, _abi.LAYER_INPUT_VEL_F, _p(_c(fp["velf"][level], np.float32)), w, h)
        L.pto_upload_layered(self.h, _abi.LAYER_INPUT_DIST_TRANS, _p(_c(fp["dt"][level], np.float32)), w, h)
        L.pto_upload_plain(self.h, _abi.LAYER_INPUT_SCALE, _p(_c(fp["scale"][level], np.float32)), w, h)

    def upload_random(self, rnd):
        h, w = rnd.shape[:2]
        lib().pto_upload_plain(self.h, _abi.LAYER_RANDOM, _p(_c(rnd, np.float32)), w, h)

    def upload_layered(self, layer, arr):
        """A level-0-sized upload into one of the layered image inputs."""
        h, w = arr.shape[:2]
        lib().pto_upload_layered(self.h, layer, _p(_c(arr, np.float32)), w, h)

    def copy_base_to_working(self):
        lib().pto_copy_base_to_working(self.h)

    def flip(self):
        lib().pto_flip(self.h)

    def reset_advected(self):
        lib().pto_reset_advected(self.h)

    def copy_base_to_advected(self, forwards):
        lib().pto_copy_base_to_advected(self.h, int(forwards))

    # --- TexSynth compute calls (each ends with syncBuffers as the reference's
    #     host wrappers do) --------------------------------------------------
    def randomize_offsets(self, level):
        lib().pto_randomize(self.h, level)

    def propagate(self, level, jump, key=-1):
        """TexSynth::propagate, texSynth_kernel.cu:1306-1357: the keyframe
        kernel when interpolateKeyFrame is set."""
        if self.params.interpolateKeyFrame:
            lib().pto_propagate_keys(self.h, level, jump, key)
        else:
            lib().pto_propagate_k(self.h, level, jump, key)
        lib().pto_sync(self.h, level, 0)

    def scatter(self, level, key=-1):
        """TexSynth::scatter, texSynth_kernel.cu:1360-1401."""
        if self.params.interpolateKeyFrame:
            lib().pto_scatter_keys(self.h, level, key)
        else:
            lib().pto_scatter_k(self.h, level, self.pass_counter, key)
        self.pass_counter += 1
        lib().pto_sync(self.h, level, 0)

    # --- keyframe interpolation ----------------------------------------------
    def init_cumulative_fields(self, w, h, n):
        lib().pto_init_cumulative_fields(self.h, w, h, n)

    def upload_cumulative_field(self, forwards, layer, rgba):
        a = _c(rgba, np.float32)
        lib().pto_upload_cumul(self.h, int(forwards), layer, _p(a), a.shape[1], a.shape[0])

    def upload_frame_to_key_ribbon(self, forwards, rgba):
        a = _c(rgba, np.float32)
        lib().pto_upload_f2k(self.h, int(forwards), _p(a), a.shape[1], a.shape[0])

    def accumulate_ribbon_field(self, level, forwards, time_step, overwrite):
        lib().pto_accumulate_ribbon(self.h, level, int(forwards), time_step, int(overwrite))

    def merge_advected_buffers(self, level, fallback):
        lib().pto_merge_advected(self.h, level, fallback)

    def offsets_from_frame_to_key_ribbon(self, level, look_forwards):
        lib().pto_frame_to_key_ribbon(self.h, level, int(look_forwards))

    def load_ribbon_field(self, level, rib):
        lib().pto_load_ribbon(self.h, level, _p(np.ascontiguousarray(rib)))

    def get_ribbon_field(self, level):
        out = np.empty((self.lh(level), self.lw(level)), _abi.RIBBON_DTYPE)
        lib().pto_get_ribbon(self.h, level, _p(out))
        return out

    def load_canvas(self, level, rgba):
        lib().pto_load_canvas(self.h, level, _p(_c(rgba, np.float32)))

    def get_advected_output(self, forwards, level):
        out = np.empty((self.lh(level), self.lw(level), 4), np.float32)
        lib().pto_get_advected_output(self.h, int(forwards), level, _p(out))
        return out

    def upsample(self, level):
        lib().pto_upsample(self.h, level)

    def advect(self, level, time_step, forwards, flags):
        lib().pto_advect(self.h, level, time_step, int(forwards), flags)

    def merge_randomly(self, level, forwards, weight=0.5, force=False):
        lib().pto_merge_randomly(self.h, level, int(forwards), weight, int(force))

    def merge_using_residual(self, level, forwards):
        lib().pto_merge_using_residual(self.h, level, int(forwards))

    def update_residual(self, level):
        lib().pto_update_residual(self.h, level)

    def sync(self, level, flags=0):
        lib().pto_sync(self.h, level, flags)

    # --- state ---------------------------------------------------------------
    def load_offsets(self, level, offs):
        lib().pto_load_offsets(self.h, level, _p(np.ascontiguousarray(offs)))

    def load_residual(self, level, res):
        lib().pto_load_residual(self.h, level, _p(_c(res, np.float32)))

    def get_offsets(self, level):
        out = np.empty((self.lh(level), self.lw(level)), _abi.PATCH_DTYPE)
        lib().pto_get_offsets(self.h, level, _p(out))
        return out

    def get_residual(self, level):
        out = np.empty((self.lh(level), self.lw(level)), np.float32)
        lib().pto_get_residual(self.h, level, _p(out))
        return out

    def get_output(self, level):
        out = np.empty((self.lh(level), self.lw(level), 4), np.float32)
        lib().pto_get_output(self.h, level, _p(out))
        return out

    def energy_map(self, level, offs, f32=True, f64=True):
        offs = np.ascontiguousarray(offs)
        o32 = np.empty(offs.shape, np.float32) if f32 else None
        o64 = np.empty(offs.shape, np.float64) if f64 else None
        lib().pto_energy_map(self.h, level, _p(offs),
                             _p(o32) if f32 else None, _p(o64) if f64 else None)
        return o32, o64


# ---------------------------------------------------------------------------
# the reference's per-frame driver, restated over the oracle
# ---------------------------------------------------------------------------

class OracleDriver:
    """renderAnimationFMBM + renderConsecutivePass + synthesizeConsecutive."""

    def __init__(self, params, styles, frames, threads=1):
        self.user = params.copy()
        self.styles = [style_pyramids(s) for s in styles]
        self.frames = {i: frame_pyramids(f) for i, f in enumerate(frames)}
        f0 = frames[0]
        self.W, self.H = f0["w"], f0["h"]
        sw = max(s["w"] for s in styles)
        sh = max(s["h"] for s in styles)
        self.o = self._make_backend(self.W, self.H, sw, sh, len(styles), threads)
        self.store = {}
        self.last_saved = {}  # SynthesisFrame::_last_saved_pass: (frame, level) -> pass
        self.levels = params.levels
        self.keys = []        # DataAccess::keyFrameIndices: style i is the key of frame keys[i]
        self.key_sub = []
        self.keyed = False
        self.f2k = ({}, {})   # frame -> frame-to-key ribbon pyramid, [0] backward, [1] forward
        self.k2k = ({}, {})   # key full index -> key-to-key ribbon pyramid
        self.ribbons = {}     # (frame, step) -> velocities over `step` frames

    def _make_backend(self, W, H, SW, SH, NS, threads):
        """The object with TexSynth's step surface that the driver calls."""
        return Oracle(W, H, SW, SH, NS, threads=threads)

    def _update_parameters(self, frame, direction):
        """SynthesisFrame::updateParameters, synthesisFrame.cpp:522-542."""
        p = self.user.copy()
        p.advectionJitter = self.user.advectionJitter * 0.01 if frame % 3 == 0 else 0.0
        p.direction = direction
        self.o.set_params(p)

    def _random_level(self, frame, level):
        """createRandomPyramid (single style)."""
        fp = self.frames[frame]
        s = self.styles[0]
        args = (level, s["w"], s["h"], fp["rgba"][level], fp["orient"][level], s["output"][level],
                s["orient"][level], bool(self.user.transparencyOk), bool(self.user.orientationEnabled))
        if self.keyed:
            rnd = self._random_level_keyed(frame, level)
        elif self.user.rngMode == _abi.RNG_COUNTER:
            rnd = counter_random_level(counter_seed(self.user.rngSeed, frame, level), *args)
        else:
            rnd = random_level(frame * level, *args)
        self.o.upload_random(rnd)

    def _save(self, level, frame, pass_):
        self.store[(level, frame, pass_)] = (self.o.get_offsets(level), self.o.get_residual(level),
                                            self.o.get_output(level))

    def _load_offsets(self, level, frame, pass_):
        self.o.load_offsets(level, self.store[(level, frame, pass_)][0])

    def _load_residual(self, level, frame, pass_):
        self.o.load_residual(level, self.store[(level, frame, pass_)][1])

    def propagate_and_scatter(self, level, iterations, key=-1):
        """synthesisFrame.cpp:483-508 (with keys: a jump-0 pass first, and
        every pass with the frame's key index)."""
        for itr in range(iterations):
            if self.keyed:
                self.o.propagate(level, 0, key)
            j = 128
            while j > 1:
                self.o.propagate(level, j, key)
                j //= 2
            self.o.propagate(level, 1, key)
            self.o.propagate(level, 1, key)
            if itr < iterations - 1:
                self.o.scatter(level, key)

    def synthesize_consecutive(self, frame, level, pass_, is_first, forwards, source_pass, first_pass, time_step=1):
        o = self.o
        self._update_parameters(frame, _abi.FORWARD if forwards else _abi.BACKWARD)
        rm = self.user.scheme == _abi.S_FMBM_RM
        ops = (_abi.ADVECT_CHECK_FRAME_TO_KEY if self.keyed else 0) | (0 if rm else _abi.ADVECT_UPDATE_RESIDUAL)
        weight = self._key_advect_weight(frame, forwards) if self.keyed else 0.5
        coarsest = level == self.levels - 1
        if first_pass:
            self._random_level(frame, level)
            if is_first:
                if coarsest and self.keyed:
                    o.offsets_from_frame_to_key_ribbon(level, forwards)
                elif coarsest:
                    o.randomize_offsets(level)
                else:
                    self._load_offsets(level + 1, frame, source_pass)
                    o.upsample(level)
                    o.sync(level)
            if not is_first and coarsest:
                o.advect(level, time_step, forwards, ops)
                # copyBaseToWorking
                self._copy_base_to_working(level)
            elif not is_first:
                o.advect(level, time_step, forwards, ops | _abi.ADVECT_IGNORE_RANDOM)
                self._load_offsets(level + 1, frame, source_pass)
                self._load_residual(level + 1, frame, source_pass)
                o.upsample(level)
                o.sync(level)
                if rm:
                    o.merge_randomly(level, forwards, weight, False)
                else:
                    o.merge_using_residual(level, forwards)
        else:
            o.advect(level, time_step, forwards, ops | _abi.ADVECT_IGNORE_RANDOM)
            self._load_offsets(level, frame, pass_ - 1)
            self._load_residual(level, frame, pass_ - 1)
            o.sync(level, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
            if rm:
                o.merge_randomly(level, forwards, weight, False)
            else:
                o.merge_using_residual(level, forwards)
        o.sync(level)
        self.propagate_and_scatter(level, self.user.iterations, self._key_full(frame) if self.keyed else -1)
        self._save_images(level, frame, pass_)

    def _save_images(self, level, frame, pass_):
        """SynthesisFrame::saveImages, synthesisFrame.cpp:758-767."""
        self._save(level, frame, pass_)
        self.last_saved[(frame, level)] = pass_

    def _copy_base_to_working(self, level):
        """CudaBufferPair::copyBaseToWorking for the offsets pair."""
        self.o.copy_base_to_working()

    def render(self, first, last):
        """SynthesisProcessor::renderAnimation, synthesisProcessor.cpp:769-805,
        for the scheme of the parameters; returns {frame: (offsets, residual,
        output)} at the level PT_OUTPUT_LEVEL names."""
        if self.user.interpolateKeyFrame:
            return self._render_keyed(first, last)
        if self.user.scheme == _abi.S_IND:
            return self._render_ind(first, last)
        if self.user.scheme == _abi.S_FBMO:
            return self._render_fbmo(first, last)
        if self.user.scheme == _abi.S_TCTF:
            return self._render_tctf(first, last)
        return self._render_fmbm(first, last)

    # --- keyframe interpolation ------------------------------------------------
    def set_keyframes(self, frames):
        self.keys = list(frames)

    def _key_full(self, frame):
        return self.keys.index(frame) if frame in self.keys else -1

    def _key_sub_index(self, frame):
        return self.key_sub.index(frame) if frame in self.key_sub else -1

    def _update_key_subrange(self, first, last):
        """Style::updateKeyFrameSubrange, style.cpp:175-196."""
        K = self.keys
        self.key_sub = []
        for i, idx in enumerate(K):
            if first <= idx <= last:
                self.key_sub.append(idx)
            else:
                if i + 1 < len(K) and first < K[i + 1] <= last:
                    self.key_sub.append(idx)
                if i > 0 and first <= K[i - 1] < last:
                    self.key_sub.append(idx)

    def _key_advect_weight(self, frame, forwards):
        """Style::keyFrameAdvectWeight, style.cpp:207-223."""
        K = self.key_sub
        prev_key = -1
        while prev_key < len(K) - 1 and frame > K[prev_key + 1]:
            prev_key += 1
        has_prev, has_next = prev_key >= 0, prev_key < len(K) - 1
        prev_frame = K[prev_key] if has_prev else self.run_first
        next_frame = K[prev_key + 1] if has_next else self.run_last
        f32 = np.float32
        with np.errstate(invalid="ignore", divide="ignore"):  # 0/0 at a key: NaN, as in C
            if forwards:
                return float(f32(next_frame - frame) / f32(next_frame - prev_frame)) if has_next else 1.0
            return float(f32(frame - prev_frame) / f32(next_frame - prev_frame)) if has_prev else 1.0

    def _random_level_keyed(self, frame, level):
        """createRandomPyramid with setupWithKeys, synthesisFrame.cpp:94-139."""
        fp = self.frames[frame]
        h, w = fp["orient"][level].shape
        ew, eh = self.styles[0]["w"] >> level, self.styles[0]["h"] >> level
        ex_out = np.ascontiguousarray(np.stack([s["output"][level] for s in self.styles]), np.float32)
        ex_or = np.ascontiguousarray(np.stack([s["orient"][level] for s in self.styles]), np.float32)
        out = np.empty((h, w, 4), np.float32)
        lib().pto_random_level_keys((frame * level) & 0xFFFFFFFF, w, h, level, self.styles[0]["w"],
                                    self.styles[0]["h"], _p(_c(fp["rgba"][level], np.float32)),
                                    _p(_c(fp["orient"][level], np.float32)), _p(ex_out), _p(ex_or), ew, eh,
                                    len(self.styles), len(self.key_sub), self._key_full(self.key_sub[0]),
                                    int(self.user.transparencyOk), int(self.user.orientationEnabled), _p(out))
        return out

    def _ribbon_pyramid(self, rib, levels):
        """initializeRibbonPyramid, imagePyramid.cpp:211-235."""
        lv0 = np.stack([rib["time_step"].astype(np.float32), rib["y"], rib["x"],
                        rib["layer"].astype(np.float32)], axis=-1).astype(np.float32)
        pyr = [lv0]
        for l in range(1, levels):
            h, w = self.H >> l, self.W >> l
            p00 = pyr[-1][0:2 * h:2, 0:2 * w:2]
            lv = np.empty((h, w, 4), np.float32)
            lv[..., 0] = np.trunc(p00[..., 0])
            lv[..., 1] = p00[..., 1] * np.float32(0.5)
            lv[..., 2] = p00[..., 2] * np.float32(0.5)
            lv[..., 3] = np.trunc(p00[..., 3])
            pyr.append(lv)
        return pyr

    @staticmethod
    def _ribbons(h, w, layer):
        r = np.zeros((h, w), _abi.RIBBON_DTYPE)
        r["layer"] = layer
        return r

    def _accumulate(self, forwards, sfirst, slast):
        """SynthesisProcessor::accumulateRibbon, synthesisProcessor.cpp:528-627
        (level 0; steps above one frame through the ribbon inputs)."""
        o = self.o
        d = 0 if forwards else 1
        fk, lk = self.key_sub[0], self.key_sub[-1]
        if forwards:
            blank, frames = range(self.run_first, fk), list(range(fk, slast + 1))
        else:
            blank, frames = range(lk + 1, self.run_last + 1), list(range(lk, sfirst - 1, -1))
        acc = {frames[0]: self._ribbons(self.H, self.W, -1)}
        o.load_ribbon_field(0, acc[frames[0]])
        for f in blank:
            self.f2k[d][f] = self._ribbon_pyramid(acc[frames[0]], len(self.frames[f]["orient"]))
        def vel(f, step, key):
            if step == 1:
                return self.frames[f][key][0]
            r = self.ribbons.get((f, step))
            return None if r is None else r[key][0]

        for f in frames:
            fp = self.frames[f]
            o.load_images(fp, 0)
            ts = -1 if forwards else 1
            while (forwards and f + ts >= fk) or (not forwards and f + ts <= lk):
                pf, step = f + ts, abs(ts)
                ahead = pf < f
                vc = vel(f, step, "velb" if ahead else "velf")
                vp = vel(pf, step, "velf" if ahead else "velb")
                if vc is None or vp is None:
                    break  # loadRibbonPair finds no ribbon of this step
                if ahead:
                    o.upload_layered(_abi.LAYER_INPUT_VEL_B, vc)
                    o.upload_layered(_abi.LAYER_INPUT_VEL_F_PREVIOUS, vp)
                else:
                    o.upload_layered(_abi.LAYER_INPUT_VEL_F, vc)
                    o.upload_layered(_abi.LAYER_INPUT_VEL_B_PREVIOUS, vp)
                o.load_ribbon_field(0, acc[pf])
                o.accumulate_ribbon_field(0, forwards, ts, step == 1)
                ts *= 2
            acc[f] = o.get_ribbon_field(0)
            k = self._key_sub_index(f)
            if k >= 0:
                full = self._key_full(f)
                self.k2k[d][full] = self._ribbon_pyramid(acc[f], len(fp["orient"]))
                o.load_canvas(0, self.styles[full]["output"][0])
                acc[f] = self._ribbons(self.H, self.W, k)
                o.load_ribbon_field(0, acc[f])
            self.f2k[d][f] = self._ribbon_pyramid(acc[f], len(fp["orient"]))

    def set_frame_ribbons(self, frame, step, vel_fwd, vel_bwd):
        """Velocities over `step` frames (pt_set_frame_ribbons)."""
        self.ribbons[(frame, step)] = dict(velf=pyramid_avg(vel_fwd, vel=True), velb=pyramid_avg(vel_bwd, vel=True))

    def _stepped(self, f, ts):
        """The frame's inputs with the velocities of time step ts
        (loadAnimImages, synthesisFrame.cpp:583-611)."""
        fp = self.frames[f]
        if ts == 1:
            return fp
        r = self.ribbons[(f, ts)]
        return dict(fp, velf=r["velf"], velb=r["velb"])

    def _max_ribbon_step(self, first, last):
        step = 1
        while all((f, step * 2) in self.ribbons for f in range(first, last + 1)):
            step *= 2
        return step

    def _frame(self, f, level, ts=1):
        """loadImages + loadAnimImages (with keys: the frame-to-key ribbons)."""
        self.o.load_frame_level(self._stepped(f, ts), level)
        if self.keyed:
            self._bind_frame_keys(f, level)

    def _anim(self, f, level, ts=1):
        self.o.load_anim_images(self._stepped(f, ts), level)
        if self.keyed:
            self._bind_frame_keys(f, level)

    def _link(self, frame, level, this_pass):
        """linkTempImagesToNextPass through linkImagesToPass (workingBuffers.cpp:
        329-365): this pass becomes the frame's last saved pass."""
        src = (level, frame, self.last_saved.get((frame, level), 0))
        if src in self.store and src[2] != this_pass:
            self.store[(level, frame, this_pass)] = self.store[src]

    def _bind_frame_keys(self, frame, level):
        for d in (0, 1):
            pyr = self.f2k[d].get(frame)
            if pyr is not None and level < len(pyr):
                self.o.upload_frame_to_key_ribbon(d == 1, pyr[level])

    def _upload_key_fields(self, level):
        """Style::load with keys, style.cpp:122-134."""
        if 0 not in self.k2k[0] or not self.key_sub:
            return
        lw, lh = self.W >> level, self.H >> level
        self.o.init_cumulative_fields(lw, lh, len(self.key_sub))
        for i, kf in enumerate(self.key_sub):
            full = self._key_full(kf)
            for d in (0, 1):
                pyr = self.k2k[d].get(full)
                if pyr is not None and level < len(pyr):
                    self.o.upload_cumulative_field(d == 1, i, pyr[level])

    def _render_keyed(self, first, last):
        """keyFramesPreprocess (synthesisProcessor.cpp:629-674), then
        renderAnimationFMBM with the keyframe paths."""
        user = self.user.copy()
        self._update_key_subrange(first, last)
        sfirst, slast = min(first, self.key_sub[0]), max(last, self.key_sub[-1])
        self.run_first, self.run_last = first, last
        self.keyed = True
        try:
            p = user.copy()
            p.interpolateKeyFrame = 0
            self.o.set_params(p)
            self.o.load_style_level(self.styles, 0)
            self._accumulate(True, sfirst, slast)
            self._accumulate(False, sfirst, slast)
            p = user.copy()
            p.interpolateKeyFrame = 1
            p.numFrames = slast - sfirst
            p.firstKeyIndex = self._key_full(self.key_sub[0])
            p.lastKeyIndex = self._key_full(self.key_sub[-1])
            self.user = p
            return {_abi.S_FBMO: self._render_fbmo, _abi.S_TCTF: self._render_tctf,
                    _abi.S_IND: self._render_ind}.get(p.scheme, self._render_fmbm)(first, last)
        finally:
            self.user = user
            self.keyed = False

    def _advect_neighbors(self, frame, level, source_pass, first, last, neighbours=True, ts=1):
        """SynthesisFrame::advectNeighbors, synthesisFrame.cpp:325-382, with
        the frames of the synthesised range as neighbours (with keys, a side
        without one advects the frame-to-key ribbons)."""
        o, u = self.o, self.user
        o.reset_advected()
        ops = _abi.ADVECT_CHECK_FRAME_TO_KEY if self.keyed else 0
        prior = frame - ts if neighbours and frame - ts >= first else None
        nxt = frame + ts if neighbours and frame + ts <= last else None
        temporal = (u.timeDerivativeInputWeight > 0 or u.timeDerivativeOutputWeight > 0
                    or u.temporalCoherenceWeight > 0)
        if last == first or not temporal or (prior is None and nxt is None and not self.keyed):
            self._anim(frame, level, ts)
            return
        for nb, fwd in ((prior, True), (nxt, False)):
            if nb is not None and source_pass >= 0:
                self._frame(nb, level, ts)
                o.flip()
                self._anim(frame, level, ts)
                self._load_last_saved(nb, level)
                o.advect(level, ts, fwd, ops)
            elif self.keyed:
                self._anim(frame, level, ts)
                o.advect(level, ts, fwd, ops | _abi.ADVECT_DO_NOT_CHECK_PREVIOUS)

    def synthesize_interpolated(self, frame, level, this_pass, source_pass, first, last):
        """SynthesisFrame::synthesizeInterpolated, synthesisFrame.cpp:384-418."""
        o = self.o
        self._update_parameters(frame, _abi.BIDIRECTIONAL)
        self._advect_neighbors(frame, level, source_pass, first, last)
        o.load_images(self.frames[frame], level)
        self._load_offsets(level, frame, source_pass)
        o.sync(level, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
        self.propagate_and_scatter(level, self.user.iterations, self._key_full(frame) if self.keyed else -1)
        self._save_images(level, frame, this_pass)

    def _render_fbmo(self, first, last):
        """renderAnimationFBMO, synthesisProcessor.cpp:926-1022, with
        renderInterpolatedFixupPass (:880-924) for every frame."""
        o, u = self.o, self.user
        final_pass = u.fixupPasses + 2
        for level in range(self.levels - 1, u.finalLevel - 1, -1):
            o.load_style_level(self.styles, level)
            if self.keyed:
                self._upload_key_fields(level)
            for pass_ in (0, 1):
                o.reset_advected()
                forwards = pass_ == 0
                frames = list(range(first, last + 1)) if forwards else list(range(last, first - 1, -1))
                for i, f in enumerate(frames):
                    is_first = i == 0
                    if not is_first or pass_ > 0:
                        o.flip()
                    self._frame(f, level)
                    self.synthesize_consecutive(f, level, pass_, is_first, forwards, final_pass, True)
            for f in range(first, last + 1):  # pass 2: forward and backward merged
                self._load_offsets(level, f, 0)
                self._load_residual(level, f, 0)
                o.copy_base_to_advected(True)
                o.sync(level, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
                self._load_offsets(level, f, 1)
                self._load_residual(level, f, 1)
                o.sync(level, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
                w = self._key_advect_weight(f, True) if self.keyed else 0.5
                o.merge_randomly(level, True, w, True)  # TexSynth::mergeRandomly ends with a sync
                o.sync(level)
                self._save(level, f, 2)
            for pass_ in range(3, u.fixupPasses + 3):
                for f in range(first, last + 1):
                    self._random_level(f, level)
                    self.synthesize_interpolated(f, level, pass_, pass_ - 1, first, last)
        return {f: self.store[(u.finalLevel, f, final_pass)] for f in range(first, last + 1)}

    def _render_ind(self, first, last):
        """renderAnimationIND, synthesisProcessor.cpp:807-844: every frame on
        its own, coarse to fine, each pass a first frame going forwards."""
        total = self.user.fixupPasses + 1
        for f in range(first, last + 1):
            for level in range(self.levels - 1, self.user.finalLevel - 1, -1):
                self.o.load_style_level(self.styles, level)
                if self.keyed:
                    self._upload_key_fields(level)
                self.o.reset_advected()
                for pass_ in range(total):
                    self._frame(f, level)
                    self.synthesize_consecutive(f, level, pass_, True, True, pass_, pass_ == 0)
        final_pass = total - 1 if self.user.finalLevel == 0 else 0
        return {f: self.store[(self.user.finalLevel, f, final_pass)] for f in range(first, last + 1)}

    def _render_fmbm(self, first, last):
        """renderAnimationFMBM, synthesisProcessor.cpp:846-878, with
        renderSpatialUpsample (:1025-1045) from a final level down to 0."""
        total = self.user.fixupPasses + 1
        for level in range(self.levels - 1, self.user.finalLevel - 1, -1):
            self.o.load_style_level(self.styles, level)
            if self.keyed:
                self._upload_key_fields(level)
            self.o.reset_advected()
            for pass_ in range(total):
                self._render_pass(level, pass_, total - 1, first, last)
        for level in range(self.user.finalLevel, 0, -1):
            self.o.load_style_level(self.styles, level - 1)
            if self.keyed:
                self._upload_key_fields(level - 1)
            for f in range(first, last + 1):
                self._spatial_upsample(f, level, level - 1, True)
        final_pass = total - 1 if self.user.finalLevel == 0 else 0
        return {f: self.store[(0, f, final_pass)] for f in range(first, last + 1)}

    def _load_last_saved(self, frame, level):
        """SynthesisFrame::loadLastSavedOffsets, synthesisFrame.cpp:769-772:
        pass 0 before any save (a zero-filled vector); a pass never saved
        leaves the base offsets as they are (the file load fails)."""
        key = (level, frame, self.last_saved.get((frame, level), 0))
        if key in self.store:
            self.o.load_offsets(level, self.store[key][0])

    def _spatial_upsample(self, frame, coarse, fine, save):
        """SynthesisFrame::spatialUpsample, synthesisFrame.cpp:465-481."""
        self._load_last_saved(frame, coarse)
        self.o.upsample(fine)
        self.o.sync(fine, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
        if save:
            self._save_images(fine, frame, 0)

    def _refine_pass(self, level, last_coarse_pass, this_pass, first, last, op="even_and_odd", ts=1):
        """renderRefinePass (synthesisProcessor.cpp:1078-1150) and
        renderInitializationPass (:1047-1076, op "initialize") with
        SynthesisFrame::refine (synthesisFrame.cpp:420-463)."""
        o = self.o
        coarsest = level == self.levels - 1
        coarse_step = 2 * ts
        if op == "odd":
            frames = range(first + ts, last + 1, coarse_step)
        elif op == "even":
            frames = range(first, last + 1, coarse_step)
        else:
            frames = range(first, last + 1, ts)
        init = "previous"
        if op in ("initialize", "odd"):
            init = "temporal" if coarsest else "spatial"
        elif op == "even_and_odd" and last_coarse_pass == this_pass - 1:
            init = "spatial"
        for f in frames:
            self._update_parameters(f, _abi.BIDIRECTIONAL)
            self._advect_neighbors(f, level, this_pass - 1, first, last, op != "initialize", ts)
            if init == "temporal":
                o.merge_advected_buffers(level, _abi.MERGE_FALLBACK_RANDOM)
            elif init == "spatial":
                self._spatial_upsample(f, level + 1, level, False)
            else:
                self._load_last_saved(f, level)
                o.sync(level, _abi.DONT_COPY_OFFSETS | _abi.DONT_UPDATE_RESIDUAL)
            o.load_images(self.frames[f], level)
            self.propagate_and_scatter(level, self.user.iterations, self._key_full(f) if self.keyed else -1)
            self._save_images(level, f, this_pass)
        if op == "odd":
            for f in range(first, last + 1, coarse_step):
                self._link(f, level, this_pass)
        elif op == "even":
            for f in range(first + ts, last + 1, coarse_step):
                self._link(f, level, this_pass)

    def _render_tctf(self, first, last):
        """renderAnimationTCTF, synthesisProcessor.cpp:1152-1312, run locally,
        over the longest ribbon step every frame has."""
        u = self.user
        L = self.levels - 1
        T = self._max_ribbon_step(first, last)
        ops = [("initialize" if self.keyed else "consecutive", L, T)]
        for level in range(L, u.finalLevel - 1, -1):
            ops.append(("even_and_odd", level, T))
            if T < last - first:
                ops += [("even_and_odd", level, T)] * (u.fixupPasses + 1)
        ts = T // 2
        while ts > 0:
            for level in range(L, u.finalLevel - 1, -1):
                ops.append(("odd", level, ts))
                if ts < last - first:
                    ops += [("even_and_odd", level, ts)] * u.fixupPasses
            ts //= 2
        ops += [("upsample", level, 1) for level in range(u.finalLevel - 1, -1, -1)]
        self.o.reset_advected()
        passes_this = passes_last = 0
        last_level = -1
        for op, level, ts in ops:
            if last_level != level:
                self.o.load_style_level(self.styles, level)
                if self.keyed:
                    self._upload_key_fields(level)
                passes_last = passes_this
                last_level = level
            if op == "initialize":
                self._refine_pass(level, passes_this - 1, 0, first, last, "initialize", ts)
                passes_this = 1
            elif op == "consecutive":
                self._render_pass(level, passes_this, passes_this - 1, first, last, ts)
                passes_this += 1
            elif op == "upsample":
                for f in range(first, last + 1):
                    self._spatial_upsample(f, level + 1, level, True)
                passes_this = 1
            else:
                self._refine_pass(level, passes_last - 1, passes_this, first, last, op, ts)
                passes_this += 1
        return {f: self.store[(0, f, passes_this - 1)] for f in range(first, last + 1)}

    def _render_pass(self, level, pass_, source_pass, first, last, time_step=1):
        """renderConsecutivePass, synthesisProcessor.cpp:703-753."""
        forwards = (pass_ % 2) == 0
        frames = (list(range(first, last + 1, time_step)) if forwards
                  else list(range(last, first - 1, -time_step)))
        if pass_ > 0:
            self._save(level, frames[0], pass_)
            frames = frames[1:]
        for i, f in enumerate(frames):
            is_first = (i == 0) and (pass_ == 0)
            if not is_first:
                self.o.flip()
            self._frame(f, level, time_step)
            self.synthesize_consecutive(f, level, pass_, is_first, forwards, source_pass, pass_ == 0, time_step)

