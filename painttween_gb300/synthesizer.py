"""Python mirror of the reference's synthesizer interface for the offset-field
synthesis path, over the C ABI of libpainttween_gb300.

* `TexSynth` -- the step-wise calls of the reference's `namespace TexSynth`
  (src/PaintTweenCUDA/texSynth_kernel.h:38-91) with the same names, argument
  meaning and call order; errors raise `PaintTweenError` instead of exiting.
* `Synthesizer` -- the working-set level: a style exemplar plus per-frame
  image, orientation, distance-transform, object-ID and velocity inputs,
  "synthesize frame" and "synthesize animation"
  (GUI/nlSynthesizer.h:52-75, SynthesisProcessor::renderAnimationFMBM).
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import lib


class PaintTweenError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (_abi.status_name(status), message))
        self.status = status


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


class _HostBlock:
    """A block of page-locked host memory (pt_host_alloc), freed with its last user."""

    def __init__(self, nbytes):
        p = ctypes.c_void_p()
        st = lib().pt_host_alloc(nbytes, ctypes.byref(p))
        if st != _abi.PT_OK:
            raise PaintTweenError(st, "pt_host_alloc(%d) failed" % nbytes)
        self.p = p

    def __del__(self):
        if getattr(self, "p", None):
            lib().pt_host_free(self.p)
            self.p = None


def host_array(shape, dtype=np.float32):
    """A numpy array in page-locked host memory: frame inputs and results in
    such memory move between host and GPU at the full link speed."""
    dtype = np.dtype(dtype)
    n = max(int(np.prod(shape)) * dtype.itemsize, 1)
    blk = _HostBlock(n)
    raw = (ctypes.c_uint8 * n).from_address(blk.p.value)
    raw._block = blk  # the array's base keeps the block alive
    return np.frombuffer(raw, dtype=np.uint8, count=int(np.prod(shape)) * dtype.itemsize).view(dtype).reshape(shape)


class TexSynth:
    """One synthesis context on one GPU (pt_create)."""

    def __init__(self, device=0, hbm_budget=0):
        h = ctypes.c_void_p()
        st = lib().pt_create(device, hbm_budget, ctypes.byref(h))
        if st != _abi.PT_OK:
            raise PaintTweenError(st, "pt_create(device=%d) failed" % device)
        self.h = h
        self.W = self.H = 0
        self.params = _abi.default_params()

    # -- plumbing ------------------------------------------------------------
    def _check(self, st, what):
        if st != _abi.PT_OK:
            msg = lib().pt_last_error(self.h) if self.h else b""
            raise PaintTweenError(st, "%s: %s" % (what, (msg or b"").decode(errors="replace")))

    def close(self):
        if getattr(self, "h", None):
            lib().pt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def kernel_launches(self):
        return int(lib().pt_kernel_launches(self.h))

    @property
    def device_bytes(self):
        return int(lib().pt_device_bytes(self.h))

    def synchronize(self):
        self._check(lib().pt_synchronize(self.h), "pt_synchronize")

    # -- measurement (CUDA events on the context's stream) -----------------------
    def timer_record(self, slot):
        self._check(lib().pt_timer_record(self.h, slot), "pt_timer_record")

    def timer_elapsed(self, a, b):
        ms = ctypes.c_float()
        self._check(lib().pt_timer_elapsed(self.h, a, b, ctypes.byref(ms)), "pt_timer_elapsed")
        return ms.value

    def set_tiled_kernels(self, on):
        self._check(lib().pt_set_tiled_kernels(self.h, int(on)), "pt_set_tiled_kernels")

    def set_propagate_lanes(self, warps_per_row):
        self._check(lib().pt_set_propagate_lanes(self.h, int(warps_per_row)), "pt_set_propagate_lanes")

    def set_tma_staging(self, on):
        self._check(lib().pt_set_tma_staging(self.h, int(on)), "pt_set_tma_staging")

    def set_incremental(self, on):
        self._check(lib().pt_set_incremental(self.h, int(on)), "pt_set_incremental")

    def set_profiling(self, flags):
        """flags: 0, or _abi.PROFILE_TIMING | _abi.PROFILE_COUNTERS (True = both)."""
        if flags is True:
            flags = _abi.PROFILE_TIMING | _abi.PROFILE_COUNTERS
        self._check(lib().pt_set_profiling(self.h, int(flags)), "pt_set_profiling")

    def kernel_stats(self, kernel):
        st = _abi.KernelStats()
        self._check(lib().pt_get_kernel_stats(self.h, kernel, ctypes.byref(st)), "pt_get_kernel_stats")
        return dict(launches=st.launches, total_ms=st.total_ms, energy_evals=st.energy_evals, taps=st.taps,
                    temporal_taps=st.temporal_taps)

    # -- configuration (TexSynth::setup / uploadParameters) ----------------------
    def set_params(self, params):
        self.params = params.copy()
        self._check(lib().pt_set_params(self.h, ctypes.byref(self.params)), "pt_set_params")

    def initialize(self, image_w, image_h, style_w, style_h, num_styles=1):
        self._check(lib().pt_initialize(self.h, image_w, image_h, style_w, style_h, num_styles), "pt_initialize")
        self.W, self.H = image_w, image_h

    def initialize_exemplars(self, w, h, num_styles=1):
        self._check(lib().pt_initialize_exemplars(self.h, w, h, num_styles), "pt_initialize_exemplars")

    def upload_image_color4(self, level, layer, rgba, style=0):
        a = _c(rgba, np.float32)
        self._check(lib().pt_upload_image_color4(self.h, level, layer, _p(a), a.shape[1], a.shape[0], style),
                    "pt_upload_image_color4")

    def upload_image_float(self, level, layer, data, style=0):
        a = _c(data, np.float32)
        self._check(lib().pt_upload_image_float(self.h, level, layer, _p(a), a.shape[1], a.shape[0], style),
                    "pt_upload_image_float")

    def upload_image_float2(self, level, layer, xy):
        a = _c(xy, np.float32)
        self._check(lib().pt_upload_image_float2(self.h, level, layer, _p(a), a.shape[1], a.shape[0]),
                    "pt_upload_image_float2")

    def upload_image_int(self, level, layer, data, style=0):
        a = _c(data, np.int32)
        self._check(lib().pt_upload_image_int(self.h, level, layer, _p(a), a.shape[1], a.shape[0], style),
                    "pt_upload_image_int")

    def flip_anim_buffers(self):
        self._check(lib().pt_flip_anim_buffers(self.h), "pt_flip_anim_buffers")

    # -- compute (TexSynth::*) ---------------------------------------------------
    def create_random_level(self, level, frame):
        self._check(lib().pt_create_random_level(self.h, level, frame), "pt_create_random_level")

    def randomize_offsets(self, level):
        self._check(lib().pt_randomize_offsets(self.h, level), "pt_randomize_offsets")

    def propagate(self, level, jump, key_index=-1):
        self._check(lib().pt_propagate(self.h, level, jump, key_index), "pt_propagate")

    def scatter(self, level, key_index=-1):
        self._check(lib().pt_scatter(self.h, level, key_index), "pt_scatter")

    def upsample(self, fine_level):
        self._check(lib().pt_upsample(self.h, fine_level), "pt_upsample")

    def advect_offsets(self, level, time_step, forwards, op_flags=0):
        self._check(lib().pt_advect_offsets(self.h, level, time_step, int(forwards), op_flags), "pt_advect_offsets")

    def merge_randomly(self, level, forwards, weight_advected=0.5, force_valid=False):
        self._check(lib().pt_merge_randomly(self.h, level, int(forwards), weight_advected, int(force_valid)),
                    "pt_merge_randomly")

    def merge_using_residual(self, level, forwards):
        self._check(lib().pt_merge_using_residual(self.h, level, int(forwards)), "pt_merge_using_residual")

    def update_residual_cache(self, level):
        self._check(lib().pt_update_residual_cache(self.h, level), "pt_update_residual_cache")

    def sync_buffers(self, level, op_flags=0):
        self._check(lib().pt_sync_buffers(self.h, level, op_flags), "pt_sync_buffers")

    def reset_advected_buffers(self):
        self._check(lib().pt_reset_advected_buffers(self.h), "pt_reset_advected_buffers")

    def copy_offsets_to_advected(self, forwards):
        self._check(lib().pt_copy_offsets_to_advected(self.h, int(forwards)), "pt_copy_offsets_to_advected")

    # -- keyframe interpolation (TexSynth::accumulateRibbonField,
    #    offsetsFromFrameToKeyRibbon, initialize_cumulativeFields) -----------------
    def initialize_cumulative_fields(self, w, h, layers):
        self._check(lib().pt_initialize_cumulative_fields(self.h, w, h, layers), "pt_initialize_cumulative_fields")

    def accumulate_ribbon_field(self, level, forwards, time_step, overwrite):
        self._check(lib().pt_accumulate_ribbon_field(self.h, level, int(forwards), time_step, int(overwrite)),
                    "pt_accumulate_ribbon_field")

    def offsets_from_frame_to_key_ribbon(self, level, look_forwards):
        self._check(lib().pt_offsets_from_frame_to_key_ribbon(self.h, level, int(look_forwards)),
                    "pt_offsets_from_frame_to_key_ribbon")

    def set_keyframes(self, frames):
        """Style layer i is the key of frames[i] (increasing)."""
        a = np.ascontiguousarray(frames, dtype=np.int32)
        self._check(lib().pt_set_keyframes(self.h, _p(a), int(a.size)), "pt_set_keyframes")

    def merge_advected_buffers(self, level, merge_fallback):
        self._check(lib().pt_merge_advected_buffers(self.h, level, merge_fallback), "pt_merge_advected_buffers")

    def load_ribbon_field(self, level, ribbons):
        a = np.ascontiguousarray(ribbons, dtype=_abi.RIBBON_DTYPE)
        self._check(lib().pt_load_ribbon_field(self.h, level, _p(a)), "pt_load_ribbon_field")

    def get_ribbon_field(self, level):
        out = np.empty((self.H >> level, self.W >> level), _abi.RIBBON_DTYPE)
        self._check(lib().pt_get_ribbon_field(self.h, level, _p(out)), "pt_get_ribbon_field")
        return out

    def load_canvas(self, level, rgba):
        a = _c(rgba, np.float32)
        self._check(lib().pt_load_canvas(self.h, level, _p(a)), "pt_load_canvas")

    def get_advected_output(self, forwards, level):
        out = np.empty((self.H >> level, self.W >> level, 4), np.float32)
        self._check(lib().pt_get_advected_output(self.h, int(forwards), level, _p(out)), "pt_get_advected_output")
        return out

    def convolve_separable(self, src_dev, dst_dev, w, h, pitch, radius):
        """Gaussian blur of a device float image (device pointers as ints)."""
        self._check(lib().pt_convolve_separable(self.h, ctypes.c_void_p(src_dev), ctypes.c_void_p(dst_dev), w, h,
                                                pitch, radius), "pt_convolve_separable")

    # -- state transfer ------------------------------------------------------------
    def load_offsets(self, level, offsets):
        a = np.ascontiguousarray(offsets, dtype=_abi.PATCH_DTYPE)
        self._check(lib().pt_load_offsets(self.h, level, _p(a)), "pt_load_offsets")

    def load_residual(self, level, residual):
        a = _c(residual, np.float32)
        self._check(lib().pt_load_residual(self.h, level, _p(a)), "pt_load_residual")

    def get_offsets(self, level):
        out = np.empty((self.H >> level, self.W >> level), _abi.PATCH_DTYPE)
        self._check(lib().pt_get_offsets(self.h, level, _p(out)), "pt_get_offsets")
        return out

    def get_residual(self, level):
        out = np.empty((self.H >> level, self.W >> level), np.float32)
        self._check(lib().pt_get_residual(self.h, level, _p(out)), "pt_get_residual")
        return out

    def get_output(self, level):
        out = np.empty((self.H >> level, self.W >> level, 4), np.float32)
        self._check(lib().pt_get_output(self.h, level, _p(out)), "pt_get_output")
        return out


FRAME_CB = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_void_p,
                            ctypes.c_int, ctypes.c_int, ctypes.c_void_p)


class Synthesizer(TexSynth):
    """Working-set API: resident style and frame pyramids on the device."""

    def setup(self, params, image_w, image_h, style_w, style_h, num_styles=1):
        self.initialize(image_w, image_h, style_w, style_h, num_styles)
        self.set_params(params)

    def set_style(self, style, base, output, orient_tensor=None, dist_trans=None, object_ids=None):
        b, o = _c(base, np.float32), _c(output, np.float32)
        h, w = b.shape[:2]
        self._check(lib().pt_set_style(self.h, style, w, h, _p(b), _p(o), _p(_c(orient_tensor, np.float32)),
                                       _p(_c(dist_trans, np.float32)), _p(_c(object_ids, np.int32))),
                    "pt_set_style")

    def set_frame(self, frame, rgba, orient_tensor=None, dist_trans=None, object_ids=None, vel_fwd=None,
                  vel_bwd=None, scale=None):
        c = _c(rgba, np.float32)
        h, w = c.shape[:2]
        self._check(lib().pt_set_frame(self.h, frame, w, h, _p(c), _p(_c(orient_tensor, np.float32)),
                                       _p(_c(dist_trans, np.float32)), _p(_c(object_ids, np.int32)),
                                       _p(_c(vel_fwd, np.float32)), _p(_c(vel_bwd, np.float32)),
                                       _p(_c(scale, np.float32))), "pt_set_frame")

    def set_frame_ribbons(self, frame, step, vel_fwd, vel_bwd):
        """Velocities over `step` frames (2, 4, ...), forwards and backwards."""
        f, b = _c(vel_fwd, np.float32), _c(vel_bwd, np.float32)
        h, w = f.shape[:2]
        self._check(lib().pt_set_frame_ribbons(self.h, frame, step, w, h, _p(f), _p(b)), "pt_set_frame_ribbons")

    def set_frame_dict(self, frame, fr):
        self.set_frame(frame, fr["rgba"], fr.get("orient_tensor"), fr.get("dist_trans"), fr.get("object_ids"),
                       fr.get("vel_fwd"), fr.get("vel_bwd"), fr.get("scale"))

    def clear_frames(self):
        self._check(lib().pt_clear_frames(self.h), "pt_clear_frames")

    def _final_shape(self):
        fl = _abi.output_level(self.params)
        return self.H >> fl, self.W >> fl

    def synthesize_frame(self, frame):
        h, w = self._final_shape()
        rgba = np.empty((h, w, 4), np.float32)
        offs = np.empty((h, w), _abi.PATCH_DTYPE)
        self._check(lib().pt_synthesize_frame(self.h, frame, _p(rgba), _p(offs)), "pt_synthesize_frame")
        return rgba, offs

    def synthesize_animation(self, first, last):
        results = {}

        def cb(frame, rgba, offs, w, h, user):
            a = np.ctypeslib.as_array(rgba, shape=(h, w, 4)).copy()
            nb = w * h * _abi.PATCH_DTYPE.itemsize
            o = np.ctypeslib.as_array(ctypes.cast(offs, ctypes.POINTER(ctypes.c_uint8)), shape=(nb,))
            results[frame] = (a, o.view(_abi.PATCH_DTYPE).reshape(h, w).copy())

        cfn = FRAME_CB(cb)
        self._check(lib().pt_synthesize_animation(self.h, first, last, ctypes.cast(cfn, ctypes.c_void_p), None),
                    "pt_synthesize_animation")
        return results

    def get_frame_residual(self, frame):
        """The residual stored with a synthesised frame's final offsets."""
        h, w = self._final_shape()
        out = np.empty((h, w), np.float32)
        self._check(lib().pt_get_frame_residual(self.h, frame, _p(out)), "pt_get_frame_residual")
        return out

    def get_frame_result(self, frame, rgba=None, offsets=None):
        """Final output and offsets of one synthesised frame, written into the
        given arrays (e.g. host_array ones) or new ones."""
        h, w = self._final_shape()
        if rgba is None:
            rgba = np.empty((h, w, 4), np.float32)
        if offsets is None:
            offsets = np.empty((h, w), _abi.PATCH_DTYPE)
        assert rgba.shape == (h, w, 4) and rgba.dtype == np.float32 and rgba.flags.c_contiguous
        assert offsets.shape == (h, w) and offsets.dtype == _abi.PATCH_DTYPE and offsets.flags.c_contiguous
        self._check(lib().pt_get_frame_result(self.h, frame, _p(rgba), _p(offsets)), "pt_get_frame_result")
        return rgba, offsets
