"""Python driver of the reference-kernel port (test and baseline
infrastructure only).

RefPort has the step surface of oracle.oracle.Oracle, backed by the
reference's own CUDA kernels and TexSynth host wrappers
(src/PaintTweenCUDA/texSynth_kernel.cu and convolution.cu compiled unchanged
over texture objects; see oracle/refport/build.py), so that
RefPortDriver -- the oracle's restatement of the reference's per-frame
driver over this backend -- runs the reference's synthesis on a GPU.  The
host-side steps the reference performs in Qt code (the random-offset pyramid
drawn with glibc rand(), the image pyramids, the half-precision residual file
between passes) come from the oracle's restatements, which are pinned
against the reference's own host code and libc.
"""
import ctypes

import numpy as np

from oracle import oracle as O
from painttween_gb300 import _abi

_LIB = None

LAYER_SURF = 10


def lib():
    global _LIB
    if _LIB is None:
        from oracle.refport import build as rb
        path = rb.build()
        if path is None:
            raise RuntimeError("the reference port is not staged (no reference tree and no oracle/_ref/refport_src)")
        L = ctypes.CDLL(path)
        vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        sig = {
            "rp_create": (i, [i, i, i, i, i]), "rp_destroy": (None, []),
            "rp_error_count": (i, []), "rp_last_error": (ctypes.c_char_p, []),
            "rp_set_params": (None, [ctypes.POINTER(_abi.Params)]),
            "rp_init_exemplars": (None, [i, i, i]), "rp_init_cumulative_fields": (None, [i, i, i]),
            "rp_upload": (None, [i, i, vp, i, i, i]),
            "rp_flip": (None, []), "rp_reset_advected": (None, []), "rp_copy_base_to_working": (None, []),
            "rp_copy_base_to_advected": (None, [i]),
            "rp_randomize": (None, [i]), "rp_propagate": (None, [i, i, i]), "rp_scatter": (None, [i, i]),
            "rp_upsample": (None, [i]), "rp_advect": (None, [i, i, i, i]),
            "rp_merge_randomly": (None, [i, i, f, i]), "rp_merge_using_residual": (None, [i, i]),
            "rp_merge_advected": (None, [i, i]), "rp_update_residual": (None, [i]), "rp_sync": (None, [i, i]),
            "rp_accumulate_ribbon": (None, [i, i, i, i]), "rp_frame_to_key_ribbon": (None, [i, i]),
            "rp_get_offsets": (None, [i, vp]), "rp_get_residual": (None, [i, vp]), "rp_get_output": (None, [i, vp]),
            "rp_get_ribbon": (None, [i, vp]), "rp_get_advected_output": (None, [i, i, vp]),
            "rp_load_offsets": (None, [i, vp]), "rp_load_residual": (None, [i, vp]),
            "rp_load_ribbon": (None, [i, vp]), "rp_load_canvas": (None, [i, vp]),
            "rp_synchronize": (i, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


_KIND = {np.float32: None}


class RefPort:
    """TexSynth::* of the reference on the GPU, with the oracle's method names.
    One per process at a time (the reference keeps its state in file-scope
    globals)."""

    def __init__(self, W, H, SW, SH, NS=1, threads=1):
        self.W, self.H, self.SW, self.SH, self.NS = W, H, SW, SH, NS
        self.params = _abi.default_params()
        self.pass_counter = 0
        lib().rp_create(W, H, SW, SH, NS)
        self.check("rp_create")

    def check(self, where=""):
        L = lib()
        if L.rp_error_count():
            raise RuntimeError("reference port: %s (%s)" % (L.rp_last_error().decode(), where))

    def close(self):
        lib().rp_destroy()

    def set_threads(self, n):
        pass

    def set_params(self, p):
        self.params = p.copy()
        lib().rp_set_params(ctypes.byref(self.params))

    def lw(self, level):
        return self.W >> level

    def lh(self, level):
        return self.H >> level

    # --- uploads (TexSynth::uploadImage_*) ----------------------------------------
    def _up(self, kind, layer, arr, style=0):
        dt = {0: np.float32, 1: np.float32, 2: np.float32, 3: np.int32}[kind]
        a = np.ascontiguousarray(arr, dt)
        lib().rp_upload(kind, layer, _p(a), a.shape[1], a.shape[0], style)

    def load_style_level(self, styles, level):
        """Style::load(level), style.cpp:62-140."""
        s0 = styles[0]
        lib().rp_init_exemplars(s0["w"] >> level, s0["h"] >> level, len(styles))
        for k, s in enumerate(styles):
            self._up(0, _abi.LAYER_EXEMPLAR_BASE, s["base"][level], k)
            self._up(0, _abi.LAYER_EXEMPLAR_OUTPUT, s["output"][level], k)
            self._up(1, _abi.LAYER_EXEMPLAR_ORIENTATION, s["orient"][level], k)
            self._up(1, _abi.LAYER_EXEMPLAR_DIST_TRANS, s["dt"][level], k)
            self._up(3, _abi.LAYER_EXEMPLAR_OBJECT_IDS, s["ids"][level], k)

    def load_frame_level(self, fp, level):
        self.load_images(fp, level)
        self.load_anim_images(fp, level)

    def load_images(self, fp, level):
        """SynthesisFrame::loadImages, synthesisFrame.cpp:562-580."""
        self._up(0, _abi.LAYER_INPUT_COLOR, fp["rgba"][level])
        self._up(1, _abi.LAYER_INPUT_ORIENTATION, fp["orient"][level])
        self._up(3, _abi.LAYER_INPUT_ID, fp["ids"][level])

    def load_anim_images(self, fp, level):
        """SynthesisFrame::loadAnimImages, synthesisFrame.cpp:583-656 (the
        surface ids it uploads are read by no kernel)."""
        self._up(2, _abi.LAYER_INPUT_VEL_B, fp["velb"][level])
        self._up(2, _abi.LAYER_INPUT_VEL_F, fp["velf"][level])
        self._up(1, _abi.LAYER_INPUT_DIST_TRANS, fp["dt"][level])
        self._up(2, _abi.LAYER_INPUT_SCALE, fp["scale"][level])

    def upload_layered(self, layer, arr):
        kind = 2 if layer in (_abi.LAYER_INPUT_VEL_B, _abi.LAYER_INPUT_VEL_F, _abi.LAYER_INPUT_VEL_B_PREVIOUS,
                              _abi.LAYER_INPUT_VEL_F_PREVIOUS) else (1 if layer == _abi.LAYER_INPUT_DIST_TRANS else 0)
        self._up(kind, layer, arr)

    def upload_random(self, rnd):
        self._up(0, _abi.LAYER_RANDOM, rnd)

    def flip(self):
        lib().rp_flip()

    def reset_advected(self):
        lib().rp_reset_advected()

    def copy_base_to_advected(self, forwards):
        lib().rp_copy_base_to_advected(int(forwards))

    def copy_base_to_working(self):
        lib().rp_copy_base_to_working()

    # --- compute (each TexSynth wrapper syncs as the reference's does) ---------
    def randomize_offsets(self, level):
        lib().rp_randomize(level)

    def propagate(self, level, jump, key=-1):
        lib().rp_propagate(level, jump, key)

    def scatter(self, level, key=-1):
        lib().rp_scatter(level, key)
        self.pass_counter += 1

    def init_cumulative_fields(self, w, h, n):
        lib().rp_init_cumulative_fields(w, h, n)

    def upload_cumulative_field(self, forwards, layer, rgba):
        self._up(0, _abi.LAYER_CUMUL_FIELD_F if forwards else _abi.LAYER_CUMUL_FIELD_B, rgba, layer)

    def upload_frame_to_key_ribbon(self, forwards, rgba):
        self._up(0, _abi.LAYER_FRAME_TO_KEY_RIBBON_F if forwards else _abi.LAYER_FRAME_TO_KEY_RIBBON_B, rgba)

    def accumulate_ribbon_field(self, level, forwards, time_step, overwrite):
        lib().rp_accumulate_ribbon(level, int(forwards), time_step, int(overwrite))

    def merge_advected_buffers(self, level, fallback):
        lib().rp_merge_advected(level, fallback)

    def offsets_from_frame_to_key_ribbon(self, level, look_forwards):
        lib().rp_frame_to_key_ribbon(level, int(look_forwards))

    def load_ribbon_field(self, level, rib):
        lib().rp_load_ribbon(level, _p(np.ascontiguousarray(rib)))

    def get_ribbon_field(self, level):
        out = np.empty((self.lh(level), self.lw(level)), _abi.RIBBON_DTYPE)
        lib().rp_get_ribbon(level, _p(out))
        return out

    def load_canvas(self, level, rgba):
        lib().rp_load_canvas(level, _p(np.ascontiguousarray(rgba, np.float32)))

    def get_advected_output(self, forwards, level):
        out = np.empty((self.lh(level), self.lw(level), 4), np.float32)
        lib().rp_get_advected_output(int(forwards), level, _p(out))
        return out

    def upsample(self, level):
        lib().rp_upsample(level)

    def advect(self, level, time_step, forwards, flags):
        lib().rp_advect(level, time_step, int(forwards), flags)

    def merge_randomly(self, level, forwards, weight=0.5, force=False):
        lib().rp_merge_randomly(level, int(forwards), weight, int(force))

    def merge_using_residual(self, level, forwards):
        lib().rp_merge_using_residual(level, int(forwards))

    def update_residual(self, level):
        lib().rp_update_residual(level)

    def sync(self, level, flags=0):
        lib().rp_sync(level, flags)

    # --- state (WorkingBuffers::loadOffsets / loadResidual / getOutput) --------
    def load_offsets(self, level, offs):
        lib().rp_load_offsets(level, _p(np.ascontiguousarray(offs)))

    def load_residual(self, level, res):
        # the residual file's .b channel is half precision (workingBuffers.cpp:166-188)
        r = np.ascontiguousarray(np.asarray(res, np.float32).astype(np.float16).astype(np.float32))
        lib().rp_load_residual(level, _p(r))

    def get_offsets(self, level):
        out = np.empty((self.lh(level), self.lw(level)), _abi.PATCH_DTYPE)
        lib().rp_get_offsets(level, _p(out))
        return out

    def get_residual(self, level):
        out = np.empty((self.lh(level), self.lw(level)), np.float32)
        lib().rp_get_residual(level, _p(out))
        return out

    def get_output(self, level):
        out = np.empty((self.lh(level), self.lw(level), 4), np.float32)
        lib().rp_get_output(level, _p(out))
        return out


class RefPortDriver(O.OracleDriver):
    """The oracle's restatement of the reference's per-frame driver
    (renderAnimation* -> synthesizeConsecutive -> propagateAndScatter) over
    the reference's own kernels."""

    def _make_backend(self, W, H, SW, SH, NS, threads):
        return RefPort(W, H, SW, SH, NS)

    def render(self, first, last):
        out = super().render(first, last)
        self.o.check("render")
        return out
