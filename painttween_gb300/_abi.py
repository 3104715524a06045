"""ctypes/numpy description of the C ABI in include/painttween.h.

Pure data layout: the parameter block (a field-for-field TsParameters,
src/PaintTweenCUDA/texSynth_interface.h:79-152, plus driver fields) and the
36-byte PatchXF record (src/PaintTweenCUDA/types.h:94-109).
"""
import ctypes

import numpy as np

PT_MAX_STYLES = 5

PT_OK = 0
STATUS_NAMES = {
    0: "PT_OK", 1: "PT_ERR_INVALID", 2: "PT_ERR_CUDA", 3: "PT_ERR_OOM",
    4: "PT_ERR_STATE", 5: "PT_ERR_UNSUPPORTED", 6: "PT_ERR_TIMEOUT",
    7: "PT_ERR_BUDGET",
}

FORWARD, BACKWARD, BIDIRECTIONAL = 0, 1, 2
S_FMBM, S_FMBM_RM, S_FBMO, S_TCTF, S_IND = 0, 1, 2, 3, 4
RNG_REFERENCE, RNG_COUNTER = 0, 1
FILTER_EXACT, FILTER_TEXTURE = 0, 1

LAYER_EXEMPLAR_BASE = 0
LAYER_EXEMPLAR_OUTPUT = 1
LAYER_EXEMPLAR_ORIENTATION = 2
LAYER_EXEMPLAR_DIST_TRANS = 3
LAYER_EXEMPLAR_OBJECT_IDS = 4
LAYER_INPUT_COLOR = 5
LAYER_INPUT_ORIENTATION = 6
LAYER_INPUT_DIST_TRANS = 7
LAYER_INPUT_SCALE = 8
LAYER_INPUT_ID = 9
LAYER_INPUT_VEL_B = 11
LAYER_INPUT_VEL_F = 12
LAYER_INPUT_VEL_B_PREVIOUS = 13
LAYER_INPUT_VEL_F_PREVIOUS = 14
LAYER_RANDOM = 21

DONT_COPY_OFFSETS = 0x01
DONT_UPDATE_RESIDUAL = 0x10
MERGE_FALLBACK_RANDOM, MERGE_FALLBACK_LAST_PASS = 0x20, 0x40
ADVECT_IGNORE_RANDOM = 0x1
ADVECT_DO_NOT_CHECK_PREVIOUS = 0x10
ADVECT_CHECK_FRAME_TO_KEY = 0x20
ADVECT_UPDATE_RESIDUAL = 0x80


class Params(ctypes.Structure):
    """pt_params (include/painttween.h)."""
    _fields_ = [
        ("residualWindowSize", ctypes.c_int32),
        ("coherenceWeight", ctypes.c_float),
        ("distTransWeight", ctypes.c_float),
        ("lumShiftWeight", ctypes.c_float),
        ("lumShiftEnable", ctypes.c_int32),
        ("inputAnalogyWeight", ctypes.c_float),
        ("canvasOutputWeight", ctypes.c_float),
        ("numStyles", ctypes.c_int32),
        ("offsetsHistogramSlope", ctypes.c_float * PT_MAX_STYLES),
        ("offsetsHistogramThreshold", ctypes.c_float * PT_MAX_STYLES),
        ("maxDistortion", ctypes.c_float),
        ("alphaWeight", ctypes.c_float),
        ("transparencyOk", ctypes.c_int32),
        ("styleObjIdWeight", ctypes.c_float),
        ("orientationEnabled", ctypes.c_int32),
        ("colorspace", ctypes.c_int32),
        ("coherenceRatioRange", ctypes.c_float),
        ("coherenceAngleRange", ctypes.c_float),
        ("levels", ctypes.c_int32),
        ("scatterSamplesCount", ctypes.c_int32),
        ("advectionJitter", ctypes.c_float),
        ("timeDerivativeInputWeight", ctypes.c_float),
        ("timeDerivativeOutputWeight", ctypes.c_float),
        ("temporalCoherenceWeight", ctypes.c_float),
        ("hysteresisWeight", ctypes.c_float),
        ("interpolateKeyFrame", ctypes.c_int32),
        ("useGuide", ctypes.c_int32),
        ("currentInterpolationIndex", ctypes.c_int32),
        ("numFrames", ctypes.c_int32),
        ("numKeyFrames", ctypes.c_int32),
        ("firstKeyIndex", ctypes.c_int32),
        ("lastKeyIndex", ctypes.c_int32),
        ("distTransCull", ctypes.c_int32),
        ("residualWindowScaleU", ctypes.c_float),
        ("residualWindowScaleV", ctypes.c_float),
        ("direction", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("fixupPasses", ctypes.c_int32),
        ("scheme", ctypes.c_int32),
        ("finalLevel", ctypes.c_int32),
        ("rngMode", ctypes.c_int32),
        ("rngSeed", ctypes.c_uint32),
        ("filterMode", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 5),
    ]

    def copy(self):
        out = Params()
        ctypes.memmove(ctypes.byref(out), ctypes.byref(self), ctypes.sizeof(Params))
        return out


def default_params():
    """NLParameters::getTsDefaultParams (GUI/nlParameters.cpp:63-104) and the
    driver defaults of NLParameters::loadDefaults (:106-144); distTransCull is
    forced to 50 by SynthesisProcessor::updateParameters
    (synthesisProcessor.cpp:220)."""
    p = Params()
    p.residualWindowSize = 4
    p.coherenceWeight = 0.0
    p.distTransWeight = 0.0
    p.lumShiftWeight = 0.0
    p.lumShiftEnable = 0
    p.inputAnalogyWeight = 1.0
    p.canvasOutputWeight = 1.0
    p.orientationEnabled = 1
    for i in range(PT_MAX_STYLES):
        p.offsetsHistogramSlope[i] = 0.0
        p.offsetsHistogramThreshold[i] = 0.0
    p.numStyles = 1
    p.maxDistortion = 4.0
    p.alphaWeight = 1.0
    p.transparencyOk = 0
    p.coherenceRatioRange = 2.0
    p.coherenceAngleRange = 0.25
    p.levels = 4
    p.scatterSamplesCount = 25
    p.advectionJitter = 0.0
    p.timeDerivativeInputWeight = 1.0
    p.timeDerivativeOutputWeight = 1.0
    p.temporalCoherenceWeight = 0.2
    p.hysteresisWeight = 0.0
    p.interpolateKeyFrame = 0
    p.useGuide = 0
    p.distTransCull = 50
    p.residualWindowScaleU = 1.0
    p.residualWindowScaleV = 1.0
    p.firstKeyIndex = -1
    p.lastKeyIndex = -1
    p.styleObjIdWeight = 0.0
    p.direction = BIDIRECTIONAL
    p.colorspace = 0
    p.iterations = 3
    p.fixupPasses = 1
    p.scheme = S_FMBM_RM
    p.finalLevel = 0
    p.rngMode = RNG_REFERENCE
    p.rngSeed = 0
    p.filterMode = FILTER_TEXTURE  # the reference's texture-unit sampling
    return p


RIBBON_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("time_step", "<i4"), ("layer", "<i4")])
assert RIBBON_DTYPE.itemsize == 16
LAYER_CUMUL_FIELD_B, LAYER_CUMUL_FIELD_F = 17, 18
LAYER_FRAME_TO_KEY_RIBBON_B, LAYER_FRAME_TO_KEY_RIBBON_F = 19, 20


def output_level(p):
    """PT_OUTPUT_LEVEL: the level of the final output of a run."""
    return p.finalLevel if p.scheme in (S_IND, S_FBMO) else 0


PATCH_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"), ("theta", "<f4"), ("hysteresis", "<f4"),
    ("layer", "<i4"), ("scaleU", "<f4"), ("scaleV", "<f4"),
    ("lumShiftY", "<f4"), ("lumShiftA", "<f4"),
])
assert PATCH_DTYPE.itemsize == 36


KERNEL_PROPAGATE, KERNEL_SCATTER, KERNEL_RESIDUAL, KERNEL_CANVAS = 0, 1, 2, 3
PROFILE_TIMING, PROFILE_COUNTERS = 1, 2  # pt_set_profiling flags


class KernelStats(ctypes.Structure):
    """pt_kernel_stats (include/painttween.h)."""
    _fields_ = [("launches", ctypes.c_uint64), ("total_ms", ctypes.c_double),
                ("energy_evals", ctypes.c_uint64), ("taps", ctypes.c_uint64),
                ("temporal_taps", ctypes.c_uint64)]


def status_name(s):
    return STATUS_NAMES.get(s, "PT_STATUS_%d" % s)


class FrameInputs(ctypes.Structure):
    """pt_frame_inputs (include/painttween.h)."""
    _fields_ = [("rgba", ctypes.c_void_p), ("orient_tensor", ctypes.c_void_p), ("dist_trans", ctypes.c_void_p),
                ("ids", ctypes.c_void_p), ("vel_fwd", ctypes.c_void_p), ("vel_bwd", ctypes.c_void_p),
                ("scale", ctypes.c_void_p)]


class Request(ctypes.Structure):
    """pt_request (include/painttween.h)."""
    _fields_ = [("params", Params), ("style_w", ctypes.c_int), ("style_h", ctypes.c_int),
                ("style_base", ctypes.c_void_p), ("style_output", ctypes.c_void_p),
                ("style_orient_tensor", ctypes.c_void_p), ("style_dist_trans", ctypes.c_void_p),
                ("style_ids", ctypes.c_void_p), ("image_w", ctypes.c_int), ("image_h", ctypes.c_int),
                ("frames", ctypes.c_int), ("inputs", ctypes.POINTER(FrameInputs)), ("out_rgba", ctypes.c_void_p),
                ("out_offsets", ctypes.c_void_p), ("arrival_ms", ctypes.c_double), ("start_ms", ctypes.c_double),
                ("done_ms", ctypes.c_double), ("status", ctypes.c_int), ("device_bytes", ctypes.c_size_t)]
