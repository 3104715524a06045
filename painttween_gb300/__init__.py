"""painttween_gb300 -- GB300-native offset-field synthesis (PaintTween's
PatchMatch nearest-neighbour-field optimisation per pyramid level, with
offset advection for animations) as hand-written sm_103a CUDA kernels behind
the C ABI of include/painttween.h.
"""
from . import _abi
from ._abi import PATCH_DTYPE, Params, default_params
from .synthesizer import PaintTweenError, Synthesizer, TexSynth, host_array

__all__ = ["PATCH_DTYPE", "Params", "default_params", "PaintTweenError", "Synthesizer", "TexSynth", "_abi", "host_array"]
