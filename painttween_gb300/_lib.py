"""Loader of the in-tree CUDA library libpainttween_gb300.so.

There is no CPU fallback: if the library has not been built, or cannot be
loaded, importing the bindings raises.
"""
import ctypes
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpainttween_gb300.so")

_lib = None

# name -> (restype, argtypes); every public entry point of include/painttween.h
_VP = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_PP = ctypes.POINTER(_abi.Params)
SIGNATURES = {
    "pt_abi_version": (_I, []),
    "pt_status_string": (ctypes.c_char_p, [_I]),
    "pt_last_error": (ctypes.c_char_p, [_VP]),
    "pt_default_params": (None, [_PP]),
    "pt_device_bytes": (ctypes.c_size_t, [_VP]),
    "pt_create": (_I, [_I, ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "pt_destroy": (_I, [_VP]),
    "pt_set_params": (_I, [_VP, _PP]),
    "pt_get_params": (_I, [_VP, _PP]),
    "pt_initialize": (_I, [_VP, _I, _I, _I, _I, _I]),
    "pt_initialize_exemplars": (_I, [_VP, _I, _I, _I]),
    "pt_upload_image_color4": (_I, [_VP, _I, _I, _VP, _I, _I, _I]),
    "pt_upload_image_float": (_I, [_VP, _I, _I, _VP, _I, _I, _I]),
    "pt_upload_image_float2": (_I, [_VP, _I, _I, _VP, _I, _I]),
    "pt_upload_image_int": (_I, [_VP, _I, _I, _VP, _I, _I, _I]),
    "pt_flip_anim_buffers": (_I, [_VP]),
    "pt_create_random_level": (_I, [_VP, _I, _I]),
    "pt_randomize_offsets": (_I, [_VP, _I]),
    "pt_propagate": (_I, [_VP, _I, _I, _I]),
    "pt_scatter": (_I, [_VP, _I, _I]),
    "pt_upsample": (_I, [_VP, _I]),
    "pt_advect_offsets": (_I, [_VP, _I, _I, _I, _I]),
    "pt_merge_randomly": (_I, [_VP, _I, _I, _F, _I]),
    "pt_merge_using_residual": (_I, [_VP, _I, _I]),
    "pt_update_residual_cache": (_I, [_VP, _I]),
    "pt_sync_buffers": (_I, [_VP, _I, _I]),
    "pt_reset_advected_buffers": (_I, [_VP]),
    "pt_copy_offsets_to_advected": (_I, [_VP, _I]),
    "pt_initialize_cumulative_fields": (_I, [_VP, _I, _I, _I]),
    "pt_accumulate_ribbon_field": (_I, [_VP, _I, _I, _I, _I]),
    "pt_offsets_from_frame_to_key_ribbon": (_I, [_VP, _I, _I]),
    "pt_merge_advected_buffers": (_I, [_VP, _I, _I]),
    "pt_set_keyframes": (_I, [_VP, _VP, _I]),
    "pt_set_frame_ribbons": (_I, [_VP, _I, _I, _I, _I, _VP, _VP]),
    "pt_load_ribbon_field": (_I, [_VP, _I, _VP]),
    "pt_get_ribbon_field": (_I, [_VP, _I, _VP]),
    "pt_load_canvas": (_I, [_VP, _I, _VP]),
    "pt_get_advected_output": (_I, [_VP, _I, _I, _VP]),
    "pt_load_offsets": (_I, [_VP, _I, _VP]),
    "pt_load_residual": (_I, [_VP, _I, _VP]),
    "pt_get_offsets": (_I, [_VP, _I, _VP]),
    "pt_get_residual": (_I, [_VP, _I, _VP]),
    "pt_get_output": (_I, [_VP, _I, _VP]),
    "pt_convolve_separable": (_I, [_VP, _VP, _VP, _I, _I, _I, _I]),
    "pt_gaussian_kernel": (_I, [_I, _I, _VP]),
    "pt_convolve_separable_noalloc": (_I, [_VP, _VP, _I, _I, _I, _I, _VP]),
    "pt_set_style": (_I, [_VP, _I, _I, _I, _VP, _VP, _VP, _VP, _VP]),
    "pt_set_frame": (_I, [_VP, _I, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pt_clear_frames": (_I, [_VP]),
    "pt_synthesize_frame": (_I, [_VP, _I, _VP, _VP]),
    "pt_synthesize_animation": (_I, [_VP, _I, _I, _VP, _VP]),
    "pt_kernel_launches": (ctypes.c_uint64, [_VP]),
    "pt_synchronize": (_I, [_VP]),
    "pt_timer_record": (_I, [_VP, _I]),
    "pt_timer_elapsed": (_I, [_VP, _I, _I, ctypes.POINTER(ctypes.c_float)]),
    "pt_set_profiling": (_I, [_VP, _I]),
    "pt_set_tiled_kernels": (_I, [_VP, _I]),
    "pt_set_tma_staging": (_I, [_VP, _I]),
    "pt_set_propagate_lanes": (_I, [_VP, _I]),
    "pt_set_incremental": (_I, [_VP, _I]),
    "pt_get_frame_result": (_I, [_VP, _I, _VP, _VP]),
    "pt_get_frame_residual": (_I, [_VP, _I, _VP]),
    "pt_serve": (_I, [_I, _VP, _I, _I, ctypes.c_size_t]),
    "pt_server_create": (_I, [_I, _I, ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "pt_server_run": (_I, [_VP, _VP, _I]),
    "pt_server_destroy": (_I, [_VP]),
    "pt_measure_gather": (_I, [_I, _I, ctypes.POINTER(ctypes.c_double)]),
    "pt_host_alloc": (_I, [ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "pt_host_free": (_I, [_VP]),
    "pt_get_kernel_stats": (_I, [_VP, _I, ctypes.POINTER(_abi.KernelStats)]),
    "pt_piz_huffman_decode": (_I, [_VP, ctypes.c_size_t, _VP, ctypes.c_size_t]),
}


def lib():
    """The loaded library; raises if it is missing (no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libpainttween_gb300.so is not built; run `python -m painttween_gb300.build` "
                "(or __graft_entry__.build()) -- there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
