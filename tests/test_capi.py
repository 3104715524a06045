"""CPU checks of the C ABI: the library loads, exports every symbol declared
in include/painttween.h, and its layouts match the Python description.  No
kernel is launched here."""
import ctypes
import os
import re

import pytest

from painttween_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "painttween.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pt_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ("pt_create", "pt_propagate", "pt_scatter", "pt_upsample", "pt_advect_offsets",
                 "pt_synthesize_frame", "pt_synthesize_animation"):
        assert name in syms


def test_library_exports_every_declared_symbol(gpu_lib):
    missing = [s for s in declared_symbols() if not hasattr(gpu_lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from painttween_gb300 import _lib
    missing = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not missing, missing


def test_layouts(gpu_lib):
    assert gpu_lib.pt_abi_version() == 1
    assert _abi.PATCH_DTYPE.itemsize == 36
    p = _abi.Params()
    gpu_lib.pt_default_params(ctypes.byref(p))
    q = _abi.default_params()
    for name, _ in _abi.Params._fields_:
        a, b = getattr(p, name), getattr(q, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name


def test_status_strings(gpu_lib):
    assert gpu_lib.pt_status_string(0) == b"PT_OK"
    assert gpu_lib.pt_status_string(7) == b"PT_ERR_BUDGET"


def test_create_without_device_reports_error(gpu_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    h = ctypes.c_void_p()
    st = gpu_lib.pt_create(0, 0, ctypes.byref(h))
    assert st == 2 and not h.value  # PT_ERR_CUDA, no context, no exit()
