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


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of pt_params, pt_frame_inputs and pt_request have
    the header's sizes and field offsets (checked by a C program compiled
    against include/painttween.h)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"pt_params": _abi.Params, "pt_frame_inputs": _abi.FrameInputs, "pt_request": _abi.Request}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "painttween.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)]).decode().splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
