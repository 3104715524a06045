"""The allocation-free separable Gaussian (pt_convolve_separable_noalloc).

Callers that cannot allocate device memory when they call the library (a
plugin host owning all device memory, a process whose memory another
framework's allocator holds) use this entry point: the row-pass intermediate
lives in a fixed array in the library's device memory instead of a context
scratch buffer.  Its output must equal that of the allocating entry point,
pt_convolve_separable, on consecutive calls (the array keeps the previous
call's contents).  This file is collected last so that a failure here stops
a -x run only after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _blur_allocating(torch, src, w, h, pitch, radius):
    from painttween_gb300 import TexSynth
    dst = torch.zeros_like(src)
    t = TexSynth(device=0)
    try:
        t.convolve_separable(src.data_ptr(), dst.data_ptr(), w, h, pitch, radius)
        t.synchronize()
    finally:
        t.close()
    return dst


def test_noalloc_blur_matches_allocating_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    # consecutive calls share the device array: the second, smaller call
    # leaves the first call's values in the array outside its own rectangle,
    # and the third fills the array exactly (pitch * h == PT_NOALLOC_MAX_PIXELS)
    shapes = [(300, 257, 320, 3), (150, 100, 160, 2), (1024, 1024, 1024, 4)]
    for call, (w, h, pitch, radius) in enumerate(shapes):
        img = rng.uniform(-2, 9, (h, pitch)).astype(np.float32)
        src = torch.from_numpy(img).cuda()
        dst = torch.full_like(src, float("nan"))
        torch.cuda.synchronize()
        st = gpu_lib.pt_convolve_separable_noalloc(ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                                   w, h, pitch, radius, None)
        assert st == 0, (call, st)
        torch.cuda.synchronize()
        ref = _blur_allocating(torch, src, w, h, pitch, radius)
        got = dst.cpu().numpy()[:, :w]
        exp = ref.cpu().numpy()[:, :w]
        assert np.isfinite(got).all(), "call %d left unwritten pixels" % call
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32)), "call %d differs" % call


def test_noalloc_blur_rejects_sizes_beyond_its_array(gpu_lib):
    torch = pytest.importorskip("torch")
    src = torch.zeros(4, device="cuda")
    # 2048 x 1024 floats exceed the fixed 1 Mi-float intermediate
    st = gpu_lib.pt_convolve_separable_noalloc(ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                                               2048, 1024, 2048, 3, None)
    assert st == 1  # PT_ERR_INVALID, nothing launched
