"""Many synthesis requests on one GPU, over pt_serve (include/painttween.h).

A request is a style exemplar plus one frame (a still) or several (a clip);
up to `max_in_flight` requests run at once, each on its own context and CUDA
stream, admitted in arrival order by arrival time and device-memory budget.
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import lib
from .synthesizer import PaintTweenError, host_array

_FRAME_KEYS = (("rgba", np.float32), ("orient_tensor", np.float32), ("dist_trans", np.float32),
               ("object_ids", np.int32), ("vel_fwd", np.float32), ("vel_bwd", np.float32), ("scale", np.float32))
_FRAME_FIELDS = ("rgba", "orient_tensor", "dist_trans", "ids", "vel_fwd", "vel_bwd", "scale")


def _build(requests, offsets, pinned=False):
    """The pt_request array of `requests` and the arrays it points to
    (results in page-locked memory when `pinned`)."""
    n = len(requests)
    arr = (_abi.Request * max(n, 1))()
    keep = []
    outs = []

    def ptr(a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a.ctypes.data

    for i, rq in enumerate(requests):
        p, st, frames = rq["params"], rq["style"], rq["frames"]
        h, w = frames[0]["rgba"].shape[:2]
        sh, sw = st["base"].shape[:2]
        fl = _abi.output_level(p)
        oh, ow = h >> fl, w >> fl
        alloc = host_array if pinned else np.empty
        out_rgba = alloc((len(frames), oh, ow, 4), np.float32)
        out_offs = alloc((len(frames), oh, ow), _abi.PATCH_DTYPE) if offsets else None
        fin = (_abi.FrameInputs * len(frames))()
        keep.append(fin)
        for f, fr in enumerate(frames):
            for (key, dt), field in zip(_FRAME_KEYS, _FRAME_FIELDS):
                setattr(fin[f], field, ptr(fr.get(key), dt))
        r = arr[i]
        r.params = p
        r.style_w, r.style_h = sw, sh
        r.style_base = ptr(st["base"], np.float32)
        r.style_output = ptr(st["output"], np.float32)
        r.style_orient_tensor = ptr(st.get("orient_tensor"), np.float32)
        r.style_dist_trans = ptr(st.get("dist_trans"), np.float32)
        r.style_ids = ptr(st.get("object_ids"), np.int32)
        r.image_w, r.image_h, r.frames = w, h, len(frames)
        r.inputs = ctypes.cast(fin, ctypes.POINTER(_abi.FrameInputs))
        r.out_rgba = out_rgba.ctypes.data
        r.out_offsets = out_offs.ctypes.data if out_offs is not None else None
        r.arrival_ms = float(rq.get("arrival_ms", 0.0))
        outs.append((out_rgba, out_offs))
    return arr, keep, outs


def _results(arr, outs, n, st):
    res = []
    for i in range(n):
        r = arr[i]
        res.append(dict(rgba=outs[i][0], offsets=outs[i][1], arrival_ms=r.arrival_ms, start_ms=r.start_ms,
                        done_ms=r.done_ms, latency_ms=r.done_ms - r.arrival_ms, status=r.status,
                        device_bytes=r.device_bytes))
    if st != _abi.PT_OK:
        bad = [i for i in range(n) if arr[i].status != _abi.PT_OK]
        raise PaintTweenError(st, "%d of %d requests failed (first: %s)" % (len(bad), n, bad[:1]))
    return res


def serve(requests, max_in_flight=8, hbm_budget=0, device=0, offsets=True, pinned=False):
    """Runs the requests (pt_serve); returns one dict per request with `rgba`
    (frames, h, w, 4), `offsets` (frames, h, w; PATCH_DTYPE, when asked for),
    `start_ms`, `done_ms`, `latency_ms` (done - arrival) and `status`.

    Each request is a dict: `params` (Params), `style` (dict with `base`,
    `output` and optionally `orient_tensor`, `dist_trans`, `object_ids`),
    `frames` (list of dicts with `rgba` and optionally `orient_tensor`,
    `dist_trans`, `object_ids`, `vel_fwd`, `vel_bwd`, `scale`) and optionally
    `arrival_ms`.  With `pinned` the results are written into page-locked
    memory (as are inputs given as host_array arrays), which the copies
    between host and GPU need to run at full speed beside other requests."""
    arr, keep, outs = _build(requests, offsets, pinned)
    st = lib().pt_serve(device, ctypes.cast(arr, ctypes.c_void_p), len(requests), max_in_flight, hbm_budget)
    return _results(arr, outs, len(requests), st)


class Server:
    """pt_server: worker contexts kept between runs (their buffers, memory
    caches and streams), so that later runs skip the set-up."""

    def __init__(self, max_in_flight=8, hbm_budget=0, device=0):
        h = ctypes.c_void_p()
        st = lib().pt_server_create(device, max_in_flight, hbm_budget, ctypes.byref(h))
        if st != _abi.PT_OK:
            raise PaintTweenError(st, "pt_server_create failed")
        self.h = h

    def run(self, requests, offsets=True, pinned=False):
        """As serve(), on this server's contexts."""
        arr, keep, outs = _build(requests, offsets, pinned)
        st = lib().pt_server_run(self.h, ctypes.cast(arr, ctypes.c_void_p), len(requests))
        return _results(arr, outs, len(requests), st)

    def close(self):
        if getattr(self, "h", None):
            lib().pt_server_destroy(self.h)
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
