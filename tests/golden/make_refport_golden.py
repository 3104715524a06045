"""Writes tests/golden/refport_small.npz: the reference's own synthesis --
its CUDA kernels and TexSynth host wrappers (src/PaintTweenCUDA/
texSynth_kernel.cu, convolution.cu), compiled unchanged by
oracle/refport/build.py -- on small seeded cases, recorded on a GB300.  The
tests compare the oracle (tests/test_refport_fixture.py) and the CUDA
library (tests/test_gpu_refport.py) with it by the stated tolerances.

Run on a machine with the GPU and the staged port (oracle/_ref/refport_src,
copied from the reference tree by oracle/refport/build.py):
    python tests/golden/make_refport_golden.py
The driver is the oracle's restatement of the reference's per-frame driver
(renderAnimation*, synthesizeConsecutive, propagateAndScatter) over the
port's TexSynth calls; the host-side steps (random-offset pyramid from glibc
rand(), image pyramids, the half-precision residual file) come from the
oracle's pinned restatements.
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cases():
    """name -> (params, exemplar, clip, first, last); shared with the tests."""
    from painttween_gb300 import _abi, synthetic
    out = {}
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 3, 3
    out["still64"] = (p, synthetic.make_exemplar(64, 64, seed=701), synthetic.make_clip(64, 64, 3, 1, seed=702), 0, 0)
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 3, 2, 2
    p.distTransWeight, p.styleObjIdWeight = 1.0, 1.0
    out["still56_terms"] = (p, synthetic.make_exemplar(64, 64, seed=711), synthetic.make_clip(56, 48, 4, 1, seed=712),
                            0, 0)
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 2, 2
    p.temporalCoherenceWeight = 0.5
    p.scheme = _abi.S_FMBM_RM
    out["clip48"] = (p, synthetic.make_exemplar(48, 48, seed=721), synthetic.make_clip(48, 40, 3, 3, seed=722), 0, 2)
    return out


def main():
    from oracle.refport import build as rb
    from oracle.refport import port as RP
    if rb.build() is None:
        raise SystemExit("reference port not staged")
    arrays = {}
    manifest = {"cases": {}}
    for name, (p, ex, clip, first, last) in cases().items():
        d = RP.RefPortDriver(p, [ex], clip)
        res = d.render(first, last)
        d.o.close()
        for f, (offs, resid, outp) in res.items():
            arrays["%s/offsets_%d" % (name, f)] = offs
            arrays["%s/residual_%d" % (name, f)] = resid
            arrays["%s/output_%d" % (name, f)] = outp
        manifest["cases"][name] = {"frames": [first, last], "size": [clip[0]["w"], clip[0]["h"]],
                                   "exemplar": [ex["w"], ex["h"]], "r": p.residualWindowSize, "levels": p.levels,
                                   "iterations": p.iterations, "scheme": p.scheme}
    h = hashlib.sha256()
    for f in rb.REF_FILES:
        h.update(open(os.path.join(rb.STAGE, f), "rb").read())
    for f in rb.SHIMS:
        h.update(open(os.path.join(rb.HERE, f), "rb").read())
    manifest["port_sources_sha256"] = h.hexdigest()
    manifest["gpu"] = subprocess.run(["nvidia-smi", "--query-gpu=name,driver_version", "--format=csv,noheader"],
                                     capture_output=True, text=True).stdout.strip()
    arrays["manifest"] = np.array(json.dumps(manifest))
    np.savez_compressed(os.path.join(HERE, "refport_small.npz"), **arrays)
    print("wrote refport_small.npz:", ", ".join(manifest["cases"]))


if __name__ == "__main__":
    main()
