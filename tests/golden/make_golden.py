"""Writes the committed fixtures of tests/golden.

glibc_rand.npz: the C library's own rand() output after srand(seed) for the
seeds createRandomPyramid uses (frame * level) -- produced by libc itself,
not by the restatement.
still48.npz: the oracle's result for a 48x48 still (r2, 3 levels, 2
iterations), a regression lock of the oracle.  These three locks use exact
FP32 bilinear filtering (PT_FILTER_EXACT); the texture-unit filtering is
pinned by texfilter_gb300.npz (make_texfilter.py).
clip40.npz: the oracle's results for a 40x32 three-frame clip with moving
discs (48x48 exemplar, r2, 2 levels, 2 iterations, temporal coherence 0.5)
under the FMBM_RM, FBMO and TCTF schedules, a regression lock of the
temporal paths.
keys32.npz: the oracle's results for a 32x24 four-frame clip interpolating
keyframes 1 and 3 (FMBM_RM, r2, 2 levels, 2 iterations; part of the first
key left unpainted), a regression lock of the keyframe path.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    libc = ctypes.CDLL("libc.so.6")
    vec = {}
    for seed in (0, 1, 2, 4, 6, 12, 23, 46, 69, 92):
        libc.srand(seed)
        vec["seed_%d" % seed] = np.array([libc.rand() for _ in range(512)], np.int32)
    np.savez_compressed(os.path.join(HERE, "glibc_rand.npz"), **vec)

    from oracle import oracle as O
    from painttween_gb300 import _abi, synthetic
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 3, 2
    p.filterMode = _abi.FILTER_EXACT
    ex = synthetic.make_exemplar(48, 48, seed=101)
    fr = synthetic.make_still(48, 48, 3, seed=102)
    offs, res, out = O.OracleDriver(p, [ex], [fr], threads=4).render(0, 0)[0]
    np.savez_compressed(os.path.join(HERE, "still48.npz"), offsets=offs, residual=res, output=out,
                        ex_seed=101, fr_seed=102)

    arrays = {}
    for name, scheme in CLIP_SCHEMES:
        results = render_clip(scheme)
        for f in range(3):
            offs, res, out = results[f]
            arrays["%s_offsets_%d" % (name, f)] = offs
            arrays["%s_output_%d" % (name, f)] = out
    np.savez_compressed(os.path.join(HERE, "clip40.npz"), **arrays)

    results = render_keyed()
    np.savez_compressed(os.path.join(HERE, "keys32.npz"),
                        **{"%s_%d" % (k, f): results[f][i] for f in range(4) for i, k in ((0, "offsets"), (2, "output"))})


def render_keyed():
    """The keys32 case: 32x24, 4 frames, keys 1 and 3, FMBM_RM, r2, 2 levels,
    2 iterations; the left third of the first key's output is transparent."""
    from oracle import oracle as O
    from painttween_gb300 import _abi, synthetic
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 2, 2
    p.filterMode = _abi.FILTER_EXACT
    p.scheme = _abi.S_FMBM_RM
    p.interpolateKeyFrame = 1
    p.numStyles = 2
    styles = [synthetic.make_exemplar(32, 24, seed=120 + i) for i in range(2)]
    out = styles[0]["output"].copy()
    out[:, : 32 // 3, 3] = 0.0
    styles[0]["output"] = out
    clip = synthetic.make_clip(32, 24, 3, 4, seed=122)
    d = O.OracleDriver(p, styles, clip, threads=4)
    d.set_keyframes([1, 3])
    return d.render(0, 3)


CLIP_SCHEMES = (("fmbm_rm", 1), ("fbmo", 2), ("tctf", 3))


def render_clip(scheme):
    """The clip40 case: 40x32, 3 frames, 48x48 exemplar, r2, 2 levels,
    2 iterations, temporal coherence 0.5, the given scheme."""
    from oracle import oracle as O
    from painttween_gb300 import _abi, synthetic
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = 2, 2, 2
    p.filterMode = _abi.FILTER_EXACT
    p.temporalCoherenceWeight = 0.5
    p.scheme = scheme
    ex = synthetic.make_exemplar(48, 48, seed=111)
    clip = synthetic.make_clip(40, 32, 3, 3, seed=112)
    return O.OracleDriver(p, [ex], clip, threads=4).render(0, 2)


if __name__ == "__main__":
    main()
