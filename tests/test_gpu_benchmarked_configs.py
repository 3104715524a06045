"""The benchmarked configurations against the oracle, bit for bit.

The other parity tests use small images; here the library runs the
configurations the benchmark and the scaling runs use, cut in length: four
frames of the 512x512 animation (r2, 4 levels, 4 iterations, temporal
coherence 0.5, FMBM_RM forward and backward), and two frames of the
1920x1080 clip at full size (1024x1024 exemplar, r3, 5 levels, histogram
term on, FMBM_RM forward and backward) with 2 of its 6 iterations per level
-- grids of thousands of blocks, the largest levels, the early exit, the
change tracking and the tap queues at their real sizes.  The oracle runs on
every host thread; these are the slowest tests of the suite (the 1080p cut
at all 6 iterations takes the oracle about 11 minutes on 16 cores).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from painttween_gb300 import Synthesizer, synthetic

from _harness import assert_array_equal, assert_offsets_equal

pytestmark = pytest.mark.gpu


def _both(cfg, frames, seed):
    p = cfg["params"]
    ex = synthetic.make_exemplar(cfg["ew"], cfg["eh"], seed=seed)
    clip = synthetic.make_clip(cfg["w"], cfg["h"], cfg["discs"], frames, seed=seed + 1)
    s = Synthesizer(device=0)
    try:
        s.setup(p, cfg["w"], cfg["h"], cfg["ew"], cfg["eh"], 1)
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        for i, fr in enumerate(clip):
            s.set_frame_dict(i, fr)
        got = s.synthesize_animation(0, frames - 1)
        res = {f: s.get_frame_residual(f) for f in got}
    finally:
        s.close()
    ref = O.OracleDriver(p, [ex], clip, threads=os.cpu_count() or 8).render(0, frames - 1)
    for f in range(frames):
        assert_offsets_equal(got[f][1], ref[f][0], 1.0, "frame %d offsets" % f)
        assert_array_equal(res[f], ref[f][1], "frame %d residual" % f)
        assert_array_equal(got[f][0], ref[f][2], "frame %d output" % f)


def test_anim512_four_frame_cut_matches_oracle(gpu_lib):
    _both(synthetic.config("anim512"), 4, seed=512)


def test_clip1080p_two_frame_cut_matches_oracle(gpu_lib):
    cfg = synthetic.config("clip1080p")
    cfg["params"].iterations = 2
    _both(cfg, 2, seed=2026)
