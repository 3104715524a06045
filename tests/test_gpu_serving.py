"""pt_serve: many requests of uneven size on one GPU.

Each request runs on its own context and stream; the results must be the
same alone and in a concurrent mix, and equal to the plain single-request
path.  Arrival times and the device-memory budget gate admission.
"""
import numpy as np
import pytest

from painttween_gb300 import Synthesizer, _abi, synthetic
from painttween_gb300.serving import serve

from _harness import assert_array_equal, assert_offsets_equal, config_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def _still(w, h, ew, seed, r=2, levels=3, iterations=2):
    p = config_params(r=r, levels=levels, iterations=iterations)
    ex = synthetic.make_exemplar(ew, ew, seed=seed)
    fr = synthetic.make_still(w, h, 3, seed=seed + 1)
    return dict(params=p, style=ex, frames=[fr])


def _clip(w, h, ew, n, seed):
    p = config_params(r=2, levels=2, iterations=2)
    p.temporalCoherenceWeight = 0.5
    ex = synthetic.make_exemplar(ew, ew, seed=seed)
    return dict(params=p, style=ex, frames=synthetic.make_clip(w, h, 3, n, seed=seed + 1))


def _mix():
    return [_still(96, 80, 64, 11), _still(128, 128, 128, 12), _still(64, 96, 64, 13, r=3),
            _clip(72, 56, 64, 3, 14), _still(200, 136, 128, 15, r=3, levels=4), _still(160, 120, 64, 16)]


def test_results_same_alone_and_in_mix():
    reqs = _mix()
    alone = [serve([r], max_in_flight=1)[0] for r in reqs]
    mixed = serve(reqs, max_in_flight=4)
    for i, (a, m) in enumerate(zip(alone, mixed)):
        assert a["status"] == 0 and m["status"] == 0
        for f in range(a["rgba"].shape[0]):
            assert_offsets_equal(m["offsets"][f], a["offsets"][f], 1.0, "request %d frame %d" % (i, f))
            assert_array_equal(m["rgba"][f], a["rgba"][f], "request %d frame %d output" % (i, f))


def test_served_still_equals_plain_path():
    rq = _still(128, 96, 64, 21)
    got = serve([rq, _still(96, 64, 64, 22)], max_in_flight=2)[0]
    s = Synthesizer(device=0)
    try:
        s.setup(rq["params"], 128, 96, 64, 64, 1)
        ex = rq["style"]
        s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
        s.set_frame_dict(0, rq["frames"][0])
        rgba, offs = s.synthesize_frame(0)
    finally:
        s.close()
    assert_offsets_equal(got["offsets"][0], offs, 1.0, "served still vs plain path")
    assert_array_equal(got["rgba"][0], rgba, "served still output vs plain path")


def test_arrivals_and_budget_admission():
    reqs = [_still(96, 80, 64, 31 + i) for i in range(4)]
    for i, r in enumerate(reqs):
        r["arrival_ms"] = 40.0 * i
    res = serve(reqs, max_in_flight=4)
    for r, q in zip(res, reqs):
        assert r["start_ms"] >= q["arrival_ms"]
        assert r["done_ms"] >= r["start_ms"]
    # a budget that holds one request at a time: no two runs overlap
    res = serve([_still(96, 80, 64, 41 + i) for i in range(4)], max_in_flight=4, hbm_budget=1)
    spans = sorted((r["start_ms"], r["done_ms"]) for r in res)
    for (s0, d0), (s1, d1) in zip(spans, spans[1:]):
        assert s1 >= d0
    # the memory each request's context held once set up is reported
    assert all(r["device_bytes"] > 0 for r in res)


def test_admission_counts_the_memory_contexts_hold():
    """After set-up the budget counts what a context actually holds: a
    budget a little above one request's memory lets no two of them run at
    once, whatever the estimate from their sizes says."""
    big = [_still(320, 320, 256, 51 + i) for i in range(3)]
    alone = serve([big[0]], max_in_flight=1)[0]["device_bytes"]
    res = serve(big, max_in_flight=3, hbm_budget=int(1.1 * alone))
    spans = sorted((r["start_ms"], r["done_ms"]) for r in res)
    for (s0, d0), (s1, d1) in zip(spans, spans[1:]):
        assert s1 >= d0


def test_reused_texture_arrays_match_the_oracle():
    """A worker keeps its texture arrays: a small exemplar after a larger one
    is fetched from the corner of the larger arrays, with the coordinates
    clamped, and must give the oracle's clamp-addressing results bit for bit."""
    from oracle import oracle as O
    from painttween_gb300.serving import Server
    small = _still(96, 80, 64, 61, levels=3, iterations=3)
    small["params"].filterMode = _abi.FILTER_TEXTURE
    big = _still(128, 96, 200, 62)
    with Server(max_in_flight=1) as srv:
        got = srv.run([dict(big, arrival_ms=0.0), dict(small, arrival_ms=1.0)])[1]
    ref = O.OracleDriver(small["params"], [small["style"]], small["frames"], threads=8).render(0, 0)[0]
    assert_offsets_equal(got["offsets"][0], ref[0], 1.0, "still after a larger exemplar")
    assert np.abs(got["rgba"][0] - ref[2]).max() <= 1e-6


def test_server_keeps_contexts_between_runs():
    from painttween_gb300.serving import Server
    reqs = _mix()
    ref = serve(reqs, max_in_flight=3)
    with Server(max_in_flight=3) as srv:
        for run in range(2):
            got = srv.run(reqs)
            for i, (a, m) in enumerate(zip(ref, got)):
                for f in range(a["rgba"].shape[0]):
                    assert_offsets_equal(m["offsets"][f], a["offsets"][f], 1.0, "run %d request %d" % (run, i))
                    assert_array_equal(m["rgba"][f], a["rgba"][f], "run %d request %d output" % (run, i))
