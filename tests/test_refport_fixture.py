"""The oracle against the reference's own synthesis.

tests/golden/refport_small.npz holds the results of the reference's CUDA
kernels and TexSynth host wrappers (compiled unchanged, run on a GB300; see
make_refport_golden.py) on small seeded cases.  The oracle, which the CUDA
library equals bit for bit, is compared with them by the stated tolerance:
offset records identical, or differing with the same energy (residual)
within 1e-4 relative, and the stylised output's PSNR.  The reference is
compiled by nvcc with multiply-add contraction and evaluates sin and cos
with CUDA's library, where the oracle keeps one fixed operation order and
its own polynomials, so the two can round the last bit of an offset's
coordinates differently; such records are the equal-energy ones.
"""
import importlib.util
import json
import os

import numpy as np
import pytest

from _harness import agreement

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# agreement (identical + equal energy) and PSNR floors, per case
FLOORS = {"still64": (0.995, 60.0), "still56_terms": (0.995, 60.0), "clip48": (0.995, 60.0)}


def _cases():
    spec = importlib.util.spec_from_file_location("make_refport_golden", os.path.join(GOLDEN, "make_refport_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases()


@pytest.mark.parametrize("name", sorted(FLOORS))
def test_oracle_agrees_with_reference_kernels(name, oracle_mod):
    g = np.load(os.path.join(GOLDEN, "refport_small.npz"))
    manifest = json.loads(str(g["manifest"]))
    assert name in manifest["cases"]
    p, ex, clip, first, last = _cases()[name]
    res = oracle_mod.OracleDriver(p, [ex], clip, threads=4).render(first, last)
    agree_floor, psnr_floor = FLOORS[name]
    for f in range(first, last + 1):
        offs, resid, out = res[f]
        m = agreement(offs, resid, out, g["%s/offsets_%d" % (name, f)], g["%s/residual_%d" % (name, f)],
                      g["%s/output_%d" % (name, f)])
        assert m["agree"] >= agree_floor, (name, f, m)
        assert m["psnr_db"] >= psnr_floor, (name, f, m)


def test_energy_of_reference_offsets_matches_reference_residual(oracle_mod):
    """The oracle's patch distance, evaluated at the offsets the reference
    chose, reproduces the residual the reference stored (every term on:
    distance transform and object ids included), within 1e-5 relative."""
    from painttween_gb300 import _abi
    g = np.load(os.path.join(GOLDEN, "refport_small.npz"))
    for name in ("still64", "still56_terms"):
        p, ex, clip, first, last = _cases()[name]
        d = oracle_mod.OracleDriver(p, [ex], clip, threads=4)
        d.render(first, last)
        d.o.load_offsets(0, g["%s/offsets_0" % name])
        d.o.sync(0, _abi.DONT_COPY_OFFSETS)
        ref = g["%s/residual_0" % name].astype(np.float64)
        got = d.o.get_residual(0).astype(np.float64)
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6)
        assert rel.max() <= 1e-5, (name, rel.max())
        assert np.array_equal(d.o.get_output(0), g["%s/output_0" % name]), name
