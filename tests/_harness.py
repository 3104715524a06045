"""Shared set-up for the parity tests: the same pyramid-level data is handed
to the CPU oracle and to the CUDA library through its C ABI."""
import numpy as np

from oracle import oracle as O
from painttween_gb300 import TexSynth, _abi, synthetic


def patch_bytes(a):
    return np.ascontiguousarray(a).view(np.uint8).reshape(a.shape + (36,))


def identical_fraction(a, b):
    return float((patch_bytes(a) == patch_bytes(b)).all(-1).mean())


def assert_offsets_equal(gpu, ref, min_fraction=1.0, what="offsets"):
    frac = identical_fraction(gpu, ref)
    if frac < min_fraction:
        bad = np.argwhere(~(patch_bytes(gpu) == patch_bytes(ref)).all(-1))
        y, x = bad[0]
        raise AssertionError("%s identical on %.5f of pixels (< %.5f); first at (%d,%d): gpu %s ref %s" % (
            what, frac, min_fraction, x, y, gpu[y, x], ref[y, x]))
    return frac


def assert_array_equal(gpu, ref, what):
    g = np.ascontiguousarray(gpu)
    r = np.ascontiguousarray(ref)
    same = (g.view(np.uint32) == r.view(np.uint32)) | (np.isnan(g) & np.isnan(r))
    if not same.all():
        idx = np.argwhere(~same)[0]
        raise AssertionError("%s differs on %d of %d values; first at %s: gpu %r ref %r" % (
            what, (~same).sum(), same.size, tuple(idx), g[tuple(idx)], r[tuple(idx)]))


class Pair:
    """The oracle and the GPU library holding the same state."""

    def __init__(self, W, H, EW, EH, params, threads=8, seed=1, discs=3, frames=1, style=None, clip=None):
        self.W, self.H, self.EW, self.EH = W, H, EW, EH
        self.p = params.copy()
        ex = style if style is not None else synthetic.make_exemplar(EW, EH, seed=seed)
        self.ex = ex
        self.clip = clip if clip is not None else synthetic.make_clip(W, H, discs, frames, seed=seed + 100)
        self.sp = O.style_pyramids(ex)
        self.fps = [O.frame_pyramids(f) for f in self.clip]
        self.o = O.Oracle(W, H, EW, EH, 1, threads=threads)
        self.g = TexSynth(device=0)
        self.g.initialize(W, H, EW, EH, 1)
        self.set_params(self.p)

    def close(self):
        self.g.close()
        self.o.close()

    def set_params(self, p):
        self.p = p.copy()
        self.o.set_params(p)
        self.g.set_params(p)

    def load_style(self, level):
        self.o.load_style_level([self.sp], level)
        s = self.sp
        ew, eh = self.EW >> level, self.EH >> level
        g = self.g
        g.initialize_exemplars(ew, eh, 1)
        g.upload_image_color4(level, _abi.LAYER_EXEMPLAR_BASE, s["base"][level], 0)
        g.upload_image_color4(level, _abi.LAYER_EXEMPLAR_OUTPUT, s["output"][level], 0)
        g.upload_image_float(level, _abi.LAYER_EXEMPLAR_ORIENTATION, s["orient"][level], 0)
        g.upload_image_float(level, _abi.LAYER_EXEMPLAR_DIST_TRANS, s["dt"][level], 0)
        g.upload_image_int(level, _abi.LAYER_EXEMPLAR_OBJECT_IDS, s["ids"][level], 0)

    def load_frame(self, f, level):
        fp = self.fps[f]
        self.o.load_frame_level(fp, level)
        g = self.g
        g.upload_image_color4(level, _abi.LAYER_INPUT_COLOR, fp["rgba"][level])
        g.upload_image_float(level, _abi.LAYER_INPUT_ORIENTATION, fp["orient"][level])
        g.upload_image_int(level, _abi.LAYER_INPUT_ID, fp["ids"][level])
        g.upload_image_float2(level, _abi.LAYER_INPUT_VEL_B, fp["velb"][level])
        g.upload_image_float2(level, _abi.LAYER_INPUT_VEL_F, fp["velf"][level])
        g.upload_image_float(level, _abi.LAYER_INPUT_DIST_TRANS, fp["dt"][level])
        g.upload_image_float2(level, _abi.LAYER_INPUT_SCALE, fp["scale"][level])

    def random_level(self, f, level):
        fp = self.fps[f]
        rnd = O.random_level(f * level, level, self.EW, self.EH, fp["rgba"][level], fp["orient"][level],
                             self.sp["output"][level], self.sp["orient"][level],
                             bool(self.p.transparencyOk), bool(self.p.orientationEnabled))
        self.o.upload_random(rnd)
        self.g.create_random_level(level, f)

    def flip(self):
        self.o.flip()
        self.g.flip_anim_buffers()

    def both(self, name, *args):
        getattr(self.o, {"randomize_offsets": "randomize_offsets", "propagate": "propagate", "scatter": "scatter",
                         "upsample": "upsample", "sync": "sync", "update_residual": "update_residual",
                         "merge_randomly": "merge_randomly", "merge_using_residual": "merge_using_residual",
                         "advect": "advect", "reset_advected": "reset_advected"}[name])(*args)
        gname = {"sync": "sync_buffers", "update_residual": "update_residual_cache", "advect": "advect_offsets",
                 "reset_advected": "reset_advected_buffers"}.get(name, name)
        getattr(self.g, gname)(*args)

    def compare(self, level, what="", offsets_min=1.0, residual=True, output=True):
        frac = assert_offsets_equal(self.g.get_offsets(level), self.o.get_offsets(level), offsets_min,
                                    "offsets " + what)
        if residual:
            assert_array_equal(self.g.get_residual(level), self.o.get_residual(level), "residual " + what)
        if output:
            assert_array_equal(self.g.get_output(level), self.o.get_output(level), "output " + what)
        return frac


def config_params(r=2, levels=3, iterations=2, filter_mode=None):
    p = _abi.default_params()
    p.residualWindowSize, p.levels, p.iterations = r, levels, iterations
    if filter_mode is not None:
        p.filterMode = filter_mode
    return p


# both sampling arithmetics: the texture unit's (the default) and exact FP32
FILTER_MODES = [_abi.FILTER_TEXTURE, _abi.FILTER_EXACT]


def agreement(offs, res, out, ref_offs, ref_res, ref_out, energy_tol=1e-4):
    """Agreement of a synthesis with the reference's by the stated tolerance:
    the fraction of pixels whose offset record is identical, the fraction
    whose record differs but whose energy (stored residual) is equal within
    `energy_tol` relative, their sum, and the PSNR of the stylised output
    (peak 1)."""
    same = (patch_bytes(offs) == patch_bytes(ref_offs)).all(-1)
    a = np.asarray(res, np.float64)
    b = np.asarray(ref_res, np.float64)
    close = np.abs(a - b) <= energy_tol * np.maximum(np.abs(a), np.abs(b)) + 1e-12
    close |= (np.isnan(a) & np.isnan(b))
    equal_energy = (~same) & close
    mse = float(np.mean((np.asarray(out, np.float64) - np.asarray(ref_out, np.float64)) ** 2))
    return {"identical": float(same.mean()), "equal_energy": float(equal_energy.mean()),
            "agree": float((same | equal_energy).mean()),
            "psnr_db": float(10 * np.log10(1.0 / max(mse, 1e-20)))}
