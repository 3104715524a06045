"""Seeded synthetic working sets with the shapes of the benchmark configs.

No public dataset stands behind the benchmark; these generators produce
inputs with the stated shapes, sizes and value distributions:

* style exemplar: RGBA float32, the sum of 8 oriented sinusoidal stroke
  layers (random angle, period 6-20 px, amplitude 0.1-0.3, per-layer RGB tint)
  plus N(0, 0.05^2) noise, offset by 0.5 and clamped to [0, 1], alpha 1.  The
  exemplar "base" (style input) is the output's luminance broadcast to RGB.
  Orientation is the structure tensor (cos^2, cos sin, sin^2) of the locally
  dominant stroke layer; object IDs are that layer's index mod 4; DT is 0.
* frame: grey (0.5) background with flat-shaded random discs (radius
  0.08-0.25 of min(W, H)), alpha 1; orientation tensor from central-difference
  luminance gradients; exact Euclidean distance transform to the disc edges;
  IDs 0 (background) and 1 + (k mod 3) for disc k; scale (1, 1).
* motion: each disc rotates by up to 2 degrees and translates by up to 4 px
  per frame; forward/backward velocities are the analytic per-pixel
  displacement of the owning disc to the next/previous frame.
"""
import math

import numpy as np

try:
    from scipy import ndimage as _ndi
except Exception:  # pragma: no cover - scipy is present in both images
    _ndi = None


def make_exemplar(w, h, seed, layers=8):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    acc = np.zeros((h, w, 3))
    best_amp = np.full((h, w), -1.0)
    dom = np.zeros((h, w), np.int32)
    dom_phi = np.zeros((h, w))
    for k in range(layers):
        phi = rng.uniform(0.0, math.pi)
        period = rng.uniform(6.0, 20.0)
        amp = rng.uniform(0.1, 0.3)
        psi = rng.uniform(0.0, 2 * math.pi)
        tint = rng.uniform(0.4, 1.0, size=3)
        s = amp * np.sin(2 * math.pi * (xx * math.cos(phi) + yy * math.sin(phi)) / period + psi)
        acc += s[..., None] * tint[None, None, :] / 2.0
        mag = np.abs(s)
        sel = mag > best_amp
        best_amp[sel] = mag[sel]
        dom[sel] = k
        dom_phi[sel] = phi
    acc += rng.normal(0.0, 0.05, size=acc.shape)
    rgb = np.clip(acc + 0.5, 0.0, 1.0)
    out = np.ones((h, w, 4), np.float32)
    out[..., :3] = rgb
    lum = 0.2126 * rgb[..., 0] + 0.7152 * rgb[..., 1] + 0.0722 * rgb[..., 2]
    base = np.ones((h, w, 4), np.float32)
    base[..., 0] = base[..., 1] = base[..., 2] = lum
    c, s = np.cos(dom_phi), np.sin(dom_phi)
    tensor = np.stack([c * c, c * s, s * s], axis=-1).astype(np.float32)
    ids = (dom % 4).astype(np.int32)
    dt = np.zeros((h, w), np.float32)
    return dict(base=base, output=out, orient_tensor=tensor, dist_trans=dt,
                object_ids=ids, w=w, h=h)


def _disc_params(w, h, n, rng):
    m = min(w, h)
    discs = []
    for k in range(n):
        discs.append(dict(
            cx=rng.uniform(0.1 * w, 0.9 * w), cy=rng.uniform(0.1 * h, 0.9 * h),
            r=rng.uniform(0.08, 0.25) * m,
            color=rng.uniform(0.0, 1.0, size=3),
            rot=math.radians(rng.uniform(-2.0, 2.0)),
            tx=rng.uniform(-4.0, 4.0), ty=rng.uniform(-4.0, 4.0),
            ident=1 + (k % 3)))
    return discs


def _render(w, h, discs, t):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    owner = np.full((h, w), -1, np.int32)
    for k, d in enumerate(discs):
        cx, cy = d["cx"] + t * d["tx"], d["cy"] + t * d["ty"]
        inside = (xx - cx) ** 2 + (yy - cy) ** 2 <= d["r"] ** 2
        owner[inside] = k
    return owner, xx, yy


def _edt_to_edges(owner):
    edge = np.zeros(owner.shape, bool)
    edge[:, 1:] |= owner[:, 1:] != owner[:, :-1]
    edge[:, :-1] |= owner[:, 1:] != owner[:, :-1]
    edge[1:, :] |= owner[1:, :] != owner[:-1, :]
    edge[:-1, :] |= owner[1:, :] != owner[:-1, :]
    if not edge.any():
        return np.full(owner.shape, 1e4, np.float32)
    if _ndi is not None:
        return _ndi.distance_transform_edt(~edge).astype(np.float32)
    ys, xs = np.nonzero(edge)  # small fallback for tests without scipy
    yy, xx = np.mgrid[0:owner.shape[0], 0:owner.shape[1]]
    d = np.full(owner.shape, np.inf)
    for y0, x0 in zip(ys, xs):
        d = np.minimum(d, np.hypot(yy - y0, xx - x0))
    return d.astype(np.float32)


def make_clip(w, h, n_discs, n_frames, seed):
    """Frames of discs with analytic velocities; returns a list of dicts."""
    rng = np.random.default_rng(seed)
    discs = _disc_params(w, h, n_discs, rng)
    frames = []
    for f in range(n_frames):
        owner, xx, yy = _render(w, h, discs, f)
        rgba = np.empty((h, w, 4), np.float32)
        rgba[..., :3] = 0.5
        rgba[..., 3] = 1.0
        ids = np.zeros((h, w), np.int32)
        vf = np.zeros((h, w, 2), np.float32)
        vb = np.zeros((h, w, 2), np.float32)
        for k, d in enumerate(discs):
            sel = owner == k
            if not sel.any():
                continue
            rgba[sel, :3] = d["color"]
            ids[sel] = d["ident"]
            cx, cy = d["cx"] + f * d["tx"], d["cy"] + f * d["ty"]
            px, py = xx[sel] - cx, yy[sel] - cy
            ca, sa = math.cos(d["rot"]), math.sin(d["rot"])
            vf[sel, 0] = (ca * px - sa * py) + cx + d["tx"] - xx[sel]
            vf[sel, 1] = (sa * px + ca * py) + cy + d["ty"] - yy[sel]
            vb[sel, 0] = (ca * px + sa * py) + cx - d["tx"] - xx[sel]
            vb[sel, 1] = (-sa * px + ca * py) + cy - d["ty"] - yy[sel]
        lum = 0.2126 * rgba[..., 0] + 0.7152 * rgba[..., 1] + 0.0722 * rgba[..., 2]
        gx = np.zeros_like(lum)
        gy = np.zeros_like(lum)
        gx[:, 1:-1] = 0.5 * (lum[:, 2:] - lum[:, :-2])
        gy[1:-1, :] = 0.5 * (lum[2:, :] - lum[:-2, :])
        tensor = np.stack([gx * gx, gx * gy, gy * gy], axis=-1).astype(np.float32)
        dt = _edt_to_edges(owner)
        scale = np.ones((h, w, 2), np.float32)
        frames.append(dict(rgba=rgba, orient_tensor=tensor, dist_trans=dt,
                           object_ids=ids, vel_fwd=vf, vel_bwd=vb, scale=scale,
                           w=w, h=h))
    return frames


def make_still(w, h, n_discs, seed):
    return make_clip(w, h, n_discs, 1, seed)[0]


# --- the benchmark configurations ------------------------------------------

def config(name):
    """Synthesis parameters and input shapes of the named configuration."""
    from . import _abi
    p = _abi.default_params()
    if name == "still256":       # 256x256 still, 256x256 exemplar
        p.residualWindowSize, p.levels, p.iterations = 2, 3, 4
        return dict(params=p, w=256, h=256, ew=256, eh=256, discs=3, frames=1)
    if name == "anim512":        # 60 frames of 512x512, 512x512 exemplar
        p.residualWindowSize, p.levels, p.iterations = 2, 4, 4
        p.temporalCoherenceWeight = 0.5
        return dict(params=p, w=512, h=512, ew=512, eh=512, discs=3, frames=60)
    if name == "clip1080p":      # 24 frames of 1920x1080, 1024x1024 exemplar
        p.residualWindowSize, p.levels, p.iterations = 3, 5, 6
        p.offsetsHistogramSlope[0] = 1.0
        p.offsetsHistogramThreshold[0] = 0.0
        return dict(params=p, w=1920, h=1080, ew=1024, eh=1024, discs=6, frames=24)
    raise KeyError(name)
