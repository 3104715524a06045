// pt_kernels.cu -- sm_103a kernels of the offset-field synthesis.
//
// Each kernel restates one kernel of the reference
// (src/PaintTweenCUDA/texSynth_kernel.cu, convolution.cu) or one host-side
// pyramid step (downsample.cpp, synthesisFrame.cpp:66-150) with the same
// per-pixel semantics, over the buffer model described in pt_device.cuh.
#include "pt_common.cuh"
#include "pt_device.cuh"
#include "pt_internal.h"

namespace ptk {

// ---------------------------------------------------------------------------
// energy (calculateResidual and its terms, texSynth_kernel.cu:377-721)
// ---------------------------------------------------------------------------

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

#define PIXEL_XY                                        \
    const int x = blockIdx.x * blockDim.x + threadIdx.x; \
    const int y = blockIdx.y * blockDim.y + threadIdx.y; \
    if (!in_rect(P, x, y)) return;                      \
    const size_t k = (size_t)y * P.W + x;

// propagate_kernel, :1112-1219 (advected candidates are dead code, :981)
// With key >= 0, a pixel under the key's mask takes the key (:1137-1142).
__global__ void __launch_bounds__(128) k_propagate(const Params P, PatchPlanes work, int jump, int key) {
    PIXEL_XY
    if (image_culled(P, x, y)) {
        store_patch(work, k, make_patch(0, 0, 0, 0, 0, 1.f, 1.f));
        return;
    }
    if (keymask_alpha(P.ex, x, y, key) > 0.0f) {
        store_patch(work, k, make_patch((float)x, (float)y, 0.f, 1.f, key, 1.f, 1.f));
        return;
    }
    float best = __ldg(P.res + k);
    float ia = lay_texel(P.img.base[P.img.cur], P, x, y).w;
    Patch ow = load_patch(P.off, k);
    PixCtx pc;
    make_pixctx(P, x, y, &pc);
    // an exact repeat of an earlier candidate has the same energy and is
    // rejected by the strict "<" test: it is not evaluated again
    uint32_t s0x = 0, s0y = 0, s0t = 0, s1x = 0, s1y = 0, s1t = 0, s2x = 0, s2y = 0, s2t = 0;
    int s0l = -1, s1l = -1, s2l = -1;
#pragma unroll 1
    for (int c = 0; c < 4; c++) {
        int tx = x, ty = y;
        if (c == 0) tx = x + jump;
        else if (c == 1) tx = x - jump;
        else if (c == 2) ty = y + jump;
        else ty = y - jump;
        Patch t = propagate_offset(P, tx, ty, x, y);
        uint32_t kx = __float_as_uint(t.x), ky = __float_as_uint(t.y), kt = __float_as_uint(t.theta);
        bool dup = (c > 0 && kx == s0x && ky == s0y && kt == s0t && t.layer == s0l) ||
                   (c > 1 && kx == s1x && ky == s1y && kt == s1t && t.layer == s1l) ||
                   (c > 2 && kx == s2x && ky == s2y && kt == s2t && t.layer == s2l);
        if (c == 0) { s0x = kx; s0y = ky; s0t = kt; s0l = t.layer; }
        else if (c == 1) { s1x = kx; s1y = ky; s1t = kt; s1l = t.layer; }
        else if (c == 2) { s2x = kx; s2y = ky; s2t = kt; s2l = t.layer; }
        if (dup) continue;
        float r = test_offset(P, x, y, t, ia, pc);
        if (r < best) { ow = t; best = r; }
    }
    store_patch(work, k, ow);
}

// scatter_kernel + averageOffset, :841-952.  REFERENCE mode: randFloat()
// returns unsigned int 0 (texSynth_util.h:155-163), so candidate i is
// (best.x + 0.9*dist_i, best.y).  COUNTER mode draws r and theta in [0, 1)
// and [0, 2pi) from a counter-based hash.  write_all: the working buffer
// aliases base, so unchanged pixels are written too.
// With key >= 0, a pixel under the key's mask keeps its offset (:887-892).
__global__ void __launch_bounds__(128) k_scatter(const Params P, PatchPlanes work, int write_all, uint32_t pass_id,
                                                 int key) {
    PIXEL_XY
    Patch off = load_patch(P.off, k);
    if (image_culled(P, x, y) || keymask_alpha(P.ex, x, y, key) > 0.0f) {
        if (write_all || !image_culled(P, x, y)) store_patch(work, k, off);
        return;
    }
    float cached = __ldg(P.res + k);
    float best = (float)((double)cached + 10e-7);
    Patch ow = off;
    float ia = lay_texel(P.img.base[P.img.cur], P, x, y).w;
    float dist = (float)(P.ex.w > P.ex.h ? P.ex.w : P.ex.h);
    const float closest = 10.f, factor = 0.9f;
    float2 sc = lvl_texel_lin(P.img.scale, x, y, P.hwFilter);
    PixCtx pc;
    make_pixctx(P, x, y, &pc);
    uint32_t lastx = 0xffffffffu, lasty = 0xffffffffu;  // exact repeats are not re-evaluated
#pragma unroll 1
    for (int i = 0; i < P.scatterSamples && dist * factor >= closest; i++) {
        float dmin = dist * factor;
        float ex, ey;
        if (P.rngMode == PT_RNG_COUNTER) {
            float rr = counter_u01(P.rngSeed, pass_id, x, y, 2 * i);
            float th = counter_u01(P.rngSeed, pass_id, x, y, 2 * i + 1) * 6.28318530717958647692f;
            float s, c;
            sincos_poly(th, &s, &c);
            float len = fmaf(rr, dist - dmin, dmin);
            ex = fmaf(c, len, ow.x);
            ey = fmaf(s, len, ow.y);
        } else {
            ex = ow.x + dmin;
            ey = ow.y + 0.0f;
        }
        clamp_to_exemplar(&ex, &ey, P.ex.w, P.ex.h);
        if (__float_as_uint(ex) == lastx && __float_as_uint(ey) == lasty) {
            dist *= factor;
            continue;
        }
        lastx = __float_as_uint(ex);
        lasty = __float_as_uint(ey);
        float ang = screen_to_exemplar_angle(P, x, y, ex, ey, 0);
        Patch t = make_patch(ex, ey, ang, 0.0f, 0, sc.x, sc.y);
        float r = test_offset(P, x, y, t, ia, pc);
        if (r < best) { ow = t; best = r; }
        dist *= factor;
    }
    Patch avg = make_patch(0, 0, 0, 1.f, 0, 1.f, 1.f);
    int n = 0;
    for (int i = -1; i <= 1; i++)
        for (int j = -1; j <= 1; j++) {
            if (!in_rect(P, x + i, y + j) || (i == 0 && j == 0)) continue;
            float4 nb = __ldg(P.off.A + (size_t)(y + j) * P.W + (x + i));
            if (__float_as_int(nb.w) != 0) continue;
            avg.x = avg.x + nb.x;
            avg.y = avg.y + nb.y;
            n++;
        }
    avg.x = avg.x / (float)n;
    avg.y = avg.y / (float)n;
    avg.theta = screen_to_exemplar_angle(P, x, y, avg.x, avg.y, 0);
    float r = test_offset(P, x, y, avg, ia, pc);
    if (r < best) { ow = avg; best = r; }
    if (best < cached) store_patch(work, k, ow);
    else if (write_all) store_patch(work, k, off);
}

// updateResidualCache_kernel, :661-693
__global__ void __launch_bounds__(128) k_residual(const Params P, float* out) {
    PIXEL_XY
    if (image_culled(P, x, y)) { out[k] = 0.0f; return; }
    PixCtx pc;
    make_pixctx(P, x, y, &pc);
    Patch t = load_patch(P.off, k);
    if (P.counters) count_eval(P, x, y, pc.temporalF || pc.temporalB);
    out[k] = energy(P, x, y, t, pc);
}

// base and output exemplar texels interleaved into 32-byte records (the
// tiled kernels fetch a texel's two colours with one 256-bit load)
__global__ void k_interleave_texels(const float4* base, const float4* out, float4* bo, size_t n) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    bo[2 * t] = base[t];
    bo[2 * t + 1] = out[t];
}

// offsetsToOutput, :263-274
__global__ void k_canvas(const Params P, float4* canvas) {
    PIXEL_XY
    if (P.inc.on && !P.inc.chg[k]) return;  // tracked pass left this record unchanged
    float4 a = __ldg(P.off.A + k);
    float lumy = __ldg(&P.off.B[k].w), luma = __ldg(P.off.C + k);
    float4 c = ex_sample_out(P.ex, a.x, a.y, __float_as_int(a.w));
    canvas[k] = f4(c.x + lumy, c.y + lumy, c.z + lumy, c.w + luma);
}

// copyRandomKernel, :2044-2059
__global__ void k_random_offsets(const Params P, PatchPlanes work) {
    PIXEL_XY
    float4 r = lvl_texel(P.img.rnd, x, y);
    store_patch(work, k, make_patch(r.x, r.y, r.z, 0.f, f2i(r.w), 1.f, 1.f));
}

// offsetUpsampleNearest, :1403-1417
__device__ float2 upsample_nearest(const Params& P, const Patch& c, float dx, float dy) {
    float2 b0, b1;
    basis(c.theta, 1.0f, 1.0f, &b0, &b1);
    float ix, iy;
    new_coord(dx, dy, c.x, c.y, b0, b1, &ix, &iy);
    clamp_to_exemplar(&ix, &iy, P.ex.w, P.ex.h);
    return make_float2(fmaf(ix, 2.0f, 0.5f), fmaf(iy, 2.0f, 0.5f));
}

// upsampleBilinearKernel + TexSynth::upsample, :1453-1532.  Border pixels
// keep the working buffer's content (border_src); residual border keeps the
// base residual.
__global__ void k_upsample(const Params P, PatchPlanes work, PatchPlanes border_src, int copy_border,
                           float* res_out) {
    PIXEL_XY
    if (!in_rect(P, x, y, 1)) {
        if (copy_border) store_patch(work, k, load_patch(border_src, k));
        res_out[k] = __ldg(P.res + k);
        return;
    }
    float cx = (float)((double)x - 0.5) / 2.0f;
    float cy = (float)((double)y - 0.5) / 2.0f;
    int lcx = (int)floorf(cx), lcy = (int)floorf(cy);
    float4 o00 = __ldg(P.off.A + (size_t)lcy * P.W + lcx);
    float4 o10 = __ldg(P.off.A + (size_t)lcy * P.W + lcx + 1);
    float4 o01 = __ldg(P.off.A + (size_t)(lcy + 1) * P.W + lcx);
    float4 o11 = __ldg(P.off.A + (size_t)(lcy + 1) * P.W + lcx + 1);
    float a = cx - (float)lcx, b = cy - (float)lcy;
    float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
    // the reference's sum as nvcc contracts it (the first product fused with
    // the second, rounded, then the others added by fused multiply-adds;
    // measured on its upsample kernel)
    float ix = fmaf(w00, o00.x, w10 * o10.x); ix = fmaf(w01, o01.x, ix); ix = fmaf(w11, o11.x, ix);
    float iy = fmaf(w00, o00.y, w10 * o10.y); iy = fmaf(w01, o01.y, iy); iy = fmaf(w11, o11.y, iy);
    float2 up = make_float2(fmaf(ix, 2.0f, 0.5f), fmaf(iy, 2.0f, 0.5f));
    bool far = false;
    {
        float dx, dy;
        dx = ix - o00.x; dy = iy - o00.y; far |= fmaf(dx, dx, dy * dy) > 16.0f;
        dx = ix - o10.x; dy = iy - o10.y; far |= fmaf(dx, dx, dy * dy) > 16.0f;
        dx = ix - o01.x; dy = iy - o01.y; far |= fmaf(dx, dx, dy * dy) > 16.0f;
        dx = ix - o11.x; dy = iy - o11.y; far |= fmaf(dx, dx, dy * dy) > 16.0f;
    }
    if (far) {
        int rcx = (int)roundf(cx), rcy = (int)roundf(cy);
        Patch c = load_patch(P.off, (size_t)rcy * P.W + rcx);
        up = upsample_nearest(P, c, cx - (float)rcx, cy - (float)rcy);
    }
    int layer = __float_as_int(o00.w);
    float rw = __ldg(P.res + (size_t)lcy * P.W + lcx);
    float ang = screen_to_exemplar_angle(P, x, y, up.x, up.y, layer);
    float2 sc = lvl_texel_lin(P.img.scale, x, y, P.hwFilter);
    store_patch(work, k, make_patch(up.x, up.y, ang, 0.0f, layer, sc.x, sc.y));
    res_out[k] = rw;
}

// calculateTranslatedPosition + advectKernel, :1540-1693
__global__ void k_advect(const Params P, int d, int forwards, int time_step, int flags) {
    PIXEL_XY
    const AdvView& A = P.adv[d];
    const int cur = P.img.cur, prev = (P.img.cur + 1) % 2;
    if (image_culled(P, x, y)) {
        A.base[k] = f4(0, 0, 0, 0);
        A.out[k] = f4(0, 0, 0, 0);
        store_patch(A.off, k, make_patch(0, 0, 0, 0, 0, 1.f, 1.f));
        return;
    }
    float4 rnd = lvl_texel(P.img.rnd, x, y);
    float4 fr = f4(rnd.x - floorf(rnd.x), rnd.y - floorf(rnd.y), rnd.z - floorf(rnd.z), rnd.w - floorf(rnd.w));
    Patch out = make_patch(0, 0, 0, 0, 0, 1.f, 1.f);
    bool valid = false;
    float tx = 0, ty = 0;
    if (!(flags & PT_ADVECT_DO_NOT_CHECK_PREVIOUS)) {
        float2 fw, bk;
        if (forwards) {
            bk = lay_texel(P.img.velb[cur], P, x, y);
            tx = (float)x + bk.x; ty = (float)y + bk.y;
            fw = lay_bilinear(P.img.velf[prev], P, tx, ty);
        } else {
            fw = lay_texel(P.img.velf[cur], P, x, y);
            tx = (float)x + fw.x; ty = (float)y + fw.y;
            bk = lay_bilinear(P.img.velb[prev], P, tx, ty);
        }
        fw.x = -fw.x; fw.y = -fw.y;
        float ddx = fw.x - bk.x, ddy = fw.y - bk.y;
        float dist = sqrtf(fmaf(ddy, ddy, ddx * ddx));
        float cxf = fminf(fmaxf(ceilf(tx), -2.f), 1e9f), cyf = fminf(fmaxf(ceilf(ty), -2.f), 1e9f);
        float fxf = fminf(fmaxf(floorf(tx), -2.f), 1e9f), fyf = fminf(fmaxf(floorf(ty), -2.f), 1e9f);
        valid = in_rect(P, f2i(cxf), f2i(cyf)) && in_rect(P, f2i(fxf), f2i(fyf)) && (dist < (float)(1.414 * 2));
        if (valid) {
            float pd = lay_texel(P.img.dt[prev], P, f2i(tx), f2i(ty));
            if (pd > ((float)P.distTransCull - 8.0f)) valid = false;
        }
    }
    if (valid) {
        int rtx = (int)roundf(tx), rty = (int)roundf(ty);
        Patch nx = load_patch(P.off, (size_t)rty * P.W + rtx);
        float2 b0, b1;
        basis(nx.theta, 1.0f, 1.0f, &b0, &b1);
        float ix, iy;
        new_coord(tx - (float)rtx, ty - (float)rty, nx.x, nx.y, b0, b1, &ix, &iy);
        clamp_to_exemplar(&ix, &iy, P.ex.w, P.ex.h);
        float4 color = lay_texel(P.img.base[cur], P, x, y);
        float4 pcol = lay_bilinear(P.img.base[prev], P, tx, ty);
        out.x = ix; out.y = iy; out.theta = nx.theta;
        if (P.lumShiftEnable) {
            float dr = color.x - pcol.x, dg = color.y - pcol.y, db = color.z - pcol.z;
            float ly = (float)(0.2126 * (double)dr + 0.7152 * (double)dg + 0.0722 * (double)db);
            out.lumy = nx.lumy + ly;
        } else {
            out.lumy = 0.f;
        }
        out.luma = 0.f;
        out.layer = nx.layer;
        out.hyst = 1;
        A.base[k] = pcol;
        A.out[k] = ex_sample_out(P.ex, out.x, out.y, out.layer);
        A.ts[k] = time_step;
    }
    // keyframe interpolation, :1652-1675: long-range advection, or a pixel
    // left without one, takes the frame-to-key ribbon where it is shorter
    if ((flags & PT_ADVECT_CHECK_FRAME_TO_KEY) && (time_step > 1 || out.hyst == 0)) {
        const Arr<float4>& R = P.img.f2k[forwards ? 0 : 1];
        const float4 c = R.p ? lvl_texel_lin(R, x, y, P.hwFilter) : f4(0.f, 0.f, 0.f, 0.f);
        const int rts = f2i(c.x), rlayer = f2i(c.w);
        if (rlayer >= 0 && (abs(rts) < time_step || out.hyst == 0)) {
            out.x = c.z + (float)x;
            out.y = c.y + (float)y;
            out.layer = rlayer;
            out.hyst = 1.0f;
            out.lumy = 0.f;
            out.luma = 0.f;
        }
        float4 eb, eo;
        ex_sample2(P.ex, out.x, out.y, out.layer, &eb, &eo);
        A.base[k] = eb;
        A.out[k] = eo;
        A.ts[k] = abs(rts);
    }
    if (out.hyst == 0) {
        out = make_patch(rnd.x, rnd.y, rnd.z, 0.0f, f2i(rnd.w), 1.f, 1.f);
        A.base[k] = f4(0, 0, 0, 0);
        A.out[k] = f4(0, 0, 0, 0);
        A.ts[k] = -1;
    }
    float J = P.jitter;
    out.x = fmaf(fr.x, J, out.x * (1 - J));
    out.y = fmaf(fr.y, J, out.y * (1 - J));
    out.theta = screen_to_exemplar_angle(P, x, y, out.x, out.y, out.layer);
    store_patch(A.off, k, out);
}

// mergeRandomlyKernel, :1891-1936 (frame-to-key ribbons are unbound outside
// keyframe mode: both read as valid, so the ribbon clause is false)
__global__ void k_merge_random(const Params P, int d, int forwards, float weight, int force, PatchPlanes work) {
    PIXEL_XY
    float4 rnd = lvl_texel(P.img.rnd, x, y);
    float r = forwards ? rnd.x - floorf(rnd.x) : rnd.y - floorf(rnd.y);
    bool av = __ldg(&P.adv[d].off.B[k].x) > 0;
    const PatchPlanes& src = ((av || force) && r < weight) ? P.adv[d].off : P.off;
    store_patch(work, k, load_patch(src, k));
}

// mergeUsingResidualKernel, :1856-1889
__global__ void k_merge_residual(const Params P, int d, PatchPlanes work) {
    PIXEL_XY
    Patch r;
    if (__ldg(P.adv[d].res + k) < __ldg(P.res + k)) { r = load_patch(P.adv[d].off, k); r.hyst = 1.f; }
    else { r = load_patch(P.off, k); r.hyst = 0.f; }
    store_patch(work, k, r);
}

// separable Gaussian over the histogram, convolution.cu:76-210 (normalised
// weights, zero apron): rows (rows=1) or columns (rows=0)
__global__ void k_conv(const float* src, float* dst, int w, int h, int pitch, int rows, ConvKernel kw) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    float s = 0.0f;
    const int r = kw.r;
    for (int j = -r; j <= r; j++) {
        int xx = rows ? x + j : x, yy = rows ? y : y + j;
        float v = (xx >= 0 && xx < w && yy >= 0 && yy < h) ? __ldg(src + (size_t)yy * pitch + xx) : 0.0f;
        s = fmaf(kw.w[r - j], v, s);
    }
    dst[(size_t)y * pitch + x] = s;
}

// copies of the level rectangle
__global__ void k_copy_patch(const Params P, PatchPlanes dst, PatchPlanes src) {
    PIXEL_XY
    dst.A[k] = __ldg(src.A + k);
    dst.B[k] = __ldg(src.B + k);
    dst.C[k] = __ldg(src.C + k);
}
__global__ void k_copy_float(const Params P, float* dst, const float* src) {
    PIXEL_XY
    dst[k] = __ldg(src + k);
}

// PatchXF records <-> planes, and the half-precision residual round trip
__global__ void k_unpack_patch(const Params P, const pt_patchxf* src, PatchPlanes dst) {
    PIXEL_XY
    pt_patchxf v = src[(size_t)y * P.lw + x];
    Patch p;
    p.x = v.x; p.y = v.y; p.theta = v.theta; p.hyst = v.hysteresis; p.layer = v.layer;
    p.su = v.scaleU; p.sv = v.scaleV; p.lumy = v.lumShiftY; p.luma = v.lumShiftA;
    store_patch(dst, k, p);
}
__global__ void k_pack_patch(const Params P, PatchPlanes src, pt_patchxf* dst) {
    PIXEL_XY
    Patch p = load_patch(src, k);
    pt_patchxf v;
    v.x = p.x; v.y = p.y; v.theta = p.theta; v.hysteresis = p.hyst; v.layer = p.layer;
    v.scaleU = p.su; v.scaleV = p.sv; v.lumShiftY = p.lumy; v.lumShiftA = p.luma;
    dst[(size_t)y * P.lw + x] = v;
}
__global__ void k_load_residual(const Params P, const float* src, float* dst) {
    PIXEL_XY
    dst[k] = __half2float(__float2half_rn(src[(size_t)y * P.lw + x]));
}
__global__ void k_gather_level(const Params P, const float* src, int ch, float* dst) {
    PIXEL_XY
    for (int c = 0; c < ch; c++) dst[((size_t)y * P.lw + x) * ch + c] = __ldg(src + k * ch + c);
}

// ---------------------------------------------------------------------------
// pyramid construction (downsample.cpp:41-209, imageIO.h:136-139)
// ---------------------------------------------------------------------------

__global__ void k_down_avg(const float* src, int w, int h, int ch, int vel, float* dst) {
    int lw = w >> 1, lh = h >> 1;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= lw || y >= lh) return;
    for (int c = 0; c < ch; c++) {
        float s = 0.0f;
        s = s + __ldg(src + ((size_t)(2 * y) * w + 2 * x) * ch + c);
        s = s + __ldg(src + ((size_t)(2 * y) * w + 2 * x + 1) * ch + c);
        s = s + __ldg(src + ((size_t)(2 * y + 1) * w + 2 * x) * ch + c);
        s = s + __ldg(src + ((size_t)(2 * y + 1) * w + 2 * x + 1) * ch + c);
        s = s * 0.25f;
        if (vel) s = s * 0.5f;
        dst[((size_t)y * lw + x) * ch + c] = s;
    }
}

// majority vote of the 2x2 values; ties go to the smallest value
__global__ void k_down_vote(const int* src, int w, int h, int* dst) {
    int lw = w >> 1, lh = h >> 1;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= lw || y >= lh) return;
    int v[4] = {__ldg(src + (size_t)(2 * y) * w + 2 * x), __ldg(src + (size_t)(2 * y) * w + 2 * x + 1),
                __ldg(src + (size_t)(2 * y + 1) * w + 2 * x), __ldg(src + (size_t)(2 * y + 1) * w + 2 * x + 1)};
    int best = v[0], bestc = -1;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int c = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) c += (v[j] == v[i]);
        if (c > bestc || (c == bestc && v[i] < best)) { bestc = c; best = v[i]; }
    }
    dst[(size_t)y * lw + x] = best;
}

__global__ void k_tensor_angle(const float* t3, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float xx = __ldg(t3 + 3 * i), xy = __ldg(t3 + 3 * i + 1), yy = __ldg(t3 + 3 * i + 2);
    float a2 = atan2_poly((float)(2.0 * (double)xy), xx - yy);
    float angle = (float)(0.5 * (double)a2 + 1.57079632679489661923);
    out[i] = ((double)angle >= 1.57079632679489661923) ? (float)((double)angle - 3.14159265358979323846) : angle;
}

// ---------------------------------------------------------------------------
// random-offset level (SynthesisFrame::createRandomPyramid,
// synthesisFrame.cpp:66-150)
// ---------------------------------------------------------------------------

struct RandParams {
    int w, h, mx, my;
    int transparencyOk, orientationEnabled;
    Arr<float4> img;     // level-size input colour (alpha)
    Arr<float> iorient;  // level-size input orientation
    ExView ex;           // exemplar level (style 0)
    float4* out;
};

__device__ __forceinline__ float4 random_texel(const RandParams& R, int x, int y, uint32_t d0, uint32_t d1,
                                                uint32_t d2, uint32_t d3) {
    int ox = (int)((d0 >> 1) % (uint32_t)R.mx);
    int oy = (int)((d1 >> 1) % (uint32_t)R.my);
    float orient = R.orientationEnabled
                       ? __ldg(R.iorient.p + (size_t)y * R.iorient.w + x) - __ldg(R.ex.orient + (size_t)oy * R.ex.w + ox)
                       : 0.f;
    float rx = (float)(d2 >> 1) / (float)2147483647;
    float ry = (float)(d3 >> 1) / (float)2147483647;
    return f4((float)ox + rx, (float)oy + ry, orient, 0.0f);
}

// One thread per row: the glibc additive-feedback state at the row start is
// precomputed on the host (jump-ahead by a 31x31 matrix power over Z/2^32);
// each thread then steps the recurrence r[i] = r[i-31] + r[i-3] in a
// shared-memory ring.  Valid when no pixel retries (no exemplar texel with
// alpha < 0.99, or transparency allowed).
__global__ void k_glibc_rows(const RandParams R, const uint32_t* row_states) {
    extern __shared__ uint32_t ring_all[];
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t* ring = ring_all + threadIdx.x;  // stride blockDim.x: conflict-free
    const int S = blockDim.x;
    if (y >= R.h) return;
    for (int i = 0; i < 31; i++) ring[i * S] = row_states[(size_t)y * 31 + i];
    int head = 0;
    int h28 = 28;
    for (int x = 0; x < R.w; x++) {
        uint32_t d[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            uint32_t v = ring[head * S] + ring[h28 * S];
            ring[head * S] = v;
            head = (head == 30) ? 0 : head + 1;
            h28 = (h28 == 30) ? 0 : h28 + 1;
            d[q] = v;
        }
        R.out[(size_t)y * R.w + x] = random_texel(R, x, y, d[0], d[1], d[2], d[3]);
    }
}

// Exact serial version (one thread) with the reference's retry loop for
// opaque pixels that drew a transparent exemplar texel.
__global__ void k_glibc_serial(const RandParams R, const uint32_t* state31) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t ring[31];
    for (int i = 0; i < 31; i++) ring[i] = state31[i];
    int head = 0;
    auto next = [&]() -> uint32_t {
        int h28 = head + 28;
        if (h28 >= 31) h28 -= 31;
        uint32_t v = ring[head] + ring[h28];
        ring[head] = v;
        head = (head == 30) ? 0 : head + 1;
        return v;
    };
    for (int y = 0; y < R.h; y++)
        for (int x = 0; x < R.w; x++) {
            float ia = __ldg(R.img.p + (size_t)y * R.img.w + x).w;
            uint32_t d0, d1;
            int trial = 0;
            bool again;
            do {
                d0 = next();
                d1 = next();
                trial++;
                int ox = (int)((d0 >> 1) % (uint32_t)R.mx), oy = (int)((d1 >> 1) % (uint32_t)R.my);
                float ea = __ldg(R.ex.out + (size_t)oy * R.ex.w + ox).w;
                again = !R.transparencyOk && ia > kAlphaThreshold && ea < kAlphaThreshold && trial < 50;
            } while (again);
            uint32_t d2 = next(), d3 = next();
            R.out[(size_t)y * R.w + x] = random_texel(R, x, y, d0, d1, d2, d3);
        }
}

// Keyframe interpolation (createRandomPyramid with setupWithKeys,
// synthesisFrame.cpp:94-139): each pixel first draws its key layer
// (rand() % nk + first_key), then the offset in that layer with the retry
// rule, then the two fractions; one thread, exact glibc order.
__global__ void k_glibc_serial_keys(const RandParams R, const uint32_t* state31, int nk, int first_key) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t ring[31];
    for (int i = 0; i < 31; i++) ring[i] = state31[i];
    int head = 0;
    auto next = [&]() -> uint32_t {
        int h28 = head + 28;
        if (h28 >= 31) h28 -= 31;
        uint32_t v = ring[head] + ring[h28];
        ring[head] = v;
        head = (head == 30) ? 0 : head + 1;
        return v;
    };
    const size_t lsz = (size_t)R.ex.w * R.ex.h;
    for (int y = 0; y < R.h; y++)
        for (int x = 0; x < R.w; x++) {
            const int style = (int)((next() >> 1) % (uint32_t)nk) + first_key;
            const int sl = clampi(style, 0, R.ex.ns - 1);  // a layer of the uploaded exemplar
            float ia = __ldg(R.img.p + (size_t)y * R.img.w + x).w;
            int ox, oy, trial = 0;
            bool again;
            do {
                ox = (int)((next() >> 1) % (uint32_t)R.mx);
                oy = (int)((next() >> 1) % (uint32_t)R.my);
                trial++;
                float ea = __ldg(R.ex.out + sl * lsz + (size_t)oy * R.ex.w + ox).w;
                again = !R.transparencyOk && ia > kAlphaThreshold && ea < kAlphaThreshold && trial < 50;
            } while (again);
            float orient = R.orientationEnabled ? __ldg(R.iorient.p + (size_t)y * R.iorient.w + x) -
                                                      __ldg(R.ex.orient + sl * lsz + (size_t)oy * R.ex.w + ox)
                                                : 0.f;
            float rx = (float)(next() >> 1) / (float)2147483647;
            float ry = (float)(next() >> 1) / (float)2147483647;
            R.out[(size_t)y * R.w + x] = f4((float)ox + rx, (float)oy + ry, orient, (float)style);
        }
}

// counter-based random level: four hashed draws per pixel and trial
__global__ void k_counter_random(const RandParams R, uint32_t seed) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= R.w || y >= R.h) return;
    float ia = __ldg(R.img.p + (size_t)y * R.img.w + x).w;
    uint32_t base = hash32(seed ^ hash32(x * 0x85EBCA6BU ^ hash32(y * 0xC2B2AE35U)));
    uint32_t d0, d1;
    int trial = 0;
    bool again;
    do {
        d0 = hash32(base + 4u * trial);
        d1 = hash32(base + 4u * trial + 1u);
        trial++;
        int ox = (int)((d0 >> 1) % (uint32_t)R.mx), oy = (int)((d1 >> 1) % (uint32_t)R.my);
        float ea = __ldg(R.ex.out + (size_t)oy * R.ex.w + ox).w;
        again = !R.transparencyOk && ia > kAlphaThreshold && ea < kAlphaThreshold && trial < 50;
    } while (again);
    uint32_t d2 = hash32(base + 0x40000000u), d3 = hash32(base + 0x40000001u);
    R.out[(size_t)y * R.w + x] = random_texel(R, x, y, d0, d1, d2, d3);
}

// any exemplar output texel with alpha < 0.99 (decides whether the random
// level can be drawn row-parallel)
__global__ void k_any_transparent(const float4* out, size_t n, int* flag) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (__ldg(out + i).w < kAlphaThreshold) { atomicOr(flag, 1); return; }
}

}  // namespace ptk

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

namespace pt {

using namespace ptk;

static inline dim3 grid2(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }
static const dim3 kPix(32, 4);

#define LAUNCH_CHECK() return cudaGetLastError()

cudaError_t launch_propagate(const Params& P, PatchPlanes work, int jump, int key, cudaStream_t s) {
    k_propagate<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, work, jump, key);
    LAUNCH_CHECK();
}
cudaError_t launch_scatter(const Params& P, PatchPlanes work, int write_all, uint32_t pass_id, int key,
                           cudaStream_t s) {
    k_scatter<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, work, write_all, pass_id, key);
    LAUNCH_CHECK();
}
cudaError_t launch_residual(const Params& P, float* out, cudaStream_t s) {
    k_residual<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, out);
    LAUNCH_CHECK();
}
cudaError_t launch_canvas(const Params& P, float4* canvas, cudaStream_t s) {
    k_canvas<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, canvas);
    LAUNCH_CHECK();
}
cudaError_t launch_random_offsets(const Params& P, PatchPlanes work, cudaStream_t s) {
    k_random_offsets<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, work);
    LAUNCH_CHECK();
}
cudaError_t launch_upsample(const Params& P, PatchPlanes work, PatchPlanes border_src, int copy_border,
                            float* res_out, cudaStream_t s) {
    k_upsample<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, work, border_src, copy_border, res_out);
    LAUNCH_CHECK();
}
cudaError_t launch_advect(const Params& P, int d, int forwards, int time_step, int flags, cudaStream_t s) {
    k_advect<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, d, forwards, time_step, flags);
    LAUNCH_CHECK();
}
cudaError_t launch_merge_random(const Params& P, int d, int forwards, float weight, int force, PatchPlanes work,
                                cudaStream_t s) {
    k_merge_random<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, d, forwards, weight, force, work);
    LAUNCH_CHECK();
}
cudaError_t launch_merge_residual(const Params& P, int d, PatchPlanes work, cudaStream_t s) {
    k_merge_residual<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, d, work);
    LAUNCH_CHECK();
}
cudaError_t launch_conv(const float* src, float* dst, int w, int h, int pitch, int rows, const ConvKernel& kw,
                        cudaStream_t s) {
    dim3 b(32, 4);
    k_conv<<<grid2(w, h, b), b, 0, s>>>(src, dst, w, h, pitch, rows, kw);
    LAUNCH_CHECK();
}
cudaError_t launch_copy_patch(const Params& P, PatchPlanes dst, PatchPlanes src, cudaStream_t s) {
    k_copy_patch<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, dst, src);
    LAUNCH_CHECK();
}
cudaError_t launch_copy_float(const Params& P, float* dst, const float* src, cudaStream_t s) {
    k_copy_float<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, dst, src);
    LAUNCH_CHECK();
}
cudaError_t launch_unpack_patch(const Params& P, const pt_patchxf* src, PatchPlanes dst, cudaStream_t s) {
    k_unpack_patch<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, src, dst);
    LAUNCH_CHECK();
}
cudaError_t launch_pack_patch(const Params& P, PatchPlanes src, pt_patchxf* dst, cudaStream_t s) {
    k_pack_patch<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, src, dst);
    LAUNCH_CHECK();
}
cudaError_t launch_load_residual(const Params& P, const float* src, float* dst, cudaStream_t s) {
    k_load_residual<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, src, dst);
    LAUNCH_CHECK();
}
cudaError_t launch_gather_level(const Params& P, const float* src, int ch, float* dst, cudaStream_t s) {
    k_gather_level<<<grid2(P.lw, P.lh, kPix), kPix, 0, s>>>(P, src, ch, dst);
    LAUNCH_CHECK();
}
cudaError_t launch_down_avg(const float* src, int w, int h, int ch, int vel, float* dst, cudaStream_t s) {
    dim3 b(32, 4);
    k_down_avg<<<grid2(w >> 1, h >> 1, b), b, 0, s>>>(src, w, h, ch, vel, dst);
    LAUNCH_CHECK();
}
cudaError_t launch_down_vote(const int* src, int w, int h, int* dst, cudaStream_t s) {
    dim3 b(32, 4);
    k_down_vote<<<grid2(w >> 1, h >> 1, b), b, 0, s>>>(src, w, h, dst);
    LAUNCH_CHECK();
}
cudaError_t launch_tensor_angle(const float* t3, int n, float* out, cudaStream_t s) {
    k_tensor_angle<<<(n + 255) / 256, 256, 0, s>>>(t3, n, out);
    LAUNCH_CHECK();
}
cudaError_t launch_random_level_keys(int w, int h, int mx, int my, int transparencyOk, int orientationEnabled,
                                     Arr<float4> img, Arr<float> iorient, ExView ex, float4* out,
                                     const uint32_t* state31, int nk, int first_key, cudaStream_t s) {
    RandParams R;
    R.w = w; R.h = h; R.mx = mx; R.my = my;
    R.transparencyOk = transparencyOk; R.orientationEnabled = orientationEnabled;
    R.img = img; R.iorient = iorient; R.ex = ex; R.out = out;
    k_glibc_serial_keys<<<1, 1, 0, s>>>(R, state31, nk, first_key);
    LAUNCH_CHECK();
}
cudaError_t launch_random_level(int mode, int w, int h, int mx, int my, int transparencyOk, int orientationEnabled,
                                Arr<float4> img, Arr<float> iorient, ExView ex, float4* out,
                                const uint32_t* states, uint32_t seed, cudaStream_t s) {
    RandParams R;
    R.w = w; R.h = h; R.mx = mx; R.my = my;
    R.transparencyOk = transparencyOk; R.orientationEnabled = orientationEnabled;
    R.img = img; R.iorient = iorient; R.ex = ex; R.out = out;
    if (mode == 0) {  // row-parallel glibc
        const int tb = 64;
        k_glibc_rows<<<(h + tb - 1) / tb, tb, tb * 31 * sizeof(uint32_t), s>>>(R, states);
    } else if (mode == 1) {  // serial glibc
        k_glibc_serial<<<1, 1, 0, s>>>(R, states);
    } else {
        dim3 b(32, 4);
        k_counter_random<<<grid2(w, h, b), b, 0, s>>>(R, seed);
    }
    LAUNCH_CHECK();
}
cudaError_t launch_interleave_texels(const float4* base, const float4* out, float4* bo, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    k_interleave_texels<<<blocks, threads, 0, s>>>(base, out, bo, n);
    LAUNCH_CHECK();
}
cudaError_t launch_any_transparent(const float4* out, size_t n, int* flag, cudaStream_t s) {
    k_any_transparent<<<152 * 4, 256, 0, s>>>(out, n, flag);
    LAUNCH_CHECK();
}

}  // namespace pt
