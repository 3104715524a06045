// pt_keys.cu -- keyframe interpolation kernels: propagation and scatter
// through the key-to-key cumulative fields, the accumulated ribbon field and
// the frame-to-key ribbon initialisation (src/PaintTweenCUDA/
// texSynth_kernel.cu:290-304,723-839,984-1110,1728-1853,2061-2118).
#include "pt_common.cuh"
#include "pt_device.cuh"
#include "pt_internal.h"

namespace ptk {

namespace {

constexpr int kKeyPix = 128;
constexpr float kEpsilon = 0.000001f;  // EPSILON, types.h:38

dim3 grid_of(int w, int h) { return dim3((w + 31) / 32, (h + 3) / 4); }

#define KEY_PIXEL_XY                                    \
    const int x = blockIdx.x * blockDim.x + threadIdx.x; \
    const int y = blockIdx.y * blockDim.y + threadIdx.y; \
    if (!in_rect(P, x, y)) return;                      \
    const size_t k = (size_t)y * P.W + x;

// a cumulative-field fetch at exemplar (u, v) of key layer j (linear filter,
// clamp); a layer outside the uploaded ones reads zero
__device__ float4 cumul_sample(const KeyView& K, int d, float u, float v, int j) {
    const float4* F = K.cumul[d];
    if (!F || j < 0 || j >= K.n) return f4(0.f, 0.f, 0.f, 0.f);
    Bl b = bl_setup(u, v, K.w, K.h, K.hw);
    const float4* L = F + (size_t)j * K.w * K.h;
    const size_t r0 = (size_t)b.y0 * K.w, r1 = (size_t)b.y1 * K.w;
    return bl4(b, __ldg(L + r0 + b.x0), __ldg(L + r0 + b.x1), __ldg(L + r1 + b.x0), __ldg(L + r1 + b.x1));
}

// RibbonP(Color4): (x, y, time_step, layer) = (b, g, r, a)
__device__ __forceinline__ Ribbon ribbon_of(float4 c) {
    Ribbon r;
    r.x = c.z;
    r.y = c.y;
    r.time_step = f2i(c.x);
    r.layer = f2i(c.w);
    return r;
}

// the candidates a key-to-key ribbon reaches from exemplar (ex, ey) of
// layer `elayer`: back through the keys below it, then forward through the
// keys above (:1063-1104, :800-835); PROP: propagate's stop rule (time step
// channel < -EPSILON) instead of scatter's (invalid layer)
template <bool PROP>
__device__ void ribbon_candidates(const Params& P, const KeyView& K, int x, int y, float ex0, float ey0, int elayer,
                                  float ia, const PixCtx& pc, Patch* ow, float* best) {
    for (int side = 0; side < 2; side++) {
        const bool back = side == 0;
        float ex = ex0, ey = ey0;
        for (int j = back ? elayer - 1 : elayer + 1; back ? j >= P.firstKey : j <= P.lastKey; j += back ? -1 : 1) {
            float4 m = cumul_sample(K, back ? 0 : 1, ex, ey, back ? j + 1 : j - 1);
            if (PROP ? (m.x < -kEpsilon) : (ribbon_of(m).layer < 0)) break;
            if (PROP) {
                ex = ex + m.z;
                ey = ey + m.y;
            } else {
                Ribbon rb = ribbon_of(m);
                ex = ex + rb.x;
                ey = ey + rb.y;
            }
            Patch q = make_patch(ex, ey, screen_to_exemplar_angle(P, x, y, ex, ey, j), 0.f, j, 1.f, 1.f);
            float r = test_offset(P, x, y, q, ia, pc);
            if (r < *best) {
                *ow = q;
                *best = r;
            }
        }
    }
}

// propagate_kernel_keys, :984-1110
__global__ void __launch_bounds__(kKeyPix) k_propagate_keys(const Params P, PatchPlanes work, int jump, int key,
                                                            const KeyView K) {
    KEY_PIXEL_XY
    if (image_culled(P, x, y)) {
        store_patch(work, k, make_patch(0, 0, 0, 0, 0, 1.f, 1.f));
        return;
    }
    if (keymask_alpha(P.ex, x, y, key) > 0.0f) {
        store_patch(work, k, make_patch((float)x, (float)y, 0.f, 1.f, key, 1.f, 1.f));
        return;
    }
    float best = __ldg(P.res + k);
    const float ia = lay_texel(P.img.base[P.img.cur], P, x, y).w;
    Patch ow = load_patch(P.off, k);
    PixCtx pc;
    make_pixctx(P, x, y, &pc);
#pragma unroll 1
    for (int c = 0; c < 4; c++) {
        int tx = x, ty = y;
        if (c == 0) tx = x + jump;
        else if (c == 1) tx = x - jump;
        else if (c == 2) ty = y + jump;
        else ty = y - jump;
        Patch t = propagate_offset(P, tx, ty, x, y);
        float r = test_offset(P, x, y, t, ia, pc);
        if (r < best) {
            ow = t;
            best = r;
        }
        ribbon_candidates<true>(P, K, x, y, t.x, t.y, t.layer, ia, pc, &ow, &best);
    }
    store_patch(work, k, ow);
}

// scatter_kernel_keys, :723-839.  randFloat() returns 0 (texSynth_util.h:
// 155-163): candidate i is (best.x + 0.9*dist_i, best.y) in the best
// offset's layer, sampleCount / (lastKey - firstKey + 1) of them.
__global__ void __launch_bounds__(kKeyPix) k_scatter_keys(const Params P, PatchPlanes work, int write_all, int key,
                                                          const KeyView K) {
    KEY_PIXEL_XY
    const Patch off = load_patch(P.off, k);
    if (image_culled(P, x, y)) {
        if (write_all) store_patch(work, k, off);
        return;
    }
    if (keymask_alpha(P.ex, x, y, key) > 0.0f) {
        store_patch(work, k, off);
        return;
    }
    const float cached = __ldg(P.res + k);
    float best = (float)((double)cached + 10e-7);
    Patch ow = off;
    const float ia = lay_texel(P.img.base[P.img.cur], P, x, y).w;
    float dist = (float)(P.ex.w > P.ex.h ? P.ex.w : P.ex.h);
    const float closest = 10.f, factor = 0.9f;
    const int span = P.lastKey - P.firstKey + 1;
    const int samples = span != 0 ? P.scatterSamples / span : 0;
    PixCtx pc;
    make_pixctx(P, x, y, &pc);
#pragma unroll 1
    for (int i = 0; i < samples && dist * factor >= closest; i++) {
        const float dmin = dist * factor;
        float ex = ow.x + dmin, ey = ow.y + 0.0f;
        clamp_to_exemplar(&ex, &ey, P.ex.w, P.ex.h);
        const int elayer = ow.layer;
        Patch t = make_patch(ex, ey, screen_to_exemplar_angle(P, x, y, ex, ey, elayer), 0.f, elayer, 1.f, 1.f);
        float r = test_offset(P, x, y, t, ia, pc);
        if (r < best) {
            ow = t;
            best = r;
        }
        ribbon_candidates<false>(P, K, x, y, ex, ey, elayer, ia, pc, &ow, &best);
        dist *= factor;
    }
    if (best < cached) store_patch(work, k, ow);
    else if (write_all) store_patch(work, k, off);
}

// accumulateAdvectionKernel, :1728-1828: the ribbon field of the previous
// frame carried along the velocities (calculateTranslatedPosition,
// :1540-1574) and extended by time_step.  The chained comparison of :1776
// is kept as written: ((l00 == l10) == l01) == l11 compares booleans with
// layers.
__global__ void __launch_bounds__(kKeyPix) k_accumulate_ribbon(const Params P, int forwards, Ribbon* dest,
                                                               const Ribbon* src, int time_step, int overwrite) {
    KEY_PIXEL_XY
    const int cur = P.img.cur, prev = (P.img.cur + 1) % 2;
    Ribbon out;
    out.x = 0.f;
    out.y = 0.f;
    out.time_step = 0;
    out.layer = -1;
    const bool masked = lay_texel(P.img.base[cur], P, x, y).w == 0.0f;
    float tx = 0.f, ty = 0.f;
    bool valid = false;
    if (!masked) {
        float2 fw, bk;
        if (forwards) {
            bk = lay_texel(P.img.velb[cur], P, x, y);
            tx = (float)x + bk.x;
            ty = (float)y + bk.y;
            fw = lay_bilinear(P.img.velf[prev], P, tx, ty);
        } else {
            fw = lay_texel(P.img.velf[cur], P, x, y);
            tx = (float)x + fw.x;
            ty = (float)y + fw.y;
            bk = lay_bilinear(P.img.velb[prev], P, tx, ty);
        }
        fw.x = -fw.x;
        fw.y = -fw.y;
        const float ddx = fw.x - bk.x, ddy = fw.y - bk.y;
        const float dist = sqrtf(fmaf(ddy, ddy, ddx * ddx));
        const float cxf = fminf(fmaxf(ceilf(tx), -2.f), 1e9f), cyf = fminf(fmaxf(ceilf(ty), -2.f), 1e9f);
        const float fxf = fminf(fmaxf(floorf(tx), -2.f), 1e9f), fyf = fminf(fmaxf(floorf(ty), -2.f), 1e9f);
        valid = in_rect(P, f2i(cxf), f2i(cyf)) && in_rect(P, f2i(fxf), f2i(fyf)) && (dist < (float)(1.414 * 2));
    }
    if (!valid) {
        if (overwrite) dest[k] = out;
        return;
    }
    // floor and ceil of (tx, ty) lie inside the level rectangle
    const int ftx = (int)floorf(tx), fty = (int)floorf(ty), ctx = (int)ceilf(tx), cty = (int)ceilf(ty);
    const Ribbon s00 = src[(size_t)fty * P.W + ftx], s10 = src[(size_t)fty * P.W + ctx];
    const Ribbon s01 = src[(size_t)cty * P.W + ftx], s11 = src[(size_t)cty * P.W + ctx];
    const bool v00 = s00.layer >= 0, v10 = s10.layer >= 0, v01 = s01.layer >= 0, v11 = s11.layer >= 0;
    if (!(v00 || v10 || v01 || v11)) {
        if (overwrite) dest[k] = out;
        return;
    }
    const bool all_valid = v00 && v10 && v01 && v11;
    const int e1 = (s00.layer == s10.layer) ? 1 : 0;
    const int e2 = (e1 == s01.layer) ? 1 : 0;
    const bool same = e2 == s11.layer;
    const float th = 5.f;
    const bool diverges = fabsf(s00.x - s10.x) > th || fabsf(s00.x - s01.x) > th || fabsf(s00.x - s11.x) > th ||
                          fabsf(s00.y - s10.y) > th || fabsf(s00.y - s01.y) > th || fabsf(s00.y - s11.y) > th;
    if (!all_valid || !same || diverges) {
        const int rtx = (int)roundf(tx), rty = (int)roundf(ty);
        if (ftx == rtx && fty == rty) out = s00;
        else if (ftx + 1 == rtx && fty == rty) out = s10;
        else if (ftx == rtx && fty + 1 == rty) out = s01;
        else out = s11;
    } else {
        const float wx = tx - (float)ftx, wy = ty - (float)fty;
        const float rx0 = s00.x * (1.f - wx) + s10.x * wx;
        const float ry0 = s00.y * (1.f - wx) + s10.y * wx;
        const float rx1 = s01.x * (1.f - wx) + s11.x * wx;
        const float ry1 = s01.y * (1.f - wx) + s11.y * wx;
        out.x = rx0 * (1.f - wy) + rx1 * wy;
        out.y = ry0 * (1.f - wy) + ry1 * wy;
        out.time_step = s00.time_step;
        out.layer = s00.layer;
    }
    out.x = out.x + (tx - (float)x);
    out.y = out.y + (ty - (float)y);
    out.time_step = out.time_step + time_step;
    const Ribbon current = dest[k];
    if (overwrite || current.layer < 0 || fabsf((float)current.time_step) >= fabsf((float)out.time_step))
        dest[k] = out;
}

// cumulativeAdvectionFieldToOutput, :290-304: the key colour at the end of
// each pixel's ribbon (keyFrame.pixel(x + field.x, y + field.y), the
// coordinates truncated to int; a position outside the image reads zero)
__global__ void __launch_bounds__(kKeyPix) k_ribbon_output(const Params P, const Ribbon* rib, const float4* canvas,
                                                           float4* out) {
    KEY_PIXEL_XY
    const Ribbon f = rib[k];
    float4 c = f4(0.f, 0.f, 0.f, 0.f);
    if (f.layer >= 0) {
        const int px = f2i((float)x + f.x), py = f2i((float)y + f.y);
        if (px >= 0 && py >= 0 && px < P.W && py < P.H) c = canvas[(size_t)py * P.W + px];
    }
    out[k] = c;
}

// copyFrameToKeyRibbonKernel, :2061-2097
__global__ void __launch_bounds__(kKeyPix) k_frame_to_key(const Params P, PatchPlanes work, int look_forwards,
                                                          const KeyView K) {
    KEY_PIXEL_XY
    const Arr<float4>& R = P.img.f2k[look_forwards ? 1 : 0];
    const Ribbon rb = ribbon_of(R.p ? lvl_texel_lin(R, x, y, P.hwFilter) : f4(0.f, 0.f, 0.f, 0.f));
    Patch out;
    if (rb.layer >= 0) {
        const float ox = rb.x + (float)x, oy = rb.y + (float)y;
        out = make_patch(ox, oy, screen_to_exemplar_angle(P, x, y, ox, oy, rb.layer), 1.0f, rb.layer, 1.f, 1.f);
    } else {
        const float4 r = lvl_texel(P.img.rnd, x, y);  // copyRandomKernel's toPatchXF
        out = make_patch(r.x, r.y, r.z, 0.f, f2i(r.w), 1.f, 1.f);
    }
    store_patch(work, k, out);
}

// mergeAdvectedKernel, :1938-1976: the advected offsets of both directions
// merged (at random where both are valid), else the fallback: the random
// level's fractional parts (randomFloat4's output argument, :207-213) or
// the last pass's offsets
__global__ void __launch_bounds__(kKeyPix) k_merge_advected(const Params P, int fallback, PatchPlanes work) {
    KEY_PIXEL_XY
    const Patch f = load_patch(P.adv[0].off, k), b = load_patch(P.adv[1].off, k);
    const float4 rnd = lvl_texel(P.img.rnd, x, y);
    const float4 fr = f4(rnd.x - floorf(rnd.x), rnd.y - floorf(rnd.y), rnd.z - floorf(rnd.z), rnd.w - floorf(rnd.w));
    Patch res;
    if (f.hyst > 0 && b.hyst > 0) res = (fr.x < 0.5f) ? f : b;
    else if (f.hyst > 0) res = f;
    else if (b.hyst > 0) res = b;
    else if (fallback == PT_MERGE_FALLBACK_RANDOM) res = make_patch(fr.x, fr.y, fr.z, 0.f, f2i(fr.w), 1.f, 1.f);
    else res = load_patch(P.off, k);
    store_patch(work, k, res);
}

// RibbonP() with the given layer in every texel (resetRibbonField,
// synthesisProcessor.cpp:509-517)
__global__ void k_fill_ribbons(Ribbon* r, size_t n, int layer) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Ribbon v;
    v.x = 0.f;
    v.y = 0.f;
    v.time_step = 0;
    v.layer = layer;
    r[i] = v;
}

// initializeRibbonPyramid, imagePyramid.cpp:211-235: level 0 packed as
// RGBA (toColor4: time_step, y, x, layer) ...
__global__ void k_ribbon_pack(const Ribbon* src, int w, int h, float4* dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const Ribbon r = src[(size_t)y * w + x];
    dst[(size_t)y * w + x] = f4((float)r.time_step, r.y, r.x, (float)r.layer);
}
// ... and each coarser level the top-left texel of its 2x2 block
// (RibbonP(Color4) truncates time step and layer to int) with x, y halved
__global__ void k_ribbon_down(const float4* src, int sw, float4* dst, int w, int h) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const Ribbon r = ribbon_of(src[(size_t)(2 * y) * sw + 2 * x]);
    dst[(size_t)y * w + x] = f4((float)r.time_step, r.y * 0.5f, r.x * 0.5f, (float)r.layer);
}

}  // namespace

}  // namespace ptk

namespace pt {

#define KEY_LAUNCH_CHECK() return cudaGetLastError()

cudaError_t launch_propagate_keys(const Params& P, PatchPlanes work, int jump, int key, const KeyView& K,
                                  cudaStream_t s) {
    ptk::k_propagate_keys<<<ptk::grid_of(P.lw, P.lh), dim3(32, 4), 0, s>>>(P, work, jump, key, K);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_scatter_keys(const Params& P, PatchPlanes work, int write_all, int key, const KeyView& K,
                                cudaStream_t s) {
    ptk::k_scatter_keys<<<ptk::grid_of(P.lw, P.lh), dim3(32, 4), 0, s>>>(P, work, write_all, key, K);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_accumulate_ribbon(const Params& P, int forwards, Ribbon* dest, const Ribbon* src, int time_step,
                                     int overwrite, cudaStream_t s) {
    ptk::k_accumulate_ribbon<<<ptk::grid_of(P.lw, P.lh), dim3(32, 4), 0, s>>>(P, forwards, dest, src, time_step,
                                                                             overwrite);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_ribbon_output(const Params& P, const Ribbon* rib, const float4* canvas, float4* out,
                                 cudaStream_t s) {
    ptk::k_ribbon_output<<<ptk::grid_of(P.lw, P.lh), dim3(32, 4), 0, s>>>(P, rib, canvas, out);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_frame_to_key(const Params& P, PatchPlanes work, int look_forwards, const KeyView& K,
                                cudaStream_t s) {
    ptk::k_frame_to_key<<<ptk::grid_of(P.lw, P.lh), dim3(32, 4), 0, s>>>(P, work, look_forwards, K);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_merge_advected(const Params& P, int fallback, PatchPlanes work, cudaStream_t s) {
    ptk::k_merge_advected<<<ptk::grid_of(P.lw, P.lh), dim3(32, 4), 0, s>>>(P, fallback, work);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_fill_ribbons(Ribbon* r, size_t n, int layer, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ptk::k_fill_ribbons<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(r, n, layer);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_ribbon_pack(const Ribbon* src, int w, int h, float4* dst, cudaStream_t s) {
    ptk::k_ribbon_pack<<<ptk::grid_of(w, h), dim3(32, 4), 0, s>>>(src, w, h, dst);
    KEY_LAUNCH_CHECK();
}
cudaError_t launch_ribbon_down(const float4* src, int sw, float4* dst, int w, int h, cudaStream_t s) {
    if (w < 1 || h < 1) return cudaSuccess;
    ptk::k_ribbon_down<<<ptk::grid_of(w, h), dim3(32, 4), 0, s>>>(src, sw, dst, w, h);
    KEY_LAUNCH_CHECK();
}

}  // namespace pt
