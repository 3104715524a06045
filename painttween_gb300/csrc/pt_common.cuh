// pt_common.cuh -- device functions shared by the generic kernels
// (pt_kernels.cu) and the tiled patch-distance kernels (pt_energy.cuh): the
// terms of calculateResidual and the candidate construction of the
// reference (src/PaintTweenCUDA/texSynth_kernel.cu:176-982).
#pragma once

#include "pt_device.cuh"

namespace ptk {

static __device__ __forceinline__ bool image_culled(const Params& P, int x, int y) {
    // isImagePixelCulled, :176-186
    return lay_texel(P.img.dt[P.img.cur], P, x, y) > (float)P.distTransCull;
}

// screenToExemplarAngle, :425-436
static __device__ __forceinline__ float screen_to_exemplar_angle(const Params& P, int x, int y, float ex, float ey,
                                                          int layer) {
    if (P.orientationEnabled) {
        float theta = ex_point_orient(P.ex, ex, ey, layer) - lvl_texel(P.img.orient, x, y);
        if ((double)theta > 1.57079632679489661923) return (float)((double)theta - 3.14159265358979323846);
        if ((double)theta < -1.57079632679489661923) return (float)(3.14159265358979323846 + (double)theta);
        return theta;
    }
    return 0.0f;
}

// screenToExemplarBasis, texSynth_util.h:95-104
static __device__ __forceinline__ void basis(float angle, float su, float sv, float2* b0, float2* b1) {
    float s, c;
    sincos_poly(angle, &s, &c);
    b1->x = -s * sv;
    b1->y = c * sv;
    b0->x = c * su;
    b0->y = s * su;
}

// calculateNewExemplarCoord, texSynth_util.h:106-118
static __device__ __forceinline__ void new_coord(float i, float j, float ex, float ey, float2 b0, float2 b1, float* ox,
                                          float* oy) {
    *ox = ex + fmaf(i, b0.x, j * b1.x);
    *oy = ey + fmaf(i, b0.y, j * b1.y);
}

// clampToExemplar(float*), texSynth_util.h:50-57
static __device__ __forceinline__ void clamp_to_exemplar(float* x, float* y, int w, int h) {
    if (*x < 0) *x = 0;
    if (*y < 0) *y = 0;
    if (*x >= w) *x = (float)(w - 1);
    if (*y >= h) *y = (float)(h - 1);
}

static __device__ __forceinline__ float ssd_a(float4 a, float4 b, float alpha) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dw = a.w - b.w;
    float s = dx * dx;
    s = fmaf(dy, dy, s);
    s = fmaf(dz, dz, s);
    s = fmaf(alpha * dw, dw, s);
    return s;
}
static __device__ __forceinline__ float ssd(float4 a, float4 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dw = a.w - b.w;
    float s = dx * dx;
    s = fmaf(dy, dy, s);
    s = fmaf(dz, dz, s);
    s = fmaf(dw, dw, s);
    return s;
}
static __device__ __forceinline__ float4 sub4(float4 a, float4 b) { return f4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }

// The same three functions with the channel differences formed two channels
// at a time by the packed f32x2 add (a + (-b) is a - b exactly, per
// component, in round-to-nearest); the sums of squares keep the scalar order
// x, y, z, w, so results are bit-identical.  Used where they measured faster
// (the single-candidate tap loop); the four-candidate loop keeps the scalar
// forms, which need fewer registers there.
static __device__ __forceinline__ float4 sub4p(float4 a, float4 b) {
    float2 l = __fadd2_rn(make_float2(a.x, a.y), make_float2(-b.x, -b.y));
    float2 h = __fadd2_rn(make_float2(a.z, a.w), make_float2(-b.z, -b.w));
    return f4(l.x, l.y, h.x, h.y);
}
static __device__ __forceinline__ float ssd_ap(float4 a, float4 b, float alpha) {
    const float4 d = sub4p(a, b);
    float s = d.x * d.x;
    s = fmaf(d.y, d.y, s);
    s = fmaf(d.z, d.z, s);
    s = fmaf(alpha * d.w, d.w, s);
    return s;
}
static __device__ __forceinline__ float ssdp(float4 a, float4 b) {
    const float4 d = sub4p(a, b);
    float s = d.x * d.x;
    s = fmaf(d.y, d.y, s);
    s = fmaf(d.z, d.z, s);
    s = fmaf(d.w, d.w, s);
    return s;
}

struct PixCtx {
    bool validF, validB, temporalF, temporalB;
    Patch prevF, prevB;
    float2 fb0, fb1, bb0, bb1;
    float hyst;
};

// hysteresisTerm, :506-535
static __device__ float hysteresis_term(const Params& P, int x, int y) {
    float maxD = P.maxDistortion / ldexpf(1.0f, P.level);
    const Arr<float2>& v = (P.direction == PT_FORWARD) ? P.img.velb[P.img.cur] : P.img.velf[P.img.cur];
    float2 d00 = lay_texel(v, P, x, y), d10 = lay_texel(v, P, x + 1, y);
    float2 d01 = lay_texel(v, P, x, y + 1), d11 = lay_texel(v, P, x + 1, y + 1);
    float maxX = fmaxf(d00.x, fmaxf(d01.x, fmaxf(d10.x, d11.x)));
    float maxY = fmaxf(d00.y, fmaxf(d01.y, fmaxf(d10.y, d11.y)));
    float minX = fminf(d00.x, fminf(d01.x, fminf(d10.x, d11.x)));
    float minY = fminf(d00.y, fminf(d01.y, fminf(d10.y, d11.y)));
    if ((maxX - minX) < maxD && (maxY - minY) < maxD) return P.hysteresisWeight;
    return 0.0f;
}

static __device__ void make_pixctx(const Params& P, int x, int y, PixCtx* pc) {
    size_t k = (size_t)y * P.W + x;
    pc->prevF = load_patch(P.adv[0].off, k);
    pc->prevB = load_patch(P.adv[1].off, k);
    pc->validF = pc->prevF.hyst > 0;
    pc->validB = pc->prevB.hyst > 0;
    bool td = (P.tdIn > 0.f || P.tdOut > 0.f || P.tc > 0.f);
    pc->temporalF = (P.direction == PT_FORWARD || P.direction == PT_BIDIRECTIONAL) && pc->validF && td;
    pc->temporalB = (P.direction == PT_BACKWARD || P.direction == PT_BIDIRECTIONAL) && pc->validB && td;
    if (pc->temporalF) {
        float a = screen_to_exemplar_angle(P, x, y, pc->prevF.x, pc->prevF.y, pc->prevF.layer);
        basis(a, P.scaleWU * pc->prevF.su, P.scaleWV * pc->prevF.sv, &pc->fb0, &pc->fb1);
    }
    if (pc->temporalB) {
        float a = screen_to_exemplar_angle(P, x, y, pc->prevB.x, pc->prevB.y, pc->prevB.layer);
        basis(a, P.scaleWU * pc->prevB.su, P.scaleWV * pc->prevB.sv, &pc->bb0, &pc->bb1);
    }
    pc->hyst = pc->validF ? hysteresis_term(P, x, y) : 0.0f;
}

// timeDerivativeTerms, :438-469
static __device__ float time_derivative(const Params& P, int d, const Patch& prev, float2 pb0, float2 pb1, float4 base,
                                 float4 tb, float4 canvas, float4 to, size_t k, int i, int j) {
    float4 pbase = __ldg(P.adv[d].base + k), pout = __ldg(P.adv[d].out + k);
    float px, py;
    new_coord((float)i, (float)j, prev.x, prev.y, pb0, pb1, &px, &py);
    float4 peb, peo;
    ex_sample2(P.ex, px, py, prev.layer, &peb, &peo);
    if (P.colorspace == 1) {  // :454-459
        pbase = rgb_to_lab(pbase);
        pout = rgb_to_lab(pout);
        peb = rgb_to_lab(peb);
        peo = rgb_to_lab(peo);
    }
    float r = ssd(sub4(base, pbase), sub4(tb, peb)) * P.tdIn;
    r = fmaf(ssd(sub4(canvas, pout), sub4(to, peo)), P.tdOut, r);
    r = fmaf(ssd(pout, to), P.tc, r);
    return r;
}

// coherenceTerm, :377-423
static __device__ float coherence_term(const Params& P, int x, int y, int i, int j, float tcx, float tcy, float tx,
                                float ty) {
    float4 ca = __ldg(P.off.A + (size_t)(y + j) * P.W + (x + i));
    float dx = ca.x - tcx, dy = ca.y - tcy;
    float distEx = fmaf(dy, dy, dx * dx) * (float)(1 << P.level);
    float distIm = (float)(i * i + j * j) * (float)(1 << P.level);
    float R = P.coherenceRatioRange;
    float ratio = fmaxf(1.0f / R, fminf(distEx / distIm, R));
    float lr = log_poly(ratio);
    float lR = log_poly(R);
    float Z = lR * lR;
    float Er = (lr * lr) / Z;
    float tdx = tx - tcx, tdy = ty - tcy;
    float lt = sqrtf(fmaf(tdy, tdy, tdx * tdx));
    float dtx = (lt > 1e-4f) ? tdx * (1.0f / lt) : 1.0f;
    float dty = (lt > 1e-4f) ? tdy * (1.0f / lt) : 0.0f;
    float lc = sqrtf(fmaf(dy, dy, dx * dx));
    float dcx = (lc > 1e-4f) ? dx * (1.0f / lc) : 1.0f;
    float dcy = (lc > 1e-4f) ? dy * (1.0f / lc) : 0.0f;
    float d = fmaf(dty, dcy, dtx * dcx);
    float angle = fmaxf(-1.0f, fminf(acos_poly(d), 1.0f));
    double ar = (double)P.coherenceAngleRange * 3.14159265358979323846;
    float Ea = (float)(fmin((double)angle, ar) / ar);
    return 1.0f - (1.0f - Er) * (1.0f - Ea);
}

static __device__ __forceinline__ int f2i(float v) { return (int)v; }  // cvt.rzi: saturating, NaN -> 0

// calculateResidual, :537-659
static __device__ float energy(const Params& P, int x, int y, const Patch& t, const PixCtx& pc) {
    const int r = P.r;
    float sumW = 0.0f, sum = 0.0f;
    if (pc.validF) sum = sum - pc.hyst;
    float2 b0, b1;
    basis(t.theta, P.scaleWU * t.su, P.scaleWV * t.sv, &b0, &b1);
    const float hw = (float)P.histW, hh = (float)P.histH;
    const float4* imgb = P.img.base[P.img.cur].p;
    const int imgw = P.img.base[P.img.cur].w;
    for (int i = -r; i <= r; i++) {
        for (int j = -r; j <= r; j++) {
            if (!in_rect(P, x + i, y + j)) continue;
            size_t k = (size_t)(y + j) * P.W + (x + i);
            float4 base = lin_texel_of(__ldg(imgb + (size_t)(y + j) * imgw + (x + i)), P.hwFilter);
            float4 canvas = __ldg(P.canvas + k);
            if (P.colorspace == 1) {  // :575-578
                base = rgb_to_lab(base);
                canvas = rgb_to_lab(canvas);
            }
            float tx, ty;
            new_coord((float)i, (float)j, t.x, t.y, b0, b1, &tx, &ty);
            if (tx >= hw) tx -= hw; else if (tx < 0) tx += hw;
            if (ty >= hh) ty -= hh; else if (ty < 0) ty += hh;
            float4 tb, to;
            ex_sample2(P.ex, tx, ty, t.layer, &tb, &to);
            if (P.colorspace == 1) {  // :603-606
                tb = rgb_to_lab(tb);
                to = rgb_to_lab(to);
            }
            float res = ssd_a(base, tb, P.alphaWeight) * P.inputAnalogyWeight;
            if (pc.temporalF && __ldg(&P.adv[0].off.B[k].x) > 0)
                res = res + time_derivative(P, 0, pc.prevF, pc.fb0, pc.fb1, base, tb, canvas, to, k, i, j);
            if (pc.temporalB && __ldg(&P.adv[1].off.B[k].x) > 0)
                res = res + time_derivative(P, 1, pc.prevB, pc.bb0, pc.bb1, base, tb, canvas, to, k, i, j);
            if (i == 0 && j == 0) {
                if (P.distTransWeight > 0.f) {
                    float de = ex_sample_dt(P.ex, tx, ty, t.layer) / t.sv;
                    float di = lay_texel(P.img.dt[P.img.cur], P, x, y);
                    float diff = fmaxf(0.0f, fminf(fabsf(de - di), 10.0f));  // clamp(diff, 0, 10): a NaN difference gives 10
                    res = res + diff * P.distTransWeight;
                }
                {  // histogramTerm, :486-495
                    int L = clampi(t.layer, 0, PT_MAX_STYLES - 1);
                    float sh = (float)(P.histH / P.numStyles);
                    int hx = clampi(f2i(tx), 0, P.histPitch - 1);
                    int hy = clampi(f2i(ty + sh * (float)t.layer), 0, P.histRows - 1);
                    float h = __ldg(P.hist + (size_t)hy * P.histPitch + hx);
                    float thr = P.histThreshold[L];
                    res = res + ((h > thr) ? (h - thr) * P.histSlope[L] : 0.0f);
                }
                if (P.styleObjIdWeight > 0.f) {
                    int imgID = lvl_texel(P.img.ids, x, y);
                    int styleID = ex_point_id(P.ex, tx, ty, t.layer);
                    res = res + ((imgID != styleID) ? P.styleObjIdWeight : 0.0f);
                }
            } else {
                res = fmaf(ssd_a(canvas, to, P.alphaWeight), P.canvasOutputWeight, res);
                if (P.coherenceWeight > 0.f) {
                    float c = coherence_term(P, x, y, i, j, t.x, t.y, tx, ty);
                    res = fmaf(c, P.coherenceWeight, res);
                }
            }
            float w = P.gauss[i + r] * P.gauss[j + r];
            sum = fmaf(res, w, sum);
            sumW = sumW + w;
        }
    }
    if (sumW < kEpsilon) return kBigResidual;
    return sum / sumW;
}

// profiling: one patch-distance evaluation and its in-rectangle taps,
// aggregated over the lanes that are active at this point
static __device__ __forceinline__ unsigned lane_id() {
    unsigned l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}
// every byte of the two records equal
static __device__ __forceinline__ bool same_record(const Patch& a, const Patch& b) {
    return __float_as_uint(a.x) == __float_as_uint(b.x) && __float_as_uint(a.y) == __float_as_uint(b.y) &&
           __float_as_uint(a.theta) == __float_as_uint(b.theta) && __float_as_uint(a.hyst) == __float_as_uint(b.hyst) &&
           a.layer == b.layer && __float_as_uint(a.su) == __float_as_uint(b.su) &&
           __float_as_uint(a.sv) == __float_as_uint(b.sv) && __float_as_uint(a.lumy) == __float_as_uint(b.lumy) &&
           __float_as_uint(a.luma) == __float_as_uint(b.luma);
}

// profiling counters: one evaluation and (with_taps) its taps; the tiled
// kernels count the taps they actually process after the tap loop
static __device__ __forceinline__ void count_eval(const Params& P, int x, int y, bool temporal,
                                                  bool with_taps = true) {
    int x0 = max(x - P.r, 0), x1 = min(x + P.r, P.lw - 1);
    int y0 = max(y - P.r, 0), y1 = min(y + P.r, P.lh - 1);
    unsigned taps = with_taps ? (unsigned)((x1 - x0 + 1) * (y1 - y0 + 1)) : 0u;
    unsigned mask = __activemask();
    unsigned tsum = __reduce_add_sync(mask, taps);
    unsigned ttsum = __reduce_add_sync(mask, temporal ? taps : 0u);
    if (lane_id() == (unsigned)(__ffs(mask) - 1)) {
        atomicAdd(&P.counters[0], (unsigned long long)__popc(mask));
        if (with_taps) {
            atomicAdd(&P.counters[1], (unsigned long long)tsum);
            atomicAdd(&P.counters[2], (unsigned long long)ttsum);
        }
    }
}

// test_offset + isExemplarPixelCulled, :200-205,695-721
static __device__ float test_offset(const Params& P, int x, int y, const Patch& t, float image_alpha, const PixCtx& pc) {
    float dte = ex_texel_dt(P.ex, f2i(t.x), f2i(t.y), t.layer);
    if (!((double)dte > (double)P.distTransCull * 1.25)) {
        if (!P.transparencyOk) {
            float ea = ex_sample_out_alpha(P.ex, t.x, t.y, t.layer);
            if (ea < kAlphaThreshold && image_alpha > kAlphaThreshold) return kBigResidual;
        }
        if (P.counters) count_eval(P, x, y, pc.temporalF || pc.temporalB);
        return energy(P, x, y, t, pc);
    }
    return kBigResidual;
}

// calculatePropagateOffset, :956-982 (pixelWrap with the level-0 size,
// cudaImageBuffer.h:81-87)
static __device__ __forceinline__ size_t pixel_wrap_index(const Params& P, int tx, int ty) {
    int wx = (int)((float)tx - (float)P.W * floorf((float)tx / (float)P.W));
    int wy = (int)((float)ty - (float)P.H * floorf((float)ty / (float)P.H));
    return (size_t)wy * P.W + wx;
}
static __device__ Patch propagate_offset(const Params& P, int tx, int ty, int x, int y) {
    size_t kk = pixel_wrap_index(P, tx, ty);
    float4 a = __ldg(P.off.A + kk);
    float2 sc = lvl_texel_lin(P.img.scale, tx, ty, P.hwFilter);
    float2 b0, b1;
    basis(a.z, P.scaleWU * sc.x, P.scaleWV * sc.y, &b0, &b1);
    float ex, ey;
    new_coord((float)x - (float)tx, (float)y - (float)ty, a.x, a.y, b0, b1, &ex, &ey);
    clamp_to_exemplar(&ex, &ey, P.ex.w, P.ex.h);
    int layer = __float_as_int(a.w);
    float ang = screen_to_exemplar_angle(P, x, y, ex, ey, layer);
    float2 s2 = lvl_texel_lin(P.img.scale, x, y, P.hwFilter);
    return make_patch(ex, ey, ang, 0.0f, layer, s2.x, s2.y);
}

static __device__ __forceinline__ uint32_t hash32(uint32_t a) {
    a ^= a >> 16; a *= 0x7feb352dU; a ^= a >> 15; a *= 0x846ca68bU; a ^= a >> 16;
    return a;
}
static __device__ __forceinline__ float counter_u01(uint32_t seed, uint32_t level, uint32_t x, uint32_t y, uint32_t n) {
    uint32_t h = hash32(seed ^ hash32(level * 0x9E3779B9U ^ hash32(x * 0x85EBCA6BU ^ hash32(y * 0xC2B2AE35U ^ n))));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}


}  // namespace ptk
