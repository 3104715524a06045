/*
 * pt_oracle.c -- CPU oracle for PaintTween's offset-field synthesis.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only to check the
 * library's results (or as the timed CPU baseline); the product library
 * never calls it.
 *
 * What it is: a scalar C restatement of the reference's hot path
 * (src/PaintTweenCUDA/texSynth_kernel.cu, texSynth_util.h, cudaImageBuffer.h,
 * convolution.cu, synthesisFrame.cpp, downsample.cpp), operating on the same
 * buffer model as the reference: full-resolution buffers whose level-L data
 * occupies the top-left (W>>L) x (H>>L) rectangle, persistent across levels
 * and frames.  Every function cites the reference lines it follows.
 *
 * Parity status: pinned at the helper level, unpinned end to end.  The
 * reference ships no tests, golden vectors or fixtures for this path, and its
 * CUDA kernels do not compile with the installed CUDA 13 (legacy texture
 * references and cudaThreadSynchronize are removed), so no end-to-end
 * reference output can be produced.  Its helper header texSynth_util.h does
 * compile: the pto_basis / pto_new_coord / pto_clamp_to_exemplar / pto_ssd /
 * pto_ribbon_of / pto_to_patchxf / pto_rgb_to_lab hooks are checked against it, built for the
 * host (g++) and for the GPU (nvcc cubin); pto_pixel_wrap / pto_in_bounds
 * against cudaImageBuffer.h and the pyramids against downsample.cpp, both
 * built for the host.  The glibc rand() restatement is
 * pinned against the C library's rand().
 *
 * Arithmetic contract (shared, by specification, with the CUDA kernels so the
 * two agree bit for bit): FP32 everywhere the reference uses float, with
 *  - contraction off (-ffp-contract=off) and fused multiply-adds written out
 *    with fmaf() at the places listed in the comments;
 *  - bilinear sampling with exact FP32 weights (the reference uses the
 *    texture unit's 1.8 fixed-point weights, which no CPU can reproduce);
 *  - sin/cos/atan2/log/acos from the polynomial routines below (Cody-Waite
 *    reduction + Taylor series), not from libm, so CPU and GPU agree;
 *  - double precision exactly where the reference's C++ promotes to double
 *    (comparisons and sums with M_PI, M_PI_2, 10e-7, 2.828, 0.2126 ...).
 * An FP64 energy (pto_energy_f64) serves as the accuracy reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/painttween.h"

#define ALPHA_THRESHOLD 0.99f /* types.h:39 */
#define EPSILON_F 0.000001f   /* types.h:38 */
#define BIG_RESIDUAL ((float)10e30)

/* float -> int conversion with CUDA's cvt.rzi.s32.f32 semantics: truncation,
 * saturation, NaN -> 0 (plain C conversion is undefined there) */
static inline int f2i(float v) {
    if (v != v) return 0;
    if (v >= 2147483647.0f) return 2147483647;
    if (v <= -2147483648.0f) return (int)(-2147483647 - 1);
    return (int)v;
}

typedef struct { float x, y, z, w; } f4;
typedef struct { float x, y; } f2;

typedef struct {
    int W, H;            /* level-0 image size (full-res buffers) */
    int SW, SH, NS;      /* level-0 style size, number of styles */
    pt_params p;
    float gauss[64];     /* unnormalised Gaussian, convolution.cu:37-60 */
    int cur;             /* gCurrentBuffer */
    /* image-side layered arrays: 2 layers, full resolution, zero outside the
     * uploaded level rectangle (texSynth_kernel.cu:2120-2126) */
    f4* img_base[2];
    float* img_dt[2];
    f2* vel_f[2];
    f2* vel_b[2];
    /* non-layered level-size arrays (re-initialised per upload) */
    float* img_orient; int io_w, io_h;
    f2* img_scale; int is_w, is_h;
    int32_t* img_ids; int ii_w, ii_h;
    f4* rnd; int rn_w, rn_h;
    /* exemplar level arrays: ns layers of ew x eh */
    int ew, eh, ens;
    f4* ex_base; f4* ex_out; float* ex_orient; float* ex_dt; int32_t* ex_ids;
    /* working buffers, full resolution */
    pt_patchxf* off_base; pt_patchxf* off_work;
    float* res_base; float* res_work;
    f4* canvas;
    float* hist_base; float* hist_work; /* SW x (SH*NS) */
    pt_patchxf* adv_off[2]; f4* adv_base[2]; f4* adv_out[2];
    float* adv_res[2]; int32_t* adv_ts[2]; /* [0] = F, [1] = B */
    /* keyframe interpolation: key-to-key cumulative fields [0] = B, [1] = F
     * (layered by key index, cf_w x cf_h, linear filter), frame-to-key
     * ribbons [0] = B, [1] = F (level arrays), the ribbon field pair */
    f4* cumul[2]; int cf_w, cf_h, cf_n;
    f4* f2k[2]; int fk_w[2], fk_h[2];
    pt_ribbon* rib_base; pt_ribbon* rib_work;
    int threads;
} pto;

/* ------------------------------------------------------------------------ */
/* polynomial elementary functions (shared contract with the CUDA side)     */
/* ------------------------------------------------------------------------ */

/* sin/cos: k = rint(t*2/pi), r = t - k*pi/2 (two-term Cody-Waite with fma),
 * Taylor series to r^9 (sin) and r^10 (cos) on |r| <= pi/4. */
static void pt_sincosf(float t, float* s, float* c) {
    const float two_over_pi = 0x1.45f306p-1f;
    const float pio2_hi = 0x1.921fb6p+0f;
    const float pio2_lo = -0x1.777a5cp-25f;
    float k = rintf(t * two_over_pi);
    float r = fmaf(-k, pio2_hi, t);
    r = fmaf(-k, pio2_lo, r);
    float r2 = r * r;
    float ps = fmaf(r2, (float)(1.0 / 362880.0), (float)(-1.0 / 5040.0));
    ps = fmaf(r2, ps, (float)(1.0 / 120.0));
    ps = fmaf(r2, ps, (float)(-1.0 / 6.0));
    ps = ps * r2;
    float sr = fmaf(r, ps, r);
    float pc = fmaf(r2, (float)(-1.0 / 3628800.0), (float)(1.0 / 40320.0));
    pc = fmaf(r2, pc, (float)(-1.0 / 720.0));
    pc = fmaf(r2, pc, (float)(1.0 / 24.0));
    pc = fmaf(r2, pc, -0.5f);
    float cr = fmaf(r2, pc, 1.0f);
    int q = f2i(k) & 3;
    switch (q) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

/* atan on [0,1]: for u > tan(pi/8) use atan(u) = pi/4 + atan((u-1)/(u+1));
 * Taylor series to v^19 on |v| <= tan(pi/8). */
static float pt_atan01f(float u) {
    float off = 0.0f;
    float v = u;
    if (u > 0x1.a8279ap-2f) { /* 0.41421356 */
        v = (u - 1.0f) / (u + 1.0f);
        off = 0x1.921fb6p-1f; /* pi/4 */
    }
    float v2 = v * v;
    float p = (float)(-1.0 / 19.0);
    p = fmaf(v2, p, (float)(1.0 / 17.0));
    p = fmaf(v2, p, (float)(-1.0 / 15.0));
    p = fmaf(v2, p, (float)(1.0 / 13.0));
    p = fmaf(v2, p, (float)(-1.0 / 11.0));
    p = fmaf(v2, p, (float)(1.0 / 9.0));
    p = fmaf(v2, p, (float)(-1.0 / 7.0));
    p = fmaf(v2, p, (float)(1.0 / 5.0));
    p = fmaf(v2, p, (float)(-1.0 / 3.0));
    p = p * v2;
    return off + fmaf(v, p, v);
}

static float pt_atan2f(float y, float x) {
    const float pi = 0x1.921fb6p+1f;
    const float pio2 = 0x1.921fb6p+0f;
    float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f) {
        float r = signbit(x) ? pi : 0.0f;
        return signbit(y) ? -r : r;
    }
    float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    float a = pt_atan01f(mn / mx);
    if (ay > ax) a = pio2 - a;
    if (signbit(x)) a = pi - a;
    return signbit(y) ? -a : a;
}

/* natural log: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
 * log(m) = 2 atanh(s), s = (m-1)/(m+1), series to s^11. */
static float pt_logf(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int e;
    float m = frexpf(x, &e); /* m in [0.5, 1) */
    if (m < 0x1.6a09e6p-1f) { m = m * 2.0f; e -= 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = (float)(1.0 / 11.0);
    p = fmaf(s2, p, (float)(1.0 / 9.0));
    p = fmaf(s2, p, (float)(1.0 / 7.0));
    p = fmaf(s2, p, (float)(1.0 / 5.0));
    p = fmaf(s2, p, (float)(1.0 / 3.0));
    p = p * s2;
    float lm = 2.0f * fmaf(s, p, s);
    float fe = (float)e;
    return fmaf(fe, 0x1.62e430p-1f, fmaf(fe, -0x1.05c610p-29f, lm));
}

/* double log, exp and pow for the Lab conversion (shared contract with the
 * CUDA side): log by frexp to m in [sqrt(1/2), sqrt(2)) and the atanh series
 * 2 (s + s^3/3 + ... + s^23/23), s = (m-1)/(m+1); exp by k = rint(y/ln2),
 * r = y - k ln2 (two-part ln2) and the Taylor series to r^22; pow(x, y) =
 * exp(y log x) for x > 0. */
static double pt_logd(double x) {
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) { m = m * 2.0; e -= 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double p = 1.0 / 23.0;
    for (int k = 21; k >= 3; k -= 2) p = fma(s2, p, 1.0 / (double)k);
    p = p * s2;
    double lm = 2.0 * fma(s, p, s);
    double fe = (double)e;
    return fma(fe, 6.93147180369123816490e-01, fma(fe, 1.90821492927058770002e-10, lm));
}
static double pt_expd(double y) {
    double k = rint(y * 1.44269504088896338700);
    double r = fma(-k, 6.93147180369123816490e-01, y);
    r = fma(-k, 1.90821492927058770002e-10, r);
    double p = 1.0; /* 1 + r/1 (1 + r/2 (1 + ... (1 + r/22))) */
    for (int n = 22; n >= 1; n--) p = fma(r / (double)n, p, 1.0);
    return ldexp(p, (int)k);
}
static double pt_powd(double x, double y) {
    if (!(x > 0.0)) return (x == 0.0) ? 0.0 : NAN;
    return pt_expd(y * pt_logd(x));
}

/* RGBtoLAB with Clinear and f_Lab, texSynth_util.h:175-192,220-246 (D65;
 * the double-precision steps are the ones the C++ promotes to double) */
static float lab_clinear(float c) {
    const float a = 0.055f;
    if ((double)c > 0.04045) return (float)pt_powd((double)(c + a) / (1.0 + (double)a), 2.4);
    return (float)((double)c / 12.92);
}
static float lab_f(float t) {
    const float lim = (float)pt_powd((double)(float)(6.0 / 29.0), 3.0);
    if (t > lim) return (float)pt_powd((double)t, (double)(float)(1.0 / 3.0));
    const float sq = (float)pt_powd((double)(float)(29.0 / 6.0), 2.0);
    return (float)((1.0 / 3.0) * (double)sq * (double)t + (4.0 / 29.0));
}
static f4 rgb_to_lab(f4 c) {
    const float refX = 95.047f, refY = 100.0f, refZ = 108.883f;
    float rl = 100.0f * lab_clinear(c.x), gl = 100.0f * lab_clinear(c.y), bl = 100.0f * lab_clinear(c.z);
    float X = (float)(0.4124 * (double)rl + 0.3576 * (double)gl + 0.1805 * (double)bl);
    float Y = (float)(0.2126 * (double)rl + 0.7152 * (double)gl + 0.0722 * (double)bl);
    float Z = (float)(0.0193 * (double)rl + 0.1192 * (double)gl + 0.9505 * (double)bl);
    float fy = lab_f(Y / refY);
    f4 o;
    o.x = (116.f * fy - 16.0f) / 100.f;
    o.y = (500.f * (lab_f(X / refX) - fy) + 100.0f) / 200.f;
    o.z = (200.f * (fy - lab_f(Z / refZ)) + 100.0f) / 200.f;
    o.w = c.w;
    return o;
}
float pto_rgb_to_lab(const float* in, float* out) {
    f4 c = {in[0], in[1], in[2], in[3]};
    f4 o = rgb_to_lab(c);
    out[0] = o.x; out[1] = o.y; out[2] = o.z; out[3] = o.w;
    return o.x;
}
double pto_powd(double x, double y) { return pt_powd(x, y); }

/* asin on [0, 1/2] by its Taylor series (12 terms). */
static float pt_asin_small(float x) {
    static const double c[12] = {
        1.0 / 6.0, 3.0 / 40.0, 15.0 / 336.0, 105.0 / 3456.0, 945.0 / 42240.0,
        10395.0 / 599040.0, 135135.0 / 9676800.0, 2027025.0 / 175472640.0,
        34459425.0 / 3530096640.0, 654729075.0 / 78033715200.0,
        13749310575.0 / 1880240947200.0, 316234143225.0 / 49049763430400.0};
    float z = x * x;
    float p = (float)c[11];
    for (int i = 10; i >= 0; --i) p = fmaf(z, p, (float)c[i]);
    p = p * z;
    return fmaf(x, p, x);
}

static float pt_acosf(float x) {
    const float pi = 0x1.921fb6p+1f;
    const float pio2 = 0x1.921fb6p+0f;
    if (!(fabsf(x) <= 1.0f)) return NAN;
    if (fabsf(x) <= 0.5f) return pio2 - pt_asin_small(x);
    float t = sqrtf((1.0f - fabsf(x)) * 0.5f);
    float a = 2.0f * pt_asin_small(t);
    return (x > 0.0f) ? a : pi - a;
}

/* IEEE binary16 round trip (round to nearest even), the EXR half channel. */
static float pt_half_roundtrip(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    uint32_t sign = u & 0x80000000u;
    uint32_t a = u & 0x7fffffffu;
    uint16_t h;
    if (a >= 0x7f800000u) {
        h = (uint16_t)((a > 0x7f800000u) ? 0x7e00 : 0x7c00);
    } else if (a >= 0x477ff000u) { /* >= 65520 rounds to inf */
        h = 0x7c00;
    } else if (a < 0x38800000u) { /* subnormal or zero half */
        float af;
        memcpy(&af, &a, 4);
        float scaled = af * 16777216.0f; /* 2^24: half subnormal unit */
        h = (uint16_t)rintf(scaled);
    } else {
        uint32_t mant = a & 0x007fffffu;
        int32_t exp = (int32_t)(a >> 23) - 127 + 15;
        uint32_t hm = mant >> 13;
        uint32_t rest = mant & 0x1fffu;
        uint32_t hv = ((uint32_t)exp << 10) | hm;
        if (rest > 0x1000u || (rest == 0x1000u && (hv & 1u))) hv += 1;
        h = (uint16_t)hv;
    }
    /* back to float */
    uint32_t he = (h >> 10) & 0x1f, hmant = h & 0x3ff;
    float out;
    if (he == 0) {
        out = (float)hmant / 16777216.0f;
    } else if (he == 31) {
        out = hmant ? NAN : INFINITY;
    } else {
        uint32_t bits = ((he - 15 + 127) << 23) | (hmant << 13);
        memcpy(&out, &bits, 4);
    }
    return sign ? -out : out;
}

/* counter-based hash of the PT_RNG_COUNTER mode (an integer mixing
 * function: xor-shift / multiply rounds) */
static inline uint32_t hash32(uint32_t a) {
    a ^= a >> 16; a *= 0x7feb352dU; a ^= a >> 15; a *= 0x846ca68bU; a ^= a >> 16;
    return a;
}
static inline float counter_u01(uint32_t seed, uint32_t pass, uint32_t x, uint32_t y, uint32_t n) {
    uint32_t h = hash32(seed ^ hash32(pass * 0x9E3779B9U ^ hash32(x * 0x85EBCA6BU ^ hash32(y * 0xC2B2AE35U ^ n))));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

/* ------------------------------------------------------------------------ */
/* fetches                                                                  */
/* ------------------------------------------------------------------------ */

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static inline int lvl_w(const pto* o, int level) { return o->W >> level; }
static inline int lvl_h(const pto* o, int level) { return o->H >> level; }
/* CudaImageBufferDevice::inBounds, cudaImageBuffer.h:117-120 */
static inline int in_bounds(int W, int H, int x, int y, int level, int border) {
    return x >= border && y >= border && x < (W >> level) - border && y < (H >> level) - border;
}
static inline int in_rect(const pto* o, int x, int y, int level, int border) {
    return in_bounds(o->W, o->H, x, y, level, border);
}
/* CudaImageBufferDevice::pixelWrap, cudaImageBuffer.h:81-87: the pixel index
 * of (x, y) wrapped by the buffer's (level-0) size */
static inline size_t pixel_wrap_index(int W, int H, int x, int y) {
    int wx = (int)((float)x - (float)W * floorf((float)x / (float)W));
    int wy = (int)((float)y - (float)H * floorf((float)y / (float)H));
    return (size_t)wy * W + wx;
}
/* test hooks for the two above */
int pto_in_bounds(int W, int H, int x, int y, int level, int border) { return in_bounds(W, H, x, y, level, border); }
long long pto_pixel_wrap(int W, int H, int x, int y) { return (long long)pixel_wrap_index(W, H, x, y); }

/* integer coordinate of a point-filtered fetch at unnormalised u (+0.5 as
 * PYRAMID_FETCH adds, cudaImagePyramid.h:102,108), clamp addressing */
static inline int point_index(float u, int n) {
    float f = floorf(u + 0.5f);
    f = fminf(fmaxf(f, -1.0f), (float)n);
    return clampi((int)f, 0, n - 1);
}

typedef struct {
    int x0, x1, y0, y1;
    float w00, w10, w01, w11;   /* PT_FILTER_EXACT: FP32 weights */
    int hw;                     /* PT_FILTER_TEXTURE */
    int q00, q10, q01, q11;     /* texture-unit weights, in 1/256 */
    int r00, r10, r01, r11;     /* unrounded weight products, nonzero flags */
} bl_t;

/* bilinear footprint at unnormalised (u,v) with clamp to (n x m): the texel
 * coordinate the reference's fetch macros form, u + 0.5, and the texture
 * unit's lower texel floor(u + 0.5 - 0.5) with fraction a.
 *
 * hw: the texture unit's weights.  The fractions are quantised to 1/256
 * rounding half up (A = floor(256 a + 1/2), B likewise), the corner weights
 * are q11 = floor((A B + 128) / 256), q10 = A - q11, q01 = B - q11 and
 * q00 = 256 - A - B + q11.  This rule, and the sum in bl1, reproduce the
 * bits of GB300's bilinear fetches of 1-, 2- and 4-channel float textures
 * (layered arrays and pitched memory) on every one of 4.3 million sampled
 * channels, special values included (a fixture of those samples is checked
 * in tests/test_oracle.py, and the GPU test compares live fetches). */
static inline bl_t bl_setup_at(float xs, float ys, int n, int m, int hw) {
    bl_t b;
    float xb = xs - 0.5f, yb = ys - 0.5f;
    float fx = floorf(xb), fy = floorf(yb);
    float a = xb - fx, c = yb - fy;
    fx = fminf(fmaxf(fx, -1.0f), (float)n);
    fy = fminf(fmaxf(fy, -1.0f), (float)m);
    int ix = (int)fx, iy = (int)fy;
    b.x0 = clampi(ix, 0, n - 1); b.x1 = clampi(ix + 1, 0, n - 1);
    b.y0 = clampi(iy, 0, m - 1); b.y1 = clampi(iy + 1, 0, m - 1);
    float oa = 1.0f - a, oc = 1.0f - c;
    b.w00 = oa * oc; b.w10 = a * oc; b.w01 = oa * c; b.w11 = a * c;
    b.hw = hw;
    /* a coordinate of NaN or +-inf reads the edge texel (NaN the low edge,
     * as measured): the clamps above give its index, the fraction is 0 */
    if (a != a) a = 0.0f;
    if (c != c) c = 0.0f;
    int A = (int)floor((double)a * 256.0 + 0.5), B = (int)floor((double)c * 256.0 + 0.5);
    b.q11 = (A * B + 128) >> 8;
    b.q10 = A - b.q11; b.q01 = B - b.q11; b.q00 = 256 - A - B + b.q11;
    b.r00 = (256 - A) * (256 - B) != 0; b.r10 = A * (256 - B) != 0;
    b.r01 = (256 - A) * B != 0; b.r11 = A * B != 0;
    return b;
}
static inline bl_t bl_setup(float u, float v, int n, int m, int hw) { return bl_setup_at(u + 0.5f, v + 0.5f, n, m, hw); }

/* A NaN produced by device arithmetic (0/0 here) is the GPU's canonical
 * quiet NaN, bits 0x7fffffff, where the host's x86 arithmetic produces
 * 0xffc00000; NaN inputs pass through arithmetic unchanged on both.  The
 * reference stores such a NaN offset when a pixel's average-offset candidate
 * has no same-layer neighbour and its energy is still the best (with
 * texture filtering a NaN coordinate reads the edge texel). */
static inline float gpu_nan(float v) {
    if (v == v) return v;
    uint32_t u = 0x7fffffffu;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* a texel as the texture unit reads it: subnormals as (signed) zero */
static inline float tex_ftz(float t) { return fpclassify(t) == FP_SUBNORMAL ? copysignf(0.0f, t) : t; }

static inline uint32_t f_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float f_of_bits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* the texture unit's weighted sum of one channel: the texels with a nonzero
 * weight are aligned to the largest exponent among them and truncated
 * toward zero to 28 bits below it, summed exactly with the 1/256 weights,
 * and the sum is rounded to float ties away from zero; a sum of zeros is -0
 * only if every texel with a nonzero unrounded weight is negative-signed.
 * Integer arithmetic throughout: a normal texel t = M * 2^(e - 24) with the
 * 24-bit significand M and frexp exponent e, so t * 2^(28 - E) = M * 2^(4 +
 * e - E). */
static inline float hw_sum(const bl_t* b, float t00, float t10, float t01, float t11) {
    const float t[4] = {tex_ftz(t00), tex_ftz(t10), tex_ftz(t01), tex_ftz(t11)};
    const int q[4] = {b->q00, b->q10, b->q01, b->q11};
    const int r[4] = {b->r00, b->r10, b->r01, b->r11};
    int E = -1000;
    for (int k = 0; k < 4; k++) {
        uint32_t u = f_bits(t[k]);
        int e = (int)((u >> 23) & 0xffu) - 126;
        if (q[k] > 0 && (u & 0x7fffffffu) != 0u && e > E) E = e;
    }
    if (E == -1000) {
        int neg = 1;
        for (int k = 0; k < 4; k++)
            if (r[k] && !(f_bits(t[k]) >> 31)) neg = 0;
        return neg ? -0.0f : 0.0f;
    }
    /* fast path: every weighted texel within 2^4 of the largest, so none is
     * truncated; the sum of the four 33-bit products is exact in double */
    int Emin = 1000;
    for (int k = 0; k < 4; k++) {
        uint32_t u = f_bits(t[k]);
        int e = (int)((u >> 23) & 0xffu) - 126;
        if (q[k] > 0 && (u & 0x7fffffffu) != 0u && e < Emin) Emin = e;
    }
    if (E - Emin <= 4) {
        double d = 0.0;
        for (int k = 0; k < 4; k++)
            if (q[k] > 0) d += (double)q[k] * (double)t[k];
        d *= 0x1p-8;
        float f = (float)d;
        if ((double)f == d) return f;
        float lo, hi;
        if (fabs((double)f) > fabs(d)) { hi = f; lo = nextafterf(f, 0.0f); }
        else { lo = f; hi = nextafterf(f, d > 0 ? INFINITY : -INFINITY); }
        double mid = ((double)lo + (double)hi) * 0.5;
        return fabs(d) >= fabs(mid) ? hi : lo;  /* ties away from zero */
    }
    long long S = 0;
    for (int k = 0; k < 4; k++) {
        uint32_t u = f_bits(t[k]);
        if (q[k] <= 0 || (u & 0x7fffffffu) == 0u) continue;
        int e = (int)((u >> 23) & 0xffu) - 126;
        long long M = (long long)((u & 0x7fffffu) | 0x800000u);
        int sh = 4 + e - E;
        long long m = sh >= 0 ? (M << sh) : (sh > -25 ? (M >> -sh) : 0);
        S += (long long)q[k] * ((u >> 31) ? -m : m);
    }
    /* S * 2^(E - 36) to float, ties away from zero */
    if (S == 0) return 0.0f;
    int neg = S < 0;
    unsigned long long mag = (unsigned long long)(neg ? -S : S);
    int msb = 63 - __builtin_clzll(mag);
    int e2 = E - 36;
    if (msb > 23) {
        int drop = msb - 23;
        unsigned long long rem = mag & ((1ull << drop) - 1ull);
        mag >>= drop;
        if (rem >= (1ull << (drop - 1))) mag += 1ull;
        e2 += drop;
    }
    float f = ldexpf((float)mag, e2);
    return neg ? -f : f;
}

static inline float bl1(const bl_t* b, float t00, float t10, float t01, float t11) {
    if (b->hw) return hw_sum(b, t00, t10, t01, t11);
    float r = t00 * b->w00;
    r = fmaf(t10, b->w10, r);
    r = fmaf(t01, b->w01, r);
    r = fmaf(t11, b->w11, r);
    return r;
}
static inline f4 bl4(const bl_t* b, f4 a, f4 c, f4 d, f4 e) {
    f4 r;
    r.x = bl1(b, a.x, c.x, d.x, e.x);
    r.y = bl1(b, a.y, c.y, d.y, e.y);
    r.z = bl1(b, a.z, c.z, d.z, e.z);
    r.w = bl1(b, a.w, c.w, d.w, e.w);
    return r;
}
/* test hook: bilinear fetches of a float texture of C channels (L layers of
 * H x W, clamp addressing) at the texture coordinates q[3i], q[3i+1] (as
 * passed to the fetch, texel centres at +0.5) of layer q[3i+2], with the
 * texture unit's arithmetic (hw) or exact FP32 */
void pto_tex_fetch(const float* tex, int W, int H, int L, int C, const float* q, int n, int hw, float* out) {
    for (int i = 0; i < n; i++) {
        bl_t b = bl_setup_at(q[3 * i], q[3 * i + 1], W, H, hw);
        int l = clampi((int)q[3 * i + 2], 0, L - 1);
        const float* T = tex + (size_t)l * W * H * C;
        for (int c = 0; c < C; c++)
            out[(size_t)i * C + c] = bl1(&b, T[((size_t)b.y0 * W + b.x0) * C + c], T[((size_t)b.y0 * W + b.x1) * C + c],
                                         T[((size_t)b.y1 * W + b.x0) * C + c], T[((size_t)b.y1 * W + b.x1) * C + c]);
    }
}

/* a texel of a linearly filtered input read at its centre */
static inline float lin_texel(const pto* o, float t) { return o->p.filterMode == PT_FILTER_TEXTURE ? tex_ftz(t) : t; }
static inline f4 lin_texel4(const pto* o, f4 t) {
    if (o->p.filterMode != PT_FILTER_TEXTURE) return t;
    t.x = tex_ftz(t.x); t.y = tex_ftz(t.y); t.z = tex_ftz(t.z); t.w = tex_ftz(t.w);
    return t;
}

static inline int ex_layer(const pto* o, int layer) { return clampi(layer, 0, o->ens - 1); }

static inline void ex_sample2(const pto* o, float u, float v, int layer, f4* base, f4* out) {
    bl_t b = bl_setup(u, v, o->ew, o->eh, o->p.filterMode == PT_FILTER_TEXTURE);
    size_t L = (size_t)ex_layer(o, layer) * o->ew * o->eh;
    const f4* B = o->ex_base + L;
    const f4* O = o->ex_out + L;
    size_t i00 = (size_t)b.y0 * o->ew + b.x0, i10 = (size_t)b.y0 * o->ew + b.x1;
    size_t i01 = (size_t)b.y1 * o->ew + b.x0, i11 = (size_t)b.y1 * o->ew + b.x1;
    *base = bl4(&b, B[i00], B[i10], B[i01], B[i11]);
    *out = bl4(&b, O[i00], O[i10], O[i01], O[i11]);
}
static inline f4 ex_sample_out(const pto* o, float u, float v, int layer) {
    bl_t b = bl_setup(u, v, o->ew, o->eh, o->p.filterMode == PT_FILTER_TEXTURE);
    const f4* O = o->ex_out + (size_t)ex_layer(o, layer) * o->ew * o->eh;
    return bl4(&b, O[(size_t)b.y0 * o->ew + b.x0], O[(size_t)b.y0 * o->ew + b.x1],
               O[(size_t)b.y1 * o->ew + b.x0], O[(size_t)b.y1 * o->ew + b.x1]);
}
static inline float ex_sample_dt(const pto* o, float u, float v, int layer) {
    bl_t b = bl_setup(u, v, o->ew, o->eh, o->p.filterMode == PT_FILTER_TEXTURE);
    const float* D = o->ex_dt + (size_t)ex_layer(o, layer) * o->ew * o->eh;
    return bl1(&b, D[(size_t)b.y0 * o->ew + b.x0], D[(size_t)b.y0 * o->ew + b.x1],
               D[(size_t)b.y1 * o->ew + b.x0], D[(size_t)b.y1 * o->ew + b.x1]);
}
static inline float ex_texel_dt(const pto* o, int x, int y, int layer) {
    x = clampi(x, 0, o->ew - 1); y = clampi(y, 0, o->eh - 1);
    return lin_texel(o, o->ex_dt[(size_t)ex_layer(o, layer) * o->ew * o->eh + (size_t)y * o->ew + x]);
}
static inline float ex_point_orient(const pto* o, float u, float v, int layer) {
    int x = point_index(u, o->ew), y = point_index(v, o->eh);
    return o->ex_orient[(size_t)ex_layer(o, layer) * o->ew * o->eh + (size_t)y * o->ew + x];
}
static inline int ex_point_id(const pto* o, float u, float v, int layer) {
    int x = point_index(u, o->ew), y = point_index(v, o->eh);
    return o->ex_ids[(size_t)ex_layer(o, layer) * o->ew * o->eh + (size_t)y * o->ew + x];
}

/* image-side layered arrays: full-resolution extent */
static inline f4 img_texel(const pto* o, int layer, int x, int y) {
    x = clampi(x, 0, o->W - 1); y = clampi(y, 0, o->H - 1);
    return lin_texel4(o, o->img_base[layer][(size_t)y * o->W + x]);
}
static inline float dt_texel(const pto* o, int layer, int x, int y) {
    x = clampi(x, 0, o->W - 1); y = clampi(y, 0, o->H - 1);
    return lin_texel(o, o->img_dt[layer][(size_t)y * o->W + x]);
}
static inline f2 vel_texel(const f2* v, const pto* o, int x, int y) {
    x = clampi(x, 0, o->W - 1); y = clampi(y, 0, o->H - 1);
    f2 t = v[(size_t)y * o->W + x];
    t.x = lin_texel(o, t.x); t.y = lin_texel(o, t.y);
    return t;
}
static inline f2 vel_bilinear(const f2* v, const pto* o, float u, float w) {
    bl_t b = bl_setup(u, w, o->W, o->H, o->p.filterMode == PT_FILTER_TEXTURE);
    f2 a = v[(size_t)b.y0 * o->W + b.x0], c = v[(size_t)b.y0 * o->W + b.x1];
    f2 d = v[(size_t)b.y1 * o->W + b.x0], e = v[(size_t)b.y1 * o->W + b.x1];
    f2 r;
    r.x = bl1(&b, a.x, c.x, d.x, e.x);
    r.y = bl1(&b, a.y, c.y, d.y, e.y);
    return r;
}
static inline f4 img_bilinear(const pto* o, int layer, float u, float w) {
    bl_t b = bl_setup(u, w, o->W, o->H, o->p.filterMode == PT_FILTER_TEXTURE);
    const f4* B = o->img_base[layer];
    return bl4(&b, B[(size_t)b.y0 * o->W + b.x0], B[(size_t)b.y0 * o->W + b.x1],
               B[(size_t)b.y1 * o->W + b.x0], B[(size_t)b.y1 * o->W + b.x1]);
}
/* non-layered level-size arrays, integer coordinates */
static inline float orient_texel(const pto* o, int x, int y) {
    x = clampi(x, 0, o->io_w - 1); y = clampi(y, 0, o->io_h - 1);
    return o->img_orient[(size_t)y * o->io_w + x];
}
static inline f2 scale_texel(const pto* o, int x, int y) {
    x = clampi(x, 0, o->is_w - 1); y = clampi(y, 0, o->is_h - 1);
    f2 t = o->img_scale[(size_t)y * o->is_w + x];
    t.x = lin_texel(o, t.x); t.y = lin_texel(o, t.y);
    return t;
}
static inline int id_texel(const pto* o, int x, int y) {
    x = clampi(x, 0, o->ii_w - 1); y = clampi(y, 0, o->ii_h - 1);
    return o->img_ids[(size_t)y * o->ii_w + x];
}
static inline f4 rnd_texel(const pto* o, int x, int y) {
    if (!o->rnd) { f4 z = {0, 0, 0, 0}; return z; } /* never uploaded: zero */
    x = clampi(x, 0, o->rn_w - 1); y = clampi(y, 0, o->rn_h - 1);
    return o->rnd[(size_t)y * o->rn_w + x];
}

/* ------------------------------------------------------------------------ */
/* device-function restatements                                             */
/* ------------------------------------------------------------------------ */

static inline int image_culled(const pto* o, int x, int y) {
    /* isImagePixelCulled, texSynth_kernel.cu:176-186 */
    return dt_texel(o, o->cur, x, y) > (float)o->p.distTransCull;
}

/* screenToExemplarAngle, texSynth_kernel.cu:425-436 */
static inline float screen_to_exemplar_angle(const pto* o, int x, int y, float ex, float ey, int layer) {
    if (o->p.orientationEnabled) {
        float theta = ex_point_orient(o, ex, ey, layer) - orient_texel(o, x, y);
        if ((double)theta > M_PI_2) return (float)((double)theta - M_PI);
        if ((double)theta < -M_PI_2) return (float)(M_PI + (double)theta);
        return theta;
    }
    return 0.0f;
}

/* screenToExemplarBasis, texSynth_util.h:95-104 */
static inline void basis(float angle, float su, float sv, f2* b0, f2* b1) {
    float s, c;
    pt_sincosf(angle, &s, &c);
    b1->x = -s * sv;
    b1->y = c * sv;
    b0->x = c * su;
    b0->y = s * su;
}

/* calculateNewExemplarCoord, texSynth_util.h:106-118: e + (i*b0 + j*b1),
 * the first product fused with the second as nvcc contracts the reference's
 * expression (checked against the reference's helper run on the GPU) */
static inline void new_coord(float i, float j, float ex, float ey, f2 b0, f2 b1, float* ox, float* oy) {
    *ox = ex + fmaf(i, b0.x, j * b1.x);
    *oy = ey + fmaf(i, b0.y, j * b1.y);
}

/* clampToExemplar(float*), texSynth_util.h:50-57 */
static inline void clamp_to_exemplar(float* x, float* y, int w, int h) {
    if (*x < 0) *x = 0;
    if (*y < 0) *y = 0;
    if (*x >= w) *x = (float)(w - 1);
    if (*y >= h) *y = (float)(h - 1);
}

/* sumSquaredDiff with alpha weight, texSynth_util.h:68-75 */
static inline float ssd_a(f4 a, f4 b, float alpha) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dw = a.w - b.w;
    float s = dx * dx;
    s = fmaf(dy, dy, s);
    s = fmaf(dz, dz, s);
    s = fmaf(alpha * dw, dw, s);
    return s;
}
/* sumSquaredDiff without alpha weight, texSynth_util.h:59-66 */
static inline float ssd(f4 a, f4 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dw = a.w - b.w;
    float s = dx * dx;
    s = fmaf(dy, dy, s);
    s = fmaf(dz, dz, s);
    s = fmaf(dw, dw, s);
    return s;
}
static inline f4 sub4(f4 a, f4 b) { f4 r = {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; return r; }

/* Test hooks: the helpers above on plain arrays, for checking them one by
 * one against the reference's own texSynth_util.h compiled for the host. */
void pto_basis(float angle, float su, float sv, float* out) {
    f2 b0, b1;
    basis(angle, su, sv, &b0, &b1);
    out[0] = b0.x; out[1] = b0.y; out[2] = b1.x; out[3] = b1.y;
}
void pto_new_coord(float i, float j, float ex, float ey, const float* b, float* out) {
    f2 b0 = {b[0], b[1]}, b1 = {b[2], b[3]};
    new_coord(i, j, ex, ey, b0, b1, &out[0], &out[1]);
}
void pto_clamp_to_exemplar(float* x, float* y, int w, int h) { clamp_to_exemplar(x, y, w, h); }
float pto_ssd(const float* a, const float* b, float alpha) {
    f4 x = {a[0], a[1], a[2], a[3]}, y = {b[0], b[1], b[2], b[3]};
    return ssd_a(x, y, alpha);
}
float pto_ssd_plain(const float* a, const float* b) {
    f4 x = {a[0], a[1], a[2], a[3]}, y = {b[0], b[1], b[2], b[3]};
    return ssd(x, y);
}

/* per-pixel values that calculateResidual recomputes for every candidate
 * but that do not depend on the candidate (texSynth_kernel.cu:545-561) */
typedef struct {
    int validF, validB;      /* advected centre hysteresis > 0 */
    pt_patchxf prevF, prevB;
    f2 fb0, fb1, bb0, bb1;
    float hyst;              /* hysteresisTerm if validF else 0 */
    int temporalF, temporalB;
} pixctx;

/* hysteresisTerm, texSynth_kernel.cu:506-535 */
static float hysteresis_term(const pto* o, int x, int y, int level) {
    float maxD = o->p.maxDistortion / ldexpf(1.0f, level);
    const f2* v = (o->p.direction == PT_FORWARD) ? o->vel_b[o->cur] : o->vel_f[o->cur];
    f2 d00 = vel_texel(v, o, x, y), d10 = vel_texel(v, o, x + 1, y);
    f2 d01 = vel_texel(v, o, x, y + 1), d11 = vel_texel(v, o, x + 1, y + 1);
    float maxX = fmaxf(d00.x, fmaxf(d01.x, fmaxf(d10.x, d11.x)));
    float maxY = fmaxf(d00.y, fmaxf(d01.y, fmaxf(d10.y, d11.y)));
    float minX = fminf(d00.x, fminf(d01.x, fminf(d10.x, d11.x)));
    float minY = fminf(d00.y, fminf(d01.y, fminf(d10.y, d11.y)));
    if ((maxX - minX) < maxD && (maxY - minY) < maxD) return o->p.hysteresisWeight;
    return 0.0f;
}

static void make_pixctx(const pto* o, int x, int y, int level, pixctx* pc) {
    size_t i = (size_t)y * o->W + x;
    pc->prevF = o->adv_off[0][i];
    pc->prevB = o->adv_off[1][i];
    pc->validF = pc->prevF.hysteresis > 0;
    pc->validB = pc->prevB.hysteresis > 0;
    int td = (o->p.timeDerivativeInputWeight > 0.f || o->p.timeDerivativeOutputWeight > 0.f ||
              o->p.temporalCoherenceWeight > 0.f);
    pc->temporalF = (o->p.direction == PT_FORWARD || o->p.direction == PT_BIDIRECTIONAL) && pc->validF && td;
    pc->temporalB = (o->p.direction == PT_BACKWARD || o->p.direction == PT_BIDIRECTIONAL) && pc->validB && td;
    if (pc->temporalF) {
        float a = screen_to_exemplar_angle(o, x, y, pc->prevF.x, pc->prevF.y, pc->prevF.layer);
        basis(a, o->p.residualWindowScaleU * pc->prevF.scaleU, o->p.residualWindowScaleV * pc->prevF.scaleV,
              &pc->fb0, &pc->fb1);
    }
    if (pc->temporalB) {
        float a = screen_to_exemplar_angle(o, x, y, pc->prevB.x, pc->prevB.y, pc->prevB.layer);
        basis(a, o->p.residualWindowScaleU * pc->prevB.scaleU, o->p.residualWindowScaleV * pc->prevB.scaleV,
              &pc->bb0, &pc->bb1);
    }
    pc->hyst = pc->validF ? hysteresis_term(o, x, y, level) : 0.0f;
}

/* timeDerivativeTerms, texSynth_kernel.cu:438-469 */
static float time_derivative(const pto* o, int dir, const pt_patchxf* prev, f2 pb0, f2 pb1,
                             f4 base, f4 tb, f4 canvas, f4 to, int x, int y, int i, int j) {
    size_t k = (size_t)(y + j) * o->W + (x + i);
    f4 pbase = o->adv_base[dir][k], pout = o->adv_out[dir][k];
    float px, py;
    new_coord((float)i, (float)j, prev->x, prev->y, pb0, pb1, &px, &py);
    f4 peb, peo;
    ex_sample2(o, px, py, prev->layer, &peb, &peo);
    if (o->p.colorspace == 1) { /* :454-459 */
        pbase = rgb_to_lab(pbase); pout = rgb_to_lab(pout);
        peb = rgb_to_lab(peb); peo = rgb_to_lab(peo);
    }
    float r = ssd(sub4(base, pbase), sub4(tb, peb)) * o->p.timeDerivativeInputWeight;
    r = fmaf(ssd(sub4(canvas, pout), sub4(to, peo)), o->p.timeDerivativeOutputWeight, r);
    r = fmaf(ssd(pout, to), o->p.temporalCoherenceWeight, r);
    return r;
}

/* coherenceTerm, texSynth_kernel.cu:377-423 */
static float coherence_term(const pto* o, int x, int y, int i, int j, float tcx, float tcy,
                            float tx, float ty, int level) {
    const pt_patchxf* co = &o->off_base[(size_t)(y + j) * o->W + (x + i)];
    float dx = co->x - tcx, dy = co->y - tcy;
    float distEx = fmaf(dy, dy, dx * dx) * (float)(1 << level);
    float distIm = (float)(i * i + j * j) * (float)(1 << level);
    float R = o->p.coherenceRatioRange;
    float ratio = fmaxf(1.0f / R, fminf(distEx / distIm, R));
    float lr = pt_logf(ratio);
    float lR = pt_logf(R);
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
    float angle = fmaxf(-1.0f, fminf(pt_acosf(d), 1.0f));
    double ar = (double)o->p.coherenceAngleRange * M_PI;
    float Ea = (float)(fmin((double)angle, ar) / ar);
    return 1.0f - (1.0f - Er) * (1.0f - Ea);
}

/* calculateResidual, texSynth_kernel.cu:537-659 (FP32 contract) */
static float energy_f32(const pto* o, int x, int y, int level, const pt_patchxf* t, const pixctx* pc) {
    const pt_params* P = &o->p;
    const int r = P->residualWindowSize;
    float sumW = 0.0f, sum = 0.0f;
    if (pc->validF) sum = sum - pc->hyst;
    f2 b0, b1;
    basis(t->theta, P->residualWindowScaleU * t->scaleU, P->residualWindowScaleV * t->scaleV, &b0, &b1);
    const int hw = (o->SW) >> level;
    const int hh = (o->SH * o->NS) >> level;
    for (int i = -r; i <= r; i++) {
        for (int j = -r; j <= r; j++) {
            if (!in_rect(o, x + i, y + j, level, 0)) continue;
            size_t k = (size_t)(y + j) * o->W + (x + i);
            f4 base = lin_texel4(o, o->img_base[o->cur][k]);
            f4 canvas = o->canvas[k];
            if (P->colorspace == 1) { base = rgb_to_lab(base); canvas = rgb_to_lab(canvas); } /* :575-578 */
            float tx, ty;
            new_coord((float)i, (float)j, t->x, t->y, b0, b1, &tx, &ty);
            if (tx >= (float)hw) tx -= (float)hw; else if (tx < 0) tx += (float)hw;
            if (ty >= (float)hh) ty -= (float)hh; else if (ty < 0) ty += (float)hh;
            f4 tb, to;
            ex_sample2(o, tx, ty, t->layer, &tb, &to);
            if (P->colorspace == 1) { tb = rgb_to_lab(tb); to = rgb_to_lab(to); } /* :603-606 */
            float res = ssd_a(base, tb, P->alphaWeight) * P->inputAnalogyWeight;
            if (pc->temporalF && o->adv_off[0][k].hysteresis > 0)
                res = res + time_derivative(o, 0, &pc->prevF, pc->fb0, pc->fb1, base, tb, canvas, to, x, y, i, j);
            if (pc->temporalB && o->adv_off[1][k].hysteresis > 0)
                res = res + time_derivative(o, 1, &pc->prevB, pc->bb0, pc->bb1, base, tb, canvas, to, x, y, i, j);
            if (i == 0 && j == 0) {
                if (P->distTransWeight > 0.f) {
                    float de = ex_sample_dt(o, tx, ty, t->layer) / t->scaleV;
                    float di = dt_texel(o, o->cur, x, y);
                    float diff = fmaxf(0.0f, fminf(fabsf(de - di), 10.0f)); /* clamp = fmaxf(a, fminf(f, b)), cutil_math.h:1027: NaN gives 10 */
                    res = res + diff * P->distTransWeight;
                }
                { /* histogramTerm, :486-495 */
                    int L = clampi(t->layer, 0, PT_MAX_STYLES - 1);
                    float sh = (float)(hh / P->numStyles);
                    int hx = f2i(tx), hy = f2i(ty + sh * (float)t->layer);
                    hx = clampi(hx, 0, o->SW - 1);
                    hy = clampi(hy, 0, o->SH * o->NS - 1);
                    float h = o->hist_base[(size_t)hy * o->SW + hx];
                    float thr = P->offsetsHistogramThreshold[L];
                    res = res + ((h > thr) ? (h - thr) * P->offsetsHistogramSlope[L] : 0.0f);
                }
                if (P->styleObjIdWeight > 0.f) {
                    int imgID = id_texel(o, x, y);
                    int styleID = ex_point_id(o, tx, ty, t->layer);
                    res = res + ((imgID != styleID) ? P->styleObjIdWeight : 0.0f);
                }
            } else {
                res = fmaf(ssd_a(canvas, to, P->alphaWeight), P->canvasOutputWeight, res);
                if (P->coherenceWeight > 0.f) {
                    float c = coherence_term(o, x, y, i, j, t->x, t->y, tx, ty, level);
                    res = fmaf(c, P->coherenceWeight, res);
                }
            }
            float w = o->gauss[i + r] * o->gauss[j + r];
            sum = fmaf(res, w, sum);
            sumW = sumW + w;
        }
    }
    if (sumW < EPSILON_F) return BIG_RESIDUAL;
    return sum / sumW;
}

/* test_offset + isExemplarPixelCulled, texSynth_kernel.cu:200-205,695-721 */
static float test_offset(const pto* o, int x, int y, const pt_patchxf* t, int level, float image_alpha,
                         const pixctx* pc) {
    float dte = ex_texel_dt(o, f2i(t->x), f2i(t->y), t->layer);
    if (!((double)dte > (double)o->p.distTransCull * 1.25)) {
        if (!o->p.transparencyOk) {
            float ea = ex_sample_out(o, t->x, t->y, t->layer).w;
            if (ea < ALPHA_THRESHOLD && image_alpha > ALPHA_THRESHOLD) return BIG_RESIDUAL;
        }
        return energy_f32(o, x, y, level, t, pc);
    }
    return BIG_RESIDUAL;
}

static inline pt_patchxf patch(float x, float y, float th, float h, int layer, float su, float sv) {
    pt_patchxf p;
    p.x = x; p.y = y; p.theta = th; p.hysteresis = h; p.layer = layer;
    p.scaleU = su; p.scaleV = sv; p.lumShiftY = 0.f; p.lumShiftA = 0.f;
    return p;
}

/* calculatePropagateOffset, texSynth_kernel.cu:956-982 */
static pt_patchxf propagate_offset(const pto* o, const pt_patchxf* src, int tx, int ty, int x, int y) {
    pt_patchxf t = src[pixel_wrap_index(o->W, o->H, tx, ty)]; /* level-0 size */
    f2 sc = scale_texel(o, tx, ty);
    f2 b0, b1;
    basis(t.theta, o->p.residualWindowScaleU * sc.x, o->p.residualWindowScaleV * sc.y, &b0, &b1);
    float ex, ey;
    new_coord((float)x - (float)tx, (float)y - (float)ty, t.x, t.y, b0, b1, &ex, &ey);
    clamp_to_exemplar(&ex, &ey, o->ew, o->eh);
    float ang = screen_to_exemplar_angle(o, x, y, ex, ey, t.layer);
    f2 s2 = scale_texel(o, x, y);
    return patch(ex, ey, ang, 0.0f, t.layer, s2.x, s2.y);
}

/* ------------------------------------------------------------------------ */
/* kernels                                                                  */
/* ------------------------------------------------------------------------ */

#define FOR_RECT(o, level)                                     \
    _Pragma("omp parallel for schedule(dynamic, 4) num_threads(o->threads)") \
    for (int y = 0; y < lvl_h(o, level); y++)                  \
        for (int x = 0; x < lvl_w(o, level); x++)

/* propagate_kernel, texSynth_kernel.cu:1112-1219 (advected candidates at
 * :1184-1216 are rebuilt with hysteresis 0 at :981 and never tested) */
static float keymask_alpha(const pto* o, int x, int y, int key);
/* with key >= 0, pixels under the key's mask take the key itself (:1137-1142) */
void pto_propagate_k(pto* o, int level, int jump, int key) {
    const pt_patchxf* base = o->off_base;
    pt_patchxf* work = o->off_work;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        if (image_culled(o, x, y)) { work[k] = patch(0, 0, 0, 0, 0, 1.f, 1.f); continue; }
        if (keymask_alpha(o, x, y, key) > 0) { work[k] = patch((float)x, (float)y, 0.f, 1.f, key, 1.f, 1.f); continue; }
        float best = o->res_base[k];
        float ia = lin_texel(o, o->img_base[o->cur][k].w);
        pt_patchxf ow = base[k];
        pixctx pc;
        make_pixctx(o, x, y, level, &pc);
        for (int c = 0; c < 4; c++) {
            int tx = x, ty = y;
            if (c == 0) tx = x + jump;
            else if (c == 1) tx = x - jump;
            else if (c == 2) ty = y + jump;
            else ty = y - jump;
            pt_patchxf t = propagate_offset(o, base, tx, ty, x, y);
            float r = test_offset(o, x, y, &t, level, ia, &pc);
            if (r < best) { ow = t; best = r; }
        }
        work[k] = ow;
    }
}
void pto_propagate(pto* o, int level, int jump) { pto_propagate_k(o, level, jump, -1); }

/* scatter_kernel + averageOffset, texSynth_kernel.cu:841-952; the reference's
 * randFloat() returns unsigned int 0 (texSynth_util.h:155-163), so every
 * candidate is (best.x + 0.9*dist, best.y). */
void pto_scatter_k(pto* o, int level, uint32_t pass_id, int key);
void pto_scatter(pto* o, int level) { pto_scatter_k(o, level, 0, -1); }
void pto_scatter_pass(pto* o, int level, uint32_t pass_id) { pto_scatter_k(o, level, pass_id, -1); }
/* with key >= 0, pixels under the key's mask keep their offset (:887-892) */
void pto_scatter_k(pto* o, int level, uint32_t pass_id, int key) {
    const pt_patchxf* base = o->off_base;
    pt_patchxf* work = o->off_work;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        if (image_culled(o, x, y)) continue;
        pt_patchxf off = base[k];
        if (keymask_alpha(o, x, y, key) > 0) { work[k] = off; continue; }
        float cached = o->res_base[k];
        float best = (float)((double)cached + 10e-7);
        pt_patchxf ow = off;
        float ia = lin_texel(o, o->img_base[o->cur][k].w);
        float dist = (float)(o->ew > o->eh ? o->ew : o->eh);
        const float closest = 10.f, factor = 0.9f;
        f2 sc = scale_texel(o, x, y);
        pixctx pc;
        make_pixctx(o, x, y, level, &pc);
        for (int i = 0; i < o->p.scatterSamplesCount && dist * factor >= closest; i++) {
            float dmin = dist * factor;
            float ex, ey;
            if (o->p.rngMode == PT_RNG_COUNTER) {
                /* opt-in mode: radius in [dmin, dist), angle in [0, 2pi) */
                float rr = counter_u01(o->p.rngSeed, pass_id, (uint32_t)x, (uint32_t)y, 2u * (uint32_t)i);
                float th = counter_u01(o->p.rngSeed, pass_id, (uint32_t)x, (uint32_t)y, 2u * (uint32_t)i + 1u) *
                           6.28318530717958647692f;
                float s, cth;
                pt_sincosf(th, &s, &cth);
                float len = fmaf(rr, dist - dmin, dmin);
                ex = fmaf(cth, len, ow.x);
                ey = fmaf(s, len, ow.y);
            } else {
                ex = ow.x + dmin;
                ey = ow.y + 0.0f;
            }
            clamp_to_exemplar(&ex, &ey, o->ew, o->eh);
            float ang = screen_to_exemplar_angle(o, x, y, ex, ey, 0);
            pt_patchxf t = patch(ex, ey, ang, 0.0f, 0, sc.x, sc.y);
            float r = test_offset(o, x, y, &t, level, ia, &pc);
            if (r < best) { ow = t; best = r; }
            dist *= factor;
        }
        /* averageOffset(offsets, x, y, level, 0) */
        pt_patchxf avg = patch(0, 0, 0, 1.f, 0, 1.f, 1.f);
        int n = 0;
        for (int i = -1; i <= 1; i++)
            for (int j = -1; j <= 1; j++) {
                if (!in_rect(o, x + i, y + j, level, 0) || (i == 0 && j == 0)) continue;
                const pt_patchxf* nb = &base[(size_t)(y + j) * o->W + (x + i)];
                if (nb->layer != 0) continue;
                avg.x = avg.x + nb->x;
                avg.y = avg.y + nb->y;
                n++;
            }
        avg.x = gpu_nan(avg.x / (float)n);  /* 0/0 without a same-layer neighbour */
        avg.y = gpu_nan(avg.y / (float)n);
        avg.theta = screen_to_exemplar_angle(o, x, y, avg.x, avg.y, 0);
        float r = test_offset(o, x, y, &avg, level, ia, &pc);
        if (r < best) { ow = avg; best = r; }
        if (best < cached) work[k] = ow;
    }
}

/* updateResidualCache_kernel, texSynth_kernel.cu:661-693 */
void pto_update_residual(pto* o, int level) {
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        if (image_culled(o, x, y)) { o->res_base[k] = 0.0f; continue; }
        pixctx pc;
        make_pixctx(o, x, y, level, &pc);
        o->res_base[k] = energy_f32(o, x, y, level, &o->off_base[k], &pc);
    }
}

/* offsetsToOutput, texSynth_kernel.cu:263-274 */
static void offsets_to_output(pto* o, int level) {
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        const pt_patchxf* p = &o->off_base[k];
        f4 c = ex_sample_out(o, p->x, p->y, p->layer);
        c.x = c.x + p->lumShiftY; c.y = c.y + p->lumShiftY; c.z = c.z + p->lumShiftY;
        c.w = c.w + p->lumShiftA;
        o->canvas[k] = c;
    }
}

/* separable Gaussian, convolution.cu:76-210 (normalised weights, zero
 * apron); the smoothed histogram is input to histogramTerm. */
/* allocateGaussianKernel, convolution.cu:37-60: sigma = r/3 in float, the
 * exponential in float, and with `normalize` the division by
 * sqrt(2*pi)*sigma in double (M_PI promotes the expression), rounded back
 * to float.  kern has 2r+1 entries. */
static void gauss_weights(int r, int normalize, float* kern) {
    float sigma = (float)r / 3.0f, s2 = sigma * sigma;
    for (int i = 0; i <= r; i++) {
        float wgt = expf(-(float)(i * i) / (2.f * s2));
        if (normalize) wgt = (float)((double)wgt / (sqrt(2.0 * M_PI) * (double)sigma));
        kern[r + i] = wgt; kern[r - i] = wgt;
    }
}
void pto_gauss_weights(int r, int normalize, float* kern) { gauss_weights(r, normalize, kern); }

static void conv_pass(pto* o, const float* src, float* dst, int w, int h, int rows, const float* kern, int r) {
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            float s = 0.0f;
            for (int j = -r; j <= r; j++) {
                int xx = rows ? x + j : x, yy = rows ? y : y + j;
                float v = (xx >= 0 && xx < w && yy >= 0 && yy < h) ? src[(size_t)yy * o->SW + xx] : 0.0f;
                s = fmaf(kern[r - j], v, s);
            }
            dst[(size_t)y * o->SW + x] = s;
        }
}

/* convolutionRowsGPU + convolutionColumnsGPU on one w x h image (pitch w) */
void pto_convolve_separable(const float* src, float* dst, int w, int h, int r) {
    float kern[64];
    gauss_weights(r, 1, kern);
    float* tmp = (float*)malloc(sizeof(float) * (size_t)w * h);
    for (int pass = 0; pass < 2; pass++) {
        const float* s = pass ? tmp : src;
        float* d = pass ? dst : tmp;
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                float acc = 0.0f;
                for (int j = -r; j <= r; j++) {
                    int xx = pass ? x : x + j, yy = pass ? y + j : y;
                    float v = (xx >= 0 && xx < w && yy >= 0 && yy < h) ? s[(size_t)yy * w + xx] : 0.0f;
                    acc = fmaf(kern[r - j], v, acc);
                }
                d[(size_t)y * w + x] = acc;
            }
    }
    free(tmp);
}

/* syncBuffers, texSynth_kernel.cu:1240-1303 (distance-transform, velocity
 * and ribbon caches are display-only and not kept) */
void pto_sync(pto* o, int level, int flags) {
    if (!(flags & PT_DONT_COPY_OFFSETS))
        memcpy(o->off_base, o->off_work, sizeof(pt_patchxf) * (size_t)o->W * o->H);
    int hist = 0;
    for (int i = 0; i < o->p.numStyles && i < PT_MAX_STYLES; i++)
        hist = hist || (o->p.offsetsHistogramSlope[i] > 0.0f);
    if (hist) {
        size_t n = (size_t)o->SW * o->SH * o->NS;
        memset(o->hist_base, 0, n * sizeof(float));
        memset(o->hist_work, 0, n * sizeof(float));
        /* calculateOffsetsHistogram adds nothing (:258 is commented out) */
        int r = o->p.residualWindowSize;
        float kern[64];
        gauss_weights(r, 1, kern);
        int w = o->SW >> level, h = (o->SH * o->NS) >> level;
        /* convolutionRowsGPU(dst = working, src = base), then
         * convolutionColumnsGPU(dst = base, src = working) */
        conv_pass(o, o->hist_base, o->hist_work, w, h, 1, kern, r);
        conv_pass(o, o->hist_work, o->hist_base, w, h, 0, kern, r);
    }
    offsets_to_output(o, level);
    if (!(flags & PT_DONT_UPDATE_RESIDUAL)) pto_update_residual(o, level);
}

/* toPatchXF, texSynth_util.h:212-214: a packed random texel (x, y, theta,
 * layer) as a PatchXF with zero hysteresis and unit scale */
static inline pt_patchxf to_patchxf(f4 r) { return patch(r.x, r.y, r.z, 0.f, f2i(r.w), 1.f, 1.f); }
void pto_to_patchxf(const float* c, pt_patchxf* out) {
    f4 r = {c[0], c[1], c[2], c[3]};
    *out = to_patchxf(r);
}

/* copyRandomKernel + randomizeOffsets, texSynth_kernel.cu:2044-2059,2100-2109 */
void pto_randomize(pto* o, int level) {
    FOR_RECT(o, level) {
        f4 r = rnd_texel(o, x, y);
        o->off_work[(size_t)y * o->W + x] = to_patchxf(r);
    }
    pto_sync(o, level, 0);
}

/* offsetUpsampleNearest, texSynth_kernel.cu:1403-1417 */
static f2 upsample_nearest(const pto* o, const pt_patchxf* c, float dx, float dy) {
    f2 b0, b1;
    basis(c->theta, 1.0f, 1.0f, &b0, &b1);
    float ix, iy;
    new_coord(dx, dy, c->x, c->y, b0, b1, &ix, &iy);
    clamp_to_exemplar(&ix, &iy, o->ew, o->eh);
    f2 r = {fmaf(ix, 2.0f, 0.5f), fmaf(iy, 2.0f, 0.5f)};
    return r;
}

/* upsampleBilinearKernel + TexSynth::upsample, texSynth_kernel.cu:1453-1532.
 * Border pixels keep the working buffer's content; the residual working
 * buffer's border is modelled as equal to the base residual. */
void pto_upsample(pto* o, int level) {
    const pt_patchxf* base = o->off_base;
    pt_patchxf* work = o->off_work;
    for (size_t k = 0; k < (size_t)o->W * o->H; k++) o->res_work[k] = o->res_base[k];
    _Pragma("omp parallel for schedule(dynamic, 4) num_threads(o->threads)")
    for (int y = 1; y < lvl_h(o, level) - 1; y++)
        for (int x = 1; x < lvl_w(o, level) - 1; x++) {
            float cx = (float)((double)x - 0.5) / 2.0f;
            float cy = (float)((double)y - 0.5) / 2.0f;
            int lcx = (int)floorf(cx), lcy = (int)floorf(cy);
            const pt_patchxf* o00 = &base[(size_t)lcy * o->W + lcx];
            const pt_patchxf* o10 = &base[(size_t)lcy * o->W + lcx + 1];
            const pt_patchxf* o01 = &base[(size_t)(lcy + 1) * o->W + lcx];
            const pt_patchxf* o11 = &base[(size_t)(lcy + 1) * o->W + lcx + 1];
            float a = cx - (float)lcx, b = cy - (float)lcy;
            float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
            /* the reference's sum as nvcc contracts it: the first product fused
             * with the second, rounded; then fused multiply-adds (measured on
             * the reference's upsample kernel) */
            float ix = fmaf(w00, o00->x, w10 * o10->x); ix = fmaf(w01, o01->x, ix); ix = fmaf(w11, o11->x, ix);
            float iy = fmaf(w00, o00->y, w10 * o10->y); iy = fmaf(w01, o01->y, iy); iy = fmaf(w11, o11->y, iy);
            f2 up = {fmaf(ix, 2.0f, 0.5f), fmaf(iy, 2.0f, 0.5f)};
            const pt_patchxf* cs[4] = {o00, o10, o01, o11};
            int far = 0;
            for (int q = 0; q < 4; q++) {
                float dx = ix - cs[q]->x, dy = iy - cs[q]->y;
                if (fmaf(dx, dx, dy * dy) > 16.0f) far = 1; /* length2: x*x + y*y, first product fused */
            }
            if (far) {
                int rcx = (int)roundf(cx), rcy = (int)roundf(cy);
                const pt_patchxf* c = &base[(size_t)rcy * o->W + rcx];
                up = upsample_nearest(o, c, cx - (float)rcx, cy - (float)rcy);
            }
            int layer = o00->layer;
            float rw = o->res_base[(size_t)lcy * o->W + lcx];
            float ang = screen_to_exemplar_angle(o, x, y, up.x, up.y, layer);
            f2 sc = scale_texel(o, x, y);
            work[(size_t)y * o->W + x] = patch(up.x, up.y, ang, 0.0f, layer, sc.x, sc.y);
            o->res_work[(size_t)y * o->W + x] = rw;
        }
    memcpy(o->off_base, o->off_work, sizeof(pt_patchxf) * (size_t)o->W * o->H);
    memcpy(o->res_base, o->res_work, sizeof(float) * (size_t)o->W * o->H);
}

static f4 f2k_texel(const pto* o, int forwards, int x, int y);
static pt_ribbon ribbon_of(f4 c);

/* calculateTranslatedPosition + advectKernel + TexSynth::advectOffsets,
 * texSynth_kernel.cu:1540-1726 */
void pto_advect(pto* o, int level, int time_step, int forwards, int flags) {
    int d = forwards ? 0 : 1;
    int prev = (o->cur + 1) % 2;
    pt_patchxf* dst = o->adv_off[d];
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        if (image_culled(o, x, y)) {
            f4 z = {0, 0, 0, 0};
            o->adv_base[d][k] = z; o->adv_out[d][k] = z;
            dst[k] = patch(0, 0, 0, 0, 0, 1.f, 1.f);
            continue;
        }
        f4 rnd = rnd_texel(o, x, y);
        f4 fr = {rnd.x - floorf(rnd.x), rnd.y - floorf(rnd.y), rnd.z - floorf(rnd.z), rnd.w - floorf(rnd.w)};
        pt_patchxf out = patch(0, 0, 0, 0, 0, 1.f, 1.f);
        int valid = 0;
        float tx = 0, ty = 0;
        if (!(flags & PT_ADVECT_DO_NOT_CHECK_PREVIOUS)) {
            f2 fw, bk;
            if (forwards) {
                bk = vel_texel(o->vel_b[o->cur], o, x, y);
                tx = (float)x + bk.x; ty = (float)y + bk.y;
                fw = vel_bilinear(o->vel_f[prev], o, tx, ty);
            } else {
                fw = vel_texel(o->vel_f[o->cur], o, x, y);
                tx = (float)x + fw.x; ty = (float)y + fw.y;
                bk = vel_bilinear(o->vel_b[prev], o, tx, ty);
            }
            fw.x = -fw.x; fw.y = -fw.y;
            float ddx = fw.x - bk.x, ddy = fw.y - bk.y;
            float dist = sqrtf(fmaf(ddy, ddy, ddx * ddx));
            float cxf = fminf(fmaxf(ceilf(tx), -2.f), 1e9f), cyf = fminf(fmaxf(ceilf(ty), -2.f), 1e9f);
            float fxf = fminf(fmaxf(floorf(tx), -2.f), 1e9f), fyf = fminf(fmaxf(floorf(ty), -2.f), 1e9f);
            valid = in_rect(o, f2i(cxf), f2i(cyf), level, 0) && in_rect(o, f2i(fxf), f2i(fyf), level, 0) &&
                    (dist < (float)(1.414 * 2));
            if (valid) {
                /* isImagePixelCulledPreviousFrame(tx, ty, level, 8.0), :188-198 */
                float pd = dt_texel(o, prev, f2i(tx), f2i(ty));
                if (pd > ((float)o->p.distTransCull - 8.0f)) valid = 0;
            }
        }
        if (valid) {
            int rtx = (int)roundf(tx), rty = (int)roundf(ty);
            const pt_patchxf* nx = &o->off_base[(size_t)rty * o->W + rtx];
            f2 b0, b1;
            basis(nx->theta, 1.0f, 1.0f, &b0, &b1);
            float ix, iy;
            new_coord(tx - (float)rtx, ty - (float)rty, nx->x, nx->y, b0, b1, &ix, &iy);
            clamp_to_exemplar(&ix, &iy, o->ew, o->eh);
            f4 color = lin_texel4(o, o->img_base[o->cur][k]);
            f4 pcol = img_bilinear(o, prev, tx, ty);
            out.x = ix; out.y = iy; out.theta = nx->theta;
            if (o->p.lumShiftEnable) {
                float dr = color.x - pcol.x, dg = color.y - pcol.y, db = color.z - pcol.z;
                float ly = (float)(0.2126 * dr + 0.7152 * dg + 0.0722 * db);
                out.lumShiftY = nx->lumShiftY + ly;
            } else {
                out.lumShiftY = 0.f;
            }
            out.lumShiftA = 0.f;
            out.layer = nx->layer;
            out.hysteresis = 1;
            o->adv_base[d][k] = pcol;
            o->adv_out[d][k] = ex_sample_out(o, out.x, out.y, out.layer);
            o->adv_ts[d][k] = time_step;
        }
        /* keyframe interpolation, :1652-1675 */
        if ((flags & PT_ADVECT_CHECK_FRAME_TO_KEY) && (time_step > 1 || out.hysteresis == 0)) {
            pt_ribbon rb = ribbon_of(f2k_texel(o, !forwards, x, y));
            if (rb.layer >= 0 && (abs(rb.time_step) < time_step || out.hysteresis == 0)) {
                out.x = rb.x + (float)x;
                out.y = rb.y + (float)y;
                out.layer = rb.layer;
                out.hysteresis = 1.0f;
                out.lumShiftY = 0.f; out.lumShiftA = 0.f;
            }
            f4 eb, eo;
            ex_sample2(o, out.x, out.y, out.layer, &eb, &eo);
            o->adv_base[d][k] = eb; o->adv_out[d][k] = eo;
            o->adv_ts[d][k] = abs(rb.time_step);
        }
        if (out.hysteresis == 0) {
            out = patch(rnd.x, rnd.y, rnd.z, 0.0f, f2i(rnd.w), 1.f, 1.f);
            f4 z = {0, 0, 0, 0};
            o->adv_base[d][k] = z; o->adv_out[d][k] = z;
            o->adv_ts[d][k] = -1;
        }
        float J = o->p.advectionJitter;
        out.x = fmaf(fr.x, J, out.x * (1 - J));
        out.y = fmaf(fr.y, J, out.y * (1 - J));
        out.theta = screen_to_exemplar_angle(o, x, y, out.x, out.y, out.layer);
        dst[k] = out;
    }
    memcpy(o->off_base, dst, sizeof(pt_patchxf) * (size_t)o->W * o->H);
    pto_sync(o, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL);
    if (flags & PT_ADVECT_UPDATE_RESIDUAL) pto_update_residual(o, level);
    memcpy(o->adv_res[d], o->res_base, sizeof(float) * (size_t)o->W * o->H);
}

/* mergeRandomlyKernel + TexSynth::mergeRandomly, texSynth_kernel.cu:1891-1936,
 * 2003-2024.  Frame-to-key ribbons are never uploaded outside keyframe mode,
 * so both ribbon fetches read zero and both count as valid. */
void pto_merge_randomly(pto* o, int level, int forwards, float weight, int force) {
    int d = forwards ? 0 : 1;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        pt_patchxf a = o->adv_off[d][k], u = o->off_base[k];
        f4 rnd = rnd_texel(o, x, y);
        float r = forwards ? rnd.x - floorf(rnd.x) : rnd.y - floorf(rnd.y);
        int av = a.hysteresis > 0;
        o->off_work[k] = ((av || force) && r < weight) ? a : u;
    }
    pto_sync(o, level, 0);
}

/* mergeUsingResidualKernel, texSynth_kernel.cu:1856-1889,1978-2001 */
void pto_merge_using_residual(pto* o, int level, int forwards) {
    int d = forwards ? 0 : 1;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        pt_patchxf r;
        if (o->adv_res[d][k] < o->res_base[k]) { r = o->adv_off[d][k]; r.hysteresis = 1.f; }
        else { r = o->off_base[k]; r.hysteresis = 0.f; }
        o->off_work[k] = r;
    }
    pto_sync(o, level, 0);
}

/* ------------------------------------------------------------------------ */
/* FP64 energy (accuracy reference; exact bilinear, libm sin/cos)           */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z, w; } d4;

/* bilinear footprint and weights in double at (u, v): exact fractions, or
 * with PT_FILTER_TEXTURE the texture unit's 1/256 weights (the FP64 energy
 * then measures only the rounding of the float arithmetic) */
typedef struct { int x0, x1, y0, y1; double w00, w10, w01, w11; int hw; } bld_t;
static bld_t bld_setup(const pto* o, double u, double v, int n, int m) {
    bld_t d;
    if (o->p.filterMode == PT_FILTER_TEXTURE) {
        bl_t b = bl_setup((float)u, (float)v, n, m, 1);
        d.x0 = b.x0; d.x1 = b.x1; d.y0 = b.y0; d.y1 = b.y1;
        d.w00 = b.q00 / 256.0; d.w10 = b.q10 / 256.0; d.w01 = b.q01 / 256.0; d.w11 = b.q11 / 256.0;
        d.hw = 1;
        return d;
    }
    double fx = floor(u), fy = floor(v);
    double a = u - fx, c = v - fy;
    fx = fmin(fmax(fx, -1.0), (double)n);
    fy = fmin(fmax(fy, -1.0), (double)m);
    int ix = (int)fx, iy = (int)fy;
    d.x0 = clampi(ix, 0, n - 1); d.x1 = clampi(ix + 1, 0, n - 1);
    d.y0 = clampi(iy, 0, m - 1); d.y1 = clampi(iy + 1, 0, m - 1);
    d.w00 = (1 - a) * (1 - c); d.w10 = a * (1 - c); d.w01 = (1 - a) * c; d.w11 = a * c;
    d.hw = 0;
    return d;
}
static double bld1(const bld_t* d, float t00, float t10, float t01, float t11) {
    if (d->hw) { t00 = tex_ftz(t00); t10 = tex_ftz(t10); t01 = tex_ftz(t01); t11 = tex_ftz(t11); }
    return t00 * d->w00 + t10 * d->w10 + t01 * d->w01 + t11 * d->w11;
}

static d4 ex_sample_d(const pto* o, const f4* arr, double u, double v, int layer) {
    bld_t b = bld_setup(o, u, v, o->ew, o->eh);
    const f4* A = arr + (size_t)ex_layer(o, layer) * o->ew * o->eh;
    f4 t00 = A[(size_t)b.y0 * o->ew + b.x0], t10 = A[(size_t)b.y0 * o->ew + b.x1];
    f4 t01 = A[(size_t)b.y1 * o->ew + b.x0], t11 = A[(size_t)b.y1 * o->ew + b.x1];
    d4 r;
    r.x = bld1(&b, t00.x, t10.x, t01.x, t11.x);
    r.y = bld1(&b, t00.y, t10.y, t01.y, t11.y);
    r.z = bld1(&b, t00.z, t10.z, t01.z, t11.z);
    r.w = bld1(&b, t00.w, t10.w, t01.w, t11.w);
    return r;
}

/* calculateResidual in double precision for the non-temporal terms
 * (inputAnalogy, canvasOutput, DT, histogram (zero), objectID).  The sample
 * positions are the reference's float positions (basis, offset + i*b0 + j*b1
 * and the one-period wrap are float arithmetic in the reference); bilinear
 * filtering, the SSDs, the Gaussian weights and the sums are in double. */
static double energy_f64(const pto* o, int x, int y, int level, const pt_patchxf* t) {
    const pt_params* P = &o->p;
    const int r = P->residualWindowSize;
    double sumW = 0, sum = 0;
    f2 fb0, fb1;
    basis(t->theta, P->residualWindowScaleU * t->scaleU, P->residualWindowScaleV * t->scaleV, &fb0, &fb1);
    const int hw = (o->SW) >> level, hh = (o->SH * o->NS) >> level;
    double sigma = r / 3.0;
    for (int i = -r; i <= r; i++)
        for (int j = -r; j <= r; j++) {
            if (!in_rect(o, x + i, y + j, level, 0)) continue;
            size_t k = (size_t)(y + j) * o->W + (x + i);
            f4 base = lin_texel4(o, o->img_base[o->cur][k]);
            f4 canvas = o->canvas[k];
            float ftx, fty;
            new_coord((float)i, (float)j, t->x, t->y, fb0, fb1, &ftx, &fty);
            if (ftx >= (float)hw) ftx -= (float)hw; else if (ftx < 0) ftx += (float)hw;
            if (fty >= (float)hh) fty -= (float)hh; else if (fty < 0) fty += (float)hh;
            double tx = ftx, ty = fty;
            d4 tb = ex_sample_d(o, o->ex_base, tx, ty, t->layer);
            d4 to = ex_sample_d(o, o->ex_out, tx, ty, t->layer);
            double dx = base.x - tb.x, dy = base.y - tb.y, dz = base.z - tb.z, dw = base.w - tb.w;
            double res = (dx * dx + dy * dy + dz * dz + (double)P->alphaWeight * dw * dw) * P->inputAnalogyWeight;
            if (i == 0 && j == 0) {
                if (P->distTransWeight > 0.f) {
                    /* bilinear DT in double */
                    bld_t b = bld_setup(o, tx, ty, o->ew, o->eh);
                    const float* D = o->ex_dt + (size_t)ex_layer(o, t->layer) * o->ew * o->eh;
                    double de = bld1(&b, D[(size_t)b.y0 * o->ew + b.x0], D[(size_t)b.y0 * o->ew + b.x1],
                                     D[(size_t)b.y1 * o->ew + b.x0], D[(size_t)b.y1 * o->ew + b.x1]);
                    de /= t->scaleV;
                    double di = dt_texel(o, o->cur, x, y);
                    double diff = fmax(0.0, fmin(fabs(de - di), 10.0));
                    res += diff * P->distTransWeight;
                }
                {
                    int L = clampi(t->layer, 0, PT_MAX_STYLES - 1);
                    if (0.0 > P->offsetsHistogramThreshold[L])
                        res += (0.0 - P->offsetsHistogramThreshold[L]) * P->offsetsHistogramSlope[L];
                }
                if (P->styleObjIdWeight > 0.f) {
                    int imgID = id_texel(o, x, y);
                    int styleID = ex_point_id(o, (float)tx, (float)ty, t->layer);
                    if (imgID != styleID) res += P->styleObjIdWeight;
                }
            } else {
                double ex = canvas.x - to.x, ey = canvas.y - to.y, ez = canvas.z - to.z, ea = canvas.w - to.w;
                res += (ex * ex + ey * ey + ez * ez + (double)P->alphaWeight * ea * ea) * P->canvasOutputWeight;
            }
            double wi = exp(-(double)(i * i) / (2 * sigma * sigma)), wj = exp(-(double)(j * j) / (2 * sigma * sigma));
            double w = wi * wj;
            sum += res * w;
            sumW += w;
        }
    if (sumW < 1e-6) return 1e31;
    return sum / sumW;
}

/* ------------------------------------------------------------------------ */
/* public C interface of the oracle (ctypes)                                */
/* ------------------------------------------------------------------------ */

static void* zalloc(size_t n) { return calloc(1, n ? n : 1); }

pto* pto_create(int W, int H, int SW, int SH, int NS) {
    pto* o = (pto*)zalloc(sizeof(pto));
    o->W = W; o->H = H; o->SW = SW; o->SH = SH; o->NS = NS;
    o->threads = 1;
    size_t n = (size_t)W * H;
    for (int l = 0; l < 2; l++) {
        o->img_base[l] = (f4*)zalloc(n * sizeof(f4));
        o->img_dt[l] = (float*)zalloc(n * sizeof(float));
        o->vel_f[l] = (f2*)zalloc(n * sizeof(f2));
        o->vel_b[l] = (f2*)zalloc(n * sizeof(f2));
        o->adv_off[l] = (pt_patchxf*)zalloc(n * sizeof(pt_patchxf));
        o->adv_base[l] = (f4*)zalloc(n * sizeof(f4));
        o->adv_out[l] = (f4*)zalloc(n * sizeof(f4));
        o->adv_res[l] = (float*)zalloc(n * sizeof(float));
        o->adv_ts[l] = (int32_t*)zalloc(n * sizeof(int32_t));
    }
    o->off_base = (pt_patchxf*)zalloc(n * sizeof(pt_patchxf));
    o->off_work = (pt_patchxf*)zalloc(n * sizeof(pt_patchxf));
    o->res_base = (float*)zalloc(n * sizeof(float));
    o->res_work = (float*)zalloc(n * sizeof(float));
    o->canvas = (f4*)zalloc(n * sizeof(f4));
    o->rib_base = (pt_ribbon*)zalloc(n * sizeof(pt_ribbon));
    o->rib_work = (pt_ribbon*)zalloc(n * sizeof(pt_ribbon));
    for (size_t i = 0; i < n; i++) o->rib_base[i].layer = o->rib_work[i].layer = -1; /* RibbonP() */
    size_t hn = (size_t)SW * SH * NS;
    o->hist_base = (float*)zalloc(hn * sizeof(float));
    o->hist_work = (float*)zalloc(hn * sizeof(float));
    return o;
}

void pto_destroy(pto* o) {
    if (!o) return;
    for (int l = 0; l < 2; l++) {
        free(o->img_base[l]); free(o->img_dt[l]); free(o->vel_f[l]); free(o->vel_b[l]);
        free(o->adv_off[l]); free(o->adv_base[l]); free(o->adv_out[l]); free(o->adv_res[l]); free(o->adv_ts[l]);
    }
    free(o->off_base); free(o->off_work); free(o->res_base); free(o->res_work); free(o->canvas);
    free(o->hist_base); free(o->hist_work);
    free(o->img_orient); free(o->img_scale); free(o->img_ids); free(o->rnd);
    free(o->ex_base); free(o->ex_out); free(o->ex_orient); free(o->ex_dt); free(o->ex_ids);
    free(o->cumul[0]); free(o->cumul[1]); free(o->f2k[0]); free(o->f2k[1]);
    free(o->rib_base); free(o->rib_work);
    free(o);
}

void pto_set_threads(pto* o, int n) { o->threads = n < 1 ? 1 : n; }

/* TexSynth::setup: unnormalised Gaussian of radius r, convolution.cu:37-60 */
void pto_set_params(pto* o, const pt_params* p) {
    o->p = *p;
    int r = p->residualWindowSize;
    if (r >= 0 && r < 32) gauss_weights(r, 0, o->gauss);
}

void pto_init_exemplars(pto* o, int ew, int eh, int ns) {
    free(o->ex_base); free(o->ex_out); free(o->ex_orient); free(o->ex_dt); free(o->ex_ids);
    size_t n = (size_t)ew * eh * ns;
    o->ew = ew; o->eh = eh; o->ens = ns;
    o->ex_base = (f4*)zalloc(n * sizeof(f4));
    o->ex_out = (f4*)zalloc(n * sizeof(f4));
    o->ex_orient = (float*)zalloc(n * sizeof(float));
    o->ex_dt = (float*)zalloc(n * sizeof(float));
    o->ex_ids = (int32_t*)zalloc(n * sizeof(int32_t));
}

void pto_upload_exemplar(pto* o, int style, const float* base, const float* out, const float* orient,
                         const float* dt, const int32_t* ids) {
    size_t n = (size_t)o->ew * o->eh, off = n * style;
    memcpy(o->ex_base + off, base, n * sizeof(f4));
    memcpy(o->ex_out + off, out, n * sizeof(f4));
    memcpy(o->ex_orient + off, orient, n * sizeof(float));
    memcpy(o->ex_dt + off, dt, n * sizeof(float));
    memcpy(o->ex_ids + off, ids, n * sizeof(int32_t));
}

/* layered uploads into the current layer's top-left rectangle (or the
 * previous layer for VEL_*_PREVIOUS), texSynth_kernel.cu:2143-2253 */
void pto_upload_layered(pto* o, int which, const float* data, int w, int h) {
    int prev = (o->cur + 1) % 2;
    for (int y = 0; y < h; y++) {
        size_t dst = (size_t)y * o->W;
        switch (which) {
            case PT_LAYER_INPUT_COLOR: memcpy(o->img_base[o->cur] + dst, data + (size_t)y * w * 4, w * sizeof(f4)); break;
            case PT_LAYER_INPUT_DIST_TRANS: memcpy(o->img_dt[o->cur] + dst, data + (size_t)y * w, w * sizeof(float)); break;
            case PT_LAYER_INPUT_VEL_B: memcpy(o->vel_b[o->cur] + dst, data + (size_t)y * w * 2, w * sizeof(f2)); break;
            case PT_LAYER_INPUT_VEL_F: memcpy(o->vel_f[o->cur] + dst, data + (size_t)y * w * 2, w * sizeof(f2)); break;
            case PT_LAYER_INPUT_VEL_B_PREVIOUS: memcpy(o->vel_b[prev] + dst, data + (size_t)y * w * 2, w * sizeof(f2)); break;
            case PT_LAYER_INPUT_VEL_F_PREVIOUS: memcpy(o->vel_f[prev] + dst, data + (size_t)y * w * 2, w * sizeof(f2)); break;
            default: break;
        }
    }
}

void pto_upload_plain(pto* o, int which, const void* data, int w, int h) {
    size_t n = (size_t)w * h;
    switch (which) {
        case PT_LAYER_INPUT_ORIENTATION:
            free(o->img_orient); o->img_orient = (float*)zalloc(n * 4); memcpy(o->img_orient, data, n * 4);
            o->io_w = w; o->io_h = h; break;
        case PT_LAYER_INPUT_SCALE:
            free(o->img_scale); o->img_scale = (f2*)zalloc(n * 8); memcpy(o->img_scale, data, n * 8);
            o->is_w = w; o->is_h = h; break;
        case PT_LAYER_INPUT_ID:
            free(o->img_ids); o->img_ids = (int32_t*)zalloc(n * 4); memcpy(o->img_ids, data, n * 4);
            o->ii_w = w; o->ii_h = h; break;
        case PT_LAYER_RANDOM:
            free(o->rnd); o->rnd = (f4*)zalloc(n * 16); memcpy(o->rnd, data, n * 16);
            o->rn_w = w; o->rn_h = h; break;
        default: break;
    }
}

void pto_flip(pto* o) { o->cur = (o->cur + 1) % 2; }
/* CudaBufferPair::copyBaseToWorking, cudaImageBuffer.h:335-337 */
void pto_copy_base_to_working(pto* o) {
    memcpy(o->off_work, o->off_base, sizeof(pt_patchxf) * (size_t)o->W * o->H);
}
/* renderAnimationFBMO's merge set-up, synthesisProcessor.cpp:979-980:
 * offsets.base().copyTo(advected.offsets()),
 * residualCache.base().copyTo(advected.residual()) */
void pto_copy_base_to_advected(pto* o, int forwards) {
    int d = forwards ? 0 : 1;
    memcpy(o->adv_off[d], o->off_base, sizeof(pt_patchxf) * (size_t)o->W * o->H);
    memcpy(o->adv_res[d], o->res_base, sizeof(float) * (size_t)o->W * o->H);
}
void pto_reset_advected(pto* o) {
    size_t n = (size_t)o->W * o->H;
    for (int l = 0; l < 2; l++) {
        memset(o->adv_off[l], 0, n * sizeof(pt_patchxf)); memset(o->adv_base[l], 0, n * sizeof(f4));
        memset(o->adv_out[l], 0, n * sizeof(f4)); memset(o->adv_res[l], 0, n * sizeof(float));
        memset(o->adv_ts[l], 0, n * sizeof(int32_t));
    }
}

/* ------------------------------------------------------------------------ */
/* keyframe interpolation                                                   */
/* ------------------------------------------------------------------------ */

/* TexSynth::initialize_cumulativeFields, texSynth_kernel.cu:2138-2142 */
void pto_init_cumulative_fields(pto* o, int w, int h, int n) {
    for (int d = 0; d < 2; d++) {
        free(o->cumul[d]);
        o->cumul[d] = (f4*)zalloc((size_t)w * h * n * sizeof(f4));
    }
    o->cf_w = w; o->cf_h = h; o->cf_n = n;
}
/* uploadImage_Color4 of TS_LAYER_CUMUL_FIELD_B/F (layer = key index) and
 * TS_LAYER_FRAME_TO_KEY_RIBBON_B/F, texSynth_kernel.cu:2196-2206 */
void pto_upload_cumul(pto* o, int forwards, int layer, const float* rgba, int w, int h) {
    f4* dst = o->cumul[forwards ? 1 : 0] + (size_t)layer * o->cf_w * o->cf_h;
    for (int y = 0; y < h; y++) memcpy(dst + (size_t)y * o->cf_w, rgba + (size_t)y * w * 4, (size_t)w * sizeof(f4));
}
void pto_upload_f2k(pto* o, int forwards, const float* rgba, int w, int h) {
    int d = forwards ? 1 : 0;
    free(o->f2k[d]);
    o->f2k[d] = (f4*)zalloc((size_t)w * h * sizeof(f4));
    memcpy(o->f2k[d], rgba, (size_t)w * h * sizeof(f4));
    o->fk_w[d] = w; o->fk_h[d] = h;
}
/* a cumulative-field fetch at exemplar (u, v) of key layer j: linear filter,
 * clamp; a layer that was never uploaded reads zero */
static f4 cumul_sample(const pto* o, int forwards, float u, float v, int j) {
    f4 z = {0, 0, 0, 0};
    const f4* F = o->cumul[forwards ? 1 : 0];
    if (!F || j < 0 || j >= o->cf_n) return z;
    bl_t b = bl_setup(u, v, o->cf_w, o->cf_h, o->p.filterMode == PT_FILTER_TEXTURE);
    const f4* L = F + (size_t)j * o->cf_w * o->cf_h;
    return bl4(&b, L[(size_t)b.y0 * o->cf_w + b.x0], L[(size_t)b.y0 * o->cf_w + b.x1],
               L[(size_t)b.y1 * o->cf_w + b.x0], L[(size_t)b.y1 * o->cf_w + b.x1]);
}
/* a frame-to-key ribbon texel at integer (x, y) (a linear texture read at
 * a texel centre), clamp */
static f4 f2k_texel(const pto* o, int forwards, int x, int y) {
    int d = forwards ? 1 : 0;
    f4 z = {0, 0, 0, 0};
    if (!o->f2k[d]) return z;
    x = clampi(x, 0, o->fk_w[d] - 1); y = clampi(y, 0, o->fk_h[d] - 1);
    return lin_texel4(o, o->f2k[d][(size_t)y * o->fk_w[d] + x]);
}
/* RibbonP(Color4): (x, y, time_step, layer) = (b, g, r, a) */
static pt_ribbon ribbon_of(f4 c) {
    pt_ribbon r;
    r.x = c.z; r.y = c.y; r.time_step = f2i(c.x); r.layer = f2i(c.w);
    return r;
}
void pto_ribbon_of(const float* c, float* xy, int* ts_layer) {
    f4 v = {c[0], c[1], c[2], c[3]};
    pt_ribbon r = ribbon_of(v);
    xy[0] = r.x; xy[1] = r.y; ts_layer[0] = r.time_step; ts_layer[1] = r.layer;
}
/* the keyframe mask of key layer `key` at pixel (x, y): the key's output
 * alpha (PYRAMID_FETCH_LAYER(gExemplarOutput, x, y, keyIndex)) */
static float keymask_alpha(const pto* o, int x, int y, int key) {
    if (key < 0) return -1.0f;
    return ex_sample_out(o, (float)x, (float)y, key).w;
}

/* propagate_kernel_keys, texSynth_kernel.cu:984-1110 */
void pto_propagate_keys(pto* o, int level, int jump, int key) {
    const pt_patchxf* base = o->off_base;
    pt_patchxf* work = o->off_work;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        if (image_culled(o, x, y)) { work[k] = patch(0, 0, 0, 0, 0, 1.f, 1.f); continue; }
        if (keymask_alpha(o, x, y, key) > 0) { work[k] = patch((float)x, (float)y, 0.f, 1.f, key, 1.f, 1.f); continue; }
        float best = o->res_base[k];
        float ia = lin_texel(o, o->img_base[o->cur][k].w);
        pt_patchxf ow = base[k];
        pixctx pc;
        make_pixctx(o, x, y, level, &pc);
        for (int c = 0; c < 4; c++) {
            int tx = x, ty = y;
            if (c == 0) tx = x + jump;
            else if (c == 1) tx = x - jump;
            else if (c == 2) ty = y + jump;
            else ty = y - jump;
            pt_patchxf t = propagate_offset(o, base, tx, ty, x, y);
            float r = test_offset(o, x, y, &t, level, ia, &pc);
            if (r < best) { ow = t; best = r; }
            const float ex0 = t.x, ey0 = t.y;
            const int elayer = t.layer;
            float ex = ex0, ey = ey0;
            for (int j = elayer - 1; j >= o->p.firstKeyIndex; j--) {
                f4 m = cumul_sample(o, 0, ex, ey, j + 1);
                if (m.x < -EPSILON_F) break;
                ex = ex + m.z; ey = ey + m.y;
                pt_patchxf q = patch(ex, ey, screen_to_exemplar_angle(o, x, y, ex, ey, j), 0.f, j, 1.f, 1.f);
                r = test_offset(o, x, y, &q, level, ia, &pc);
                if (r < best) { ow = q; best = r; }
            }
            ex = ex0; ey = ey0;
            for (int j = elayer + 1; j <= o->p.lastKeyIndex; j++) {
                f4 m = cumul_sample(o, 1, ex, ey, j - 1);
                if (m.x < -EPSILON_F) break;
                ex = ex + m.z; ey = ey + m.y;
                pt_patchxf q = patch(ex, ey, screen_to_exemplar_angle(o, x, y, ex, ey, j), 0.f, j, 1.f, 1.f);
                r = test_offset(o, x, y, &q, level, ia, &pc);
                if (r < best) { ow = q; best = r; }
            }
        }
        work[k] = ow;
    }
}

/* scatter_kernel_keys, texSynth_kernel.cu:723-839 (randFloat() is 0: the
 * candidate is (best.x + 0.9*dist, best.y)) */
void pto_scatter_keys(pto* o, int level, int key) {
    const pt_patchxf* base = o->off_base;
    pt_patchxf* work = o->off_work;
    const int span = o->p.lastKeyIndex - o->p.firstKeyIndex + 1;
    const int samples = span != 0 ? o->p.scatterSamplesCount / span : 0;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        if (image_culled(o, x, y)) continue;
        pt_patchxf off = base[k];
        if (keymask_alpha(o, x, y, key) > 0) { work[k] = off; continue; }
        float cached = o->res_base[k];
        float best = (float)((double)cached + 10e-7);
        pt_patchxf ow = off;
        float ia = lin_texel(o, o->img_base[o->cur][k].w);
        float dist = (float)(o->ew > o->eh ? o->ew : o->eh);
        const float closest = 10.f, factor = 0.9f;
        pixctx pc;
        make_pixctx(o, x, y, level, &pc);
        for (int i = 0; i < samples && dist * factor >= closest; i++) {
            float dmin = dist * factor;
            float ex = ow.x + dmin, ey = ow.y + 0.0f;
            clamp_to_exemplar(&ex, &ey, o->ew, o->eh);
            const int elayer = ow.layer;
            pt_patchxf t = patch(ex, ey, screen_to_exemplar_angle(o, x, y, ex, ey, elayer), 0.f, elayer, 1.f, 1.f);
            float r = test_offset(o, x, y, &t, level, ia, &pc);
            if (r < best) { ow = t; best = r; }
            const float ex0 = ex, ey0 = ey;
            for (int j = elayer - 1; j >= o->p.firstKeyIndex; j--) {
                pt_ribbon m = ribbon_of(cumul_sample(o, 0, ex, ey, j + 1));
                if (m.layer < 0) break;
                ex = ex + m.x; ey = ey + m.y;
                pt_patchxf q = patch(ex, ey, screen_to_exemplar_angle(o, x, y, ex, ey, j), 0.f, j, 1.f, 1.f);
                r = test_offset(o, x, y, &q, level, ia, &pc);
                if (r < best) { ow = q; best = r; }
            }
            ex = ex0; ey = ey0;
            for (int j = elayer + 1; j <= o->p.lastKeyIndex; j++) {
                pt_ribbon m = ribbon_of(cumul_sample(o, 1, ex, ey, j - 1));
                if (m.layer < 0) break;
                ex = ex + m.x; ey = ey + m.y;
                pt_patchxf q = patch(ex, ey, screen_to_exemplar_angle(o, x, y, ex, ey, j), 0.f, j, 1.f, 1.f);
                r = test_offset(o, x, y, &q, level, ia, &pc);
                if (r < best) { ow = q; best = r; }
            }
            dist *= factor;
        }
        if (best < cached) work[k] = ow;
    }
}

/* calculateTranslatedPosition, texSynth_kernel.cu:1540-1574, for a buffer
 * of the level's size */
static int translated_position(const pto* o, int forwards, int x, int y, int level, float* ptx, float* pty) {
    int prev = (o->cur + 1) % 2;
    f2 fw, bk;
    float tx, ty;
    if (forwards) {
        bk = vel_texel(o->vel_b[o->cur], o, x, y);
        tx = (float)x + bk.x; ty = (float)y + bk.y;
        fw = vel_bilinear(o->vel_f[prev], o, tx, ty);
    } else {
        fw = vel_texel(o->vel_f[o->cur], o, x, y);
        tx = (float)x + fw.x; ty = (float)y + fw.y;
        bk = vel_bilinear(o->vel_b[prev], o, tx, ty);
    }
    fw.x = -fw.x; fw.y = -fw.y;
    float ddx = fw.x - bk.x, ddy = fw.y - bk.y;
    float dist = sqrtf(fmaf(ddy, ddy, ddx * ddx));
    float cxf = fminf(fmaxf(ceilf(tx), -2.f), 1e9f), cyf = fminf(fmaxf(ceilf(ty), -2.f), 1e9f);
    float fxf = fminf(fmaxf(floorf(tx), -2.f), 1e9f), fyf = fminf(fmaxf(floorf(ty), -2.f), 1e9f);
    *ptx = tx; *pty = ty;
    return in_rect(o, f2i(cxf), f2i(cyf), level, 0) && in_rect(o, f2i(fxf), f2i(fyf), level, 0) &&
           (dist < (float)(1.414 * 2));
}

/* accumulateAdvectionKernel + cumulativeAdvectionFieldToOutput +
 * TexSynth::accumulateRibbonField, texSynth_kernel.cu:290-304,1728-1853
 * (cacheVelocities is display-only).  The chained comparison of :1776 is
 * kept as written: ((l00 == l10) == l01) == l11 compares booleans with
 * layers. */
void pto_accumulate_ribbon(pto* o, int level, int forwards, int time_step, int overwrite) {
    const pt_ribbon* src = o->rib_base;
    pt_ribbon* dest = o->rib_work;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        pt_ribbon out = {0.f, 0.f, 0, -1};
        float tx, ty;
        int masked = img_texel(o, o->cur, x, y).w == 0.0f;
        if (masked || !translated_position(o, forwards, x, y, level, &tx, &ty)) {
            if (overwrite) dest[k] = out;
            continue;
        }
        int ftx = (int)floorf(tx), fty = (int)floorf(ty), ctx = (int)ceilf(tx), cty = (int)ceilf(ty);
        pt_ribbon s00 = src[(size_t)fty * o->W + ftx], s10 = src[(size_t)fty * o->W + ctx];
        pt_ribbon s01 = src[(size_t)cty * o->W + ftx], s11 = src[(size_t)cty * o->W + ctx];
        int v00 = s00.layer >= 0, v10 = s10.layer >= 0, v01 = s01.layer >= 0, v11 = s11.layer >= 0;
        if (!(v00 || v10 || v01 || v11)) {
            if (overwrite) dest[k] = out;
            continue;
        }
        int all_valid = v00 && v10 && v01 && v11;
        int same = (((s00.layer == s10.layer) == s01.layer) == s11.layer);
        const float th = 5.f;
        int diverges = fabsf(s00.x - s10.x) > th || fabsf(s00.x - s01.x) > th || fabsf(s00.x - s11.x) > th ||
                       fabsf(s00.y - s10.y) > th || fabsf(s00.y - s01.y) > th || fabsf(s00.y - s11.y) > th;
        if (!all_valid || !same || diverges) {
            int rtx = (int)roundf(tx), rty = (int)roundf(ty);
            if (ftx == rtx && fty == rty) out = s00;
            else if (ftx + 1 == rtx && fty == rty) out = s10;
            else if (ftx == rtx && fty + 1 == rty) out = s01;
            else out = s11;
        } else {
            float wx = tx - (float)ftx, wy = ty - (float)fty;
            float rx0 = s00.x * (1.f - wx) + s10.x * wx;
            float ry0 = s00.y * (1.f - wx) + s10.y * wx;
            float rx1 = s01.x * (1.f - wx) + s11.x * wx;
            float ry1 = s01.y * (1.f - wx) + s11.y * wx;
            out.x = rx0 * (1.f - wy) + rx1 * wy;
            out.y = ry0 * (1.f - wy) + ry1 * wy;
            out.time_step = s00.time_step;
            out.layer = s00.layer;
        }
        out.x = out.x + (tx - (float)x);
        out.y = out.y + (ty - (float)y);
        out.time_step = out.time_step + time_step;
        pt_ribbon cur = dest[k];
        if (overwrite || cur.layer < 0 || fabsf((float)cur.time_step) >= fabsf((float)out.time_step)) dest[k] = out;
    }
    memcpy(o->rib_base, o->rib_work, sizeof(pt_ribbon) * (size_t)o->W * o->H); /* copyWorkingToBase */
    /* cumulativeAdvectionFieldToOutput into advectedF.output from the
     * canvas (keyFrame.pixel(x + field.x, y + field.y), truncated to int;
     * a position outside the image reads zero) */
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        pt_ribbon f = o->rib_base[k];
        f4 c = {0, 0, 0, 0};
        if (f.layer >= 0) {
            int px = f2i((float)x + f.x), py = f2i((float)y + f.y);
            if (px >= 0 && py >= 0 && px < o->W && py < o->H) c = o->canvas[(size_t)py * o->W + px];
        }
        o->adv_out[0][k] = c;
    }
}

/* mergeAdvectedKernel + TexSynth::mergeAdvectedBuffers,
 * texSynth_kernel.cu:1938-1976,2025-2042: r is the fractional part that
 * randomFloat4 returns through its argument, and the random fallback is
 * made of those fractional parts */
void pto_merge_advected(pto* o, int level, int fallback) {
    pt_patchxf* work = o->off_work;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        pt_patchxf f = o->adv_off[0][k], b = o->adv_off[1][k], res;
        f4 rnd = rnd_texel(o, x, y);
        f4 fr = {rnd.x - floorf(rnd.x), rnd.y - floorf(rnd.y), rnd.z - floorf(rnd.z), rnd.w - floorf(rnd.w)};
        if (f.hysteresis > 0 && b.hysteresis > 0) res = (fr.x < 0.5f) ? f : b;
        else if (f.hysteresis > 0) res = f;
        else if (b.hysteresis > 0) res = b;
        else if (fallback == PT_MERGE_FALLBACK_RANDOM) res = patch(fr.x, fr.y, fr.z, 0.f, f2i(fr.w), 1.f, 1.f);
        else res = o->off_base[k];
        work[k] = res;
    }
    pto_sync(o, level, 0);
}

/* copyFrameToKeyRibbonKernel + TexSynth::offsetsFromFrameToKeyRibbon,
 * texSynth_kernel.cu:2061-2097,2111-2118 */
void pto_frame_to_key_ribbon(pto* o, int level, int look_forwards) {
    pt_patchxf* work = o->off_work;
    FOR_RECT(o, level) {
        size_t k = (size_t)y * o->W + x;
        pt_ribbon rb = ribbon_of(f2k_texel(o, look_forwards, x, y));
        pt_patchxf out;
        if (rb.layer >= 0) {
            float ox = rb.x + (float)x, oy = rb.y + (float)y;
            out = patch(ox, oy, screen_to_exemplar_angle(o, x, y, ox, oy, rb.layer), 1.0f, rb.layer, 1.f, 1.f);
        } else {
            out = to_patchxf(rnd_texel(o, x, y)); /* copyRandomKernel */
        }
        work[k] = out;
    }
    pto_sync(o, level, 0);
}

/* ribbonField.base() copyFromHost / copyToHost of the level rectangle;
 * canvasOutputCache.copyFromHost; advectedF/B.output().copyToHost */
void pto_load_ribbon(pto* o, int level, const pt_ribbon* src) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(o->rib_base + (size_t)y * o->W, src + (size_t)y * w, w * sizeof(pt_ribbon));
}
void pto_get_ribbon(const pto* o, int level, pt_ribbon* out) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(out + (size_t)y * w, o->rib_base + (size_t)y * o->W, w * sizeof(pt_ribbon));
}
void pto_load_canvas(pto* o, int level, const float* rgba) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(o->canvas + (size_t)y * o->W, rgba + (size_t)y * w * 4, w * sizeof(f4));
}
void pto_get_advected_output(const pto* o, int forwards, int level, float* out) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    const f4* src = o->adv_out[forwards ? 0 : 1];
    for (int y = 0; y < h; y++) memcpy(out + (size_t)y * w * 4, src + (size_t)y * o->W, w * sizeof(f4));
}

/* WorkingBuffers::loadOffsets / loadResidual, workingBuffers.cpp:166-207 */
void pto_load_offsets(pto* o, int level, const pt_patchxf* src) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(o->off_base + (size_t)y * o->W, src + (size_t)y * w, w * sizeof(pt_patchxf));
}
void pto_load_residual(pto* o, int level, const float* src) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) o->res_base[(size_t)y * o->W + x] = pt_half_roundtrip(src[(size_t)y * w + x]);
}
void pto_get_offsets(const pto* o, int level, pt_patchxf* dst) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(dst + (size_t)y * w, o->off_base + (size_t)y * o->W, w * sizeof(pt_patchxf));
}
void pto_get_residual(const pto* o, int level, float* dst) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(dst + (size_t)y * w, o->res_base + (size_t)y * o->W, w * sizeof(float));
}
void pto_get_output(const pto* o, int level, float* dst) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    for (int y = 0; y < h; y++) memcpy(dst + (size_t)y * w * 4, o->canvas + (size_t)y * o->W, w * sizeof(f4));
}

/* Energy of given offsets at every level pixel, using the current canvas:
 * FP32 contract (out32) and FP64 (out64); culled pixels give 0. */
void pto_energy_map(const pto* o, int level, const pt_patchxf* offs, float* out32, double* out64) {
    int w = lvl_w(o, level), h = lvl_h(o, level);
    _Pragma("omp parallel for schedule(dynamic, 4) num_threads(o->threads)")
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const pt_patchxf* t = &offs[(size_t)y * w + x];
            if (image_culled(o, x, y)) {
                if (out32) out32[(size_t)y * w + x] = 0.f;
                if (out64) out64[(size_t)y * w + x] = 0.0;
                continue;
            }
            if (out32) {
                pixctx pc;
                make_pixctx(o, x, y, level, &pc);
                out32[(size_t)y * w + x] = energy_f32(o, x, y, level, t, &pc);
            }
            if (out64) out64[(size_t)y * w + x] = energy_f64(o, x, y, level, t);
        }
}

/* polynomial functions exported for tests against libm */
float pto_sinf(float t) { float s, c; pt_sincosf(t, &s, &c); return s; }
float pto_cosf(float t) { float s, c; pt_sincosf(t, &s, &c); return c; }
float pto_atan2f(float y, float x) { return pt_atan2f(y, x); }
float pto_logf(float x) { return pt_logf(x); }
float pto_acosf(float x) { return pt_acosf(x); }
float pto_half_roundtrip(float x) { return pt_half_roundtrip(x); }

/* ------------------------------------------------------------------------ */
/* glibc rand() restatement and the random-offset pyramid                   */
/* ------------------------------------------------------------------------ */

/* glibc's TYPE_3 additive feedback generator behind srand()/rand():
 * r[0] = seed (0 -> 1); r[i] = 16807 r[i-1] mod (2^31-1) for i < 31 (Schrage);
 * r[i] = r[i-31] for 31 <= i < 34; r[i] = r[i-31] + r[i-3] (mod 2^32) after;
 * outputs r[i] >> 1 for i >= 344. */
typedef struct { uint32_t r[34]; int pos; } pto_glibc;

static void glibc_srand(pto_glibc* g, uint32_t seed) {
    int32_t word = (int32_t)seed;
    if (seed == 0) word = 1;
    uint32_t r[344];
    r[0] = (uint32_t)word;
    for (int i = 1; i < 31; i++) {
        int32_t hi = word / 127773, lo = word % 127773;
        word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        r[i] = (uint32_t)word;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 34; i < 344; i++) r[i] = r[i - 31] + r[i - 3];
    for (int i = 0; i < 34; i++) g->r[i] = r[310 + i];
    g->pos = 0;
}
static uint32_t glibc_rand(pto_glibc* g) {
    /* ring of the last 34 values; new = value 31 back + value 3 back */
    uint32_t v = g->r[(g->pos + 3) % 34] + g->r[(g->pos + 31) % 34];
    g->r[g->pos] = v;
    g->pos = (g->pos + 1) % 34;
    return v >> 1;
}

void pto_glibc_stream(uint32_t seed, int n, int32_t* out) {
    pto_glibc g;
    glibc_srand(&g, seed);
    for (int i = 0; i < n; i++) out[i] = (int32_t)glibc_rand(&g);
}

/* SynthesisFrame::createRandomPyramid for one level, synthesisFrame.cpp:66-150
 * (single style, no keyframes).  img_rgba/img_orient: level-size input;
 * ex_out_rgba/ex_orient: level-size exemplar; style_w0/h0: level-0 style
 * size.  Returns the number of pixels that needed a retry. */
int pto_random_level(uint32_t seed, int w, int h, int level, int style_w0, int style_h0,
                     const float* img_rgba, const float* img_orient, const float* ex_out_rgba,
                     const float* ex_orient, int ew, int transparency_ok, int orientation_enabled,
                     float* out) {
    pto_glibc g;
    glibc_srand(&g, seed);
    int retried = 0;
    int mx = (style_w0 >> level) - 1, my = (style_h0 >> level) - 1;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int ox, oy, trial = 0;
            float ia = img_rgba[((size_t)y * w + x) * 4 + 3];
            do {
                ox = (int)(glibc_rand(&g) % (uint32_t)mx);
                oy = (int)(glibc_rand(&g) % (uint32_t)my);
                trial++;
            } while (!transparency_ok && ia > ALPHA_THRESHOLD &&
                     ex_out_rgba[((size_t)oy * ew + ox) * 4 + 3] < ALPHA_THRESHOLD && trial < 50);
            if (trial > 1) retried++;
            float orient = orientation_enabled ? img_orient[(size_t)y * w + x] - ex_orient[(size_t)oy * ew + ox] : 0.f;
            float rx = (float)glibc_rand(&g) / (float)2147483647;
            float ry = (float)glibc_rand(&g) / (float)2147483647;
            float* p = out + ((size_t)y * w + x) * 4;
            p[0] = (float)ox + rx; p[1] = (float)oy + ry; p[2] = orient; p[3] = 0.0f;
        }
    return retried;
}

/* createRandomPyramid with setupWithKeys, synthesisFrame.cpp:94-139: the
 * key layer is drawn first (rand() % nk + first_key), then the offset in
 * that layer (retry rule on its output alpha), then the two fractions.
 * ex_out_rgba / ex_orient hold ns layers of ew x eh. */
int pto_random_level_keys(uint32_t seed, int w, int h, int level, int style_w0, int style_h0,
                          const float* img_rgba, const float* img_orient, const float* ex_out_rgba,
                          const float* ex_orient, int ew, int eh, int ns, int nk, int first_key,
                          int transparency_ok, int orientation_enabled, float* out) {
    pto_glibc g;
    glibc_srand(&g, seed);
    int retried = 0;
    int mx = (style_w0 >> level) - 1, my = (style_h0 >> level) - 1;
    size_t lsz = (size_t)ew * eh;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int style = (int)(glibc_rand(&g) % (uint32_t)nk) + first_key;
            int sl = clampi(style, 0, ns - 1);
            int ox, oy, trial = 0;
            float ia = img_rgba[((size_t)y * w + x) * 4 + 3];
            do {
                ox = (int)(glibc_rand(&g) % (uint32_t)mx);
                oy = (int)(glibc_rand(&g) % (uint32_t)my);
                trial++;
            } while (!transparency_ok && ia > ALPHA_THRESHOLD &&
                     ex_out_rgba[(sl * lsz + (size_t)oy * ew + ox) * 4 + 3] < ALPHA_THRESHOLD && trial < 50);
            if (trial > 1) retried++;
            float orient = orientation_enabled
                               ? img_orient[(size_t)y * w + x] - ex_orient[sl * lsz + (size_t)oy * ew + ox]
                               : 0.f;
            float rx = (float)glibc_rand(&g) / (float)2147483647;
            float ry = (float)glibc_rand(&g) / (float)2147483647;
            float* p = out + ((size_t)y * w + x) * 4;
            p[0] = (float)ox + rx; p[1] = (float)oy + ry; p[2] = orient; p[3] = (float)style;
        }
    return retried;
}

/* PT_RNG_COUNTER random level: four hashed draws per pixel and trial, with
 * the reference's retry rule for opaque pixels on transparent texels */
void pto_counter_random_level(uint32_t seed, int w, int h, int level, int style_w0, int style_h0,
                              const float* img_rgba, const float* img_orient, const float* ex_out_rgba,
                              const float* ex_orient, int ew, int transparency_ok, int orientation_enabled,
                              float* out) {
    int mx = (style_w0 >> level) - 1, my = (style_h0 >> level) - 1;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            float ia = img_rgba[((size_t)y * w + x) * 4 + 3];
            uint32_t base = hash32(seed ^ hash32((uint32_t)x * 0x85EBCA6BU ^ hash32((uint32_t)y * 0xC2B2AE35U)));
            uint32_t d0, d1;
            int trial = 0, again, ox, oy;
            do {
                d0 = hash32(base + 4u * (uint32_t)trial);
                d1 = hash32(base + 4u * (uint32_t)trial + 1u);
                trial++;
                ox = (int)((d0 >> 1) % (uint32_t)mx);
                oy = (int)((d1 >> 1) % (uint32_t)my);
                again = !transparency_ok && ia > ALPHA_THRESHOLD &&
                        ex_out_rgba[((size_t)oy * ew + ox) * 4 + 3] < ALPHA_THRESHOLD && trial < 50;
            } while (again);
            uint32_t d2 = hash32(base + 0x40000000u), d3 = hash32(base + 0x40000001u);
            float orient = orientation_enabled ? img_orient[(size_t)y * w + x] - ex_orient[(size_t)oy * ew + ox] : 0.f;
            float rx = (float)(d2 >> 1) / (float)2147483647;
            float ry = (float)(d3 >> 1) / (float)2147483647;
            float* p = out + ((size_t)y * w + x) * 4;
            p[0] = (float)ox + rx; p[1] = (float)oy + ry; p[2] = orient; p[3] = 0.0f;
        }
}

/* ------------------------------------------------------------------------ */
/* pyramid construction, downsample.cpp:41-209, imageIO.h:136-139           */
/* ------------------------------------------------------------------------ */

/* downsampleAverage: ((((0 + p00) + p01) + p10) + p11) * 0.25 (* 0.5) */
void pto_downsample_avg(const float* src, int w, int h, int ch, float vel_scale, float* dst) {
    int lw = w >> 1, lh = h >> 1;
    for (int y = 0; y < lh; y++)
        for (int x = 0; x < lw; x++)
            for (int c = 0; c < ch; c++) {
                float s = 0.0f;
                s = s + src[((size_t)(2 * y) * w + 2 * x) * ch + c];
                s = s + src[((size_t)(2 * y) * w + 2 * x + 1) * ch + c];
                s = s + src[((size_t)(2 * y + 1) * w + 2 * x) * ch + c];
                s = s + src[((size_t)(2 * y + 1) * w + 2 * x + 1) * ch + c];
                s = s * 0.25f;
                if (vel_scale) s = s * 0.5f;
                dst[((size_t)y * lw + x) * ch + c] = s;
            }
}

/* downsampleVote: most frequent of the 2x2 values; ties go to the smallest
 * value (the reference's tie order is QHash iteration order, unspecified) */
void pto_downsample_vote(const int32_t* src, int w, int h, int32_t* dst) {
    int lw = w >> 1, lh = h >> 1;
    for (int y = 0; y < lh; y++)
        for (int x = 0; x < lw; x++) {
            int32_t v[4] = {src[(size_t)(2 * y) * w + 2 * x], src[(size_t)(2 * y) * w + 2 * x + 1],
                            src[(size_t)(2 * y + 1) * w + 2 * x], src[(size_t)(2 * y + 1) * w + 2 * x + 1]};
            int32_t best = v[0];
            int bestc = -1;
            for (int i = 0; i < 4; i++) {
                int c = 0;
                for (int j = 0; j < 4; j++) c += (v[j] == v[i]);
                if (c > bestc || (c == bestc && v[i] < best)) { bestc = c; best = v[i]; }
            }
            dst[(size_t)y * lw + x] = best;
        }
}

/* strucTensorToAngle, imageIO.h:136-139, on (xx, xy, yy) triples */
void pto_tensor_to_angle(const float* t3, int n, float* out) {
    for (int i = 0; i < n; i++) {
        float xx = t3[3 * i], xy = t3[3 * i + 1], yy = t3[3 * i + 2];
        float a2 = pt_atan2f((float)(2.0 * (double)xy), xx - yy);
        float angle = (float)(0.5 * (double)a2 + M_PI_2);
        out[i] = ((double)angle >= M_PI_2) ? (float)((double)angle - M_PI) : angle;
    }
}
