// pt_energy.cuh -- the tiled patch-distance kernels (propagate, scatter,
// residual) for a compile-time patch radius R and temporal mode TM.
//
// Same per-pixel semantics and the same FP32 arithmetic, operation by
// operation, as the generic kernels in pt_kernels.cu (which restate
// calculateResidual and its callers, src/PaintTweenCUDA/texSynth_kernel.cu:
// 537-952), organised for sm_103a:
//  * a block owns a 32 x 8 pixel tile; the pixel-side inputs of every tap
//    (input colour, canvas, and for temporal passes the advected colours and
//    validity) are staged once into shared memory with an R-pixel halo;
//  * the (2R+1)^2 tap loop is fully unrolled and straight-line: taps outside
//    the level rectangle are evaluated and then discarded by selects, which
//    leaves the sums exactly as skipping them would;
//  * an exemplar texel is 32 bytes (base RGBA, output RGBA), one sector per
//    texel of the bilinear footprint; when a candidate's whole footprint lies inside the
//    exemplar (decided for the whole warp), the wrap and clamp steps -- which
//    are then no-ops -- are left out.
#pragma once

#include <climits>

#include "pt_common.cuh"
#include "pt_internal.h"

namespace ptk {

constexpr int kTileThreads = kTileW * kTileH;

enum { TM_NONE = 0, TM_FWD = 1, TM_BWD = 2 };

// The staged planes start on 128-byte boundaries (tensor copies write
// there); a tile row is TW texels, as a tensor copy's box row is.
template <int R, int TM>
struct TileSmem {
    static constexpr int TW = kTileW + 2 * R;
    static constexpr int TH = kTileH + 2 * R;
    static constexpr int N = TW * TH;
    alignas(128) float4 base[N];
    alignas(128) float4 canvas[N];
    alignas(128) float4 pbase[TM ? N : 1];
    alignas(128) float4 pout[TM ? N : 1];
    alignas(128) float4 prec[TM ? N : 1];  // the advected records' B plane (.x: hysteresis, the validity)
    unsigned long long bar;                // completion barrier of the tensor copies
};

// both colours of one exemplar texel: a 32-byte record of the interleaved
// copy, one 256-bit read-only load (records start on 32-byte boundaries)
__device__ __forceinline__ void ld_texel(const float4* p, float4* b, float4* o) {
    float r0, r1, r2, r3, r4, r5, r6, r7;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r0), "=f"(r1), "=f"(r2), "=f"(r3), "=f"(r4), "=f"(r5), "=f"(r6), "=f"(r7)
        : "l"(p));
    *b = make_float4(r0, r1, r2, r3);
    *o = make_float4(r4, r5, r6, r7);
}

// bilinear base+output at (u, v) of one exemplar layer (LBO: its interleaved
// records); fast (warp-uniform): the footprint is known to be inside
// [0, w-1] x [0, h-1], so the clamps are no-ops and are skipped
// With HW (PT_FILTER_TEXTURE, textures bound) both colours come from the
// texture unit: layered fetches of layer `li` (the clamped style layer) at the
// texture coordinate u + 0.5, which is the reference's own sampling
// (PYRAMID_FETCH_LAYER, texSynth_kernel.cu:600-601).  The level sits in the
// corner of a larger array with its edge texels repeated once beyond, so
// outside the fast case the coordinate is clamped to [0, w-1] x [0, h-1]
// first (NaN to 0): that fetches the texels, with the weights, that clamp
// addressing on a w x h array would.
template <bool PK, int HW>
__device__ __forceinline__ void sample2(const ExView& E, int li, const float4* LBO, float u, float v, float4* base,
                                        float4* out, bool fast) {
    const int w = E.w, h = E.h;
    if (HW) {
        if (!fast) {
            u = fminf(fmaxf(u, 0.0f), (float)(w - 1));
            v = fminf(fmaxf(v, 0.0f), (float)(h - 1));
        }
        const float xs = u + 0.5f, ys = v + 0.5f;
        *base = tex2DLayered<float4>(E.tbase, xs, ys, li);
        *out = tex2DLayered<float4>(E.tout, xs, ys, li);
        return;
    }
    float xs = u + 0.5f, ys = v + 0.5f;
    float xb = xs - 0.5f, yb = ys - 0.5f;
    float fx = floorf(xb), fy = floorf(yb);
    float a = xb - fx, c = yb - fy;
    int x0, x1, y0, y1;
    if (fast) {
        x0 = (int)fx; y0 = (int)fy; x1 = x0 + 1; y1 = y0 + 1;
    } else {
        fx = fminf(fmaxf(fx, -1.0f), (float)w);
        fy = fminf(fmaxf(fy, -1.0f), (float)h);
        int ix = (int)fx, iy = (int)fy;
        x0 = clampi(ix, 0, w - 1); x1 = clampi(ix + 1, 0, w - 1);
        y0 = clampi(iy, 0, h - 1); y1 = clampi(iy + 1, 0, h - 1);
    }
    float oa = 1.0f - a, oc = 1.0f - c;
    Bl bw;
    bw.w00 = oa * oc; bw.w10 = a * oc; bw.w01 = oa * c; bw.w11 = a * c;
    const size_t r0 = (size_t)y0 * w, r1 = (size_t)y1 * w;
    float4 b00, b10, b01, b11, o00, o10, o01, o11;
    ld_texel(LBO + 2 * (r0 + x0), &b00, &o00);
    ld_texel(LBO + 2 * (r0 + x1), &b10, &o10);
    ld_texel(LBO + 2 * (r1 + x0), &b01, &o01);
    ld_texel(LBO + 2 * (r1 + x1), &b11, &o11);
    *base = PK ? bl4p(bw, b00, b10, b01, b11) : bl4(bw, b00, b10, b01, b11);
    *out = PK ? bl4p(bw, o00, o10, o01, o11) : bl4(bw, o00, o10, o01, o11);
}

// the exemplar view with its filter mode fixed at compile time (the tiled
// kernels are instantiated per mode, so the other mode's code is dropped)
template <int HW>
__device__ __forceinline__ ExView ex_mode(const ExView& e) {
    ExView v = e;
    v.hw = HW;
    return v;
}

struct Cand {
    float x, y, theta, su, sv;
    int layer;
};

// per-pixel state of the tiled kernels
struct PixT {
    int x, y;          // level coordinates
    int sidx;          // shared-memory index of the pixel
    int imin, imax, jmin, jmax;  // taps inside the level rectangle
    bool hyst_on;      // advected-F centre valid (hysteresis term subtracted)
    float hyst;
    bool temporal;     // temporal terms of direction TM apply at this pixel
    Patch prev;        // advected offset at the pixel (direction TM)
    float2 pb0, pb1;   // its basis
    bool prev_fast;    // its footprint is inside the exemplar
    float sumW;        // sum of the valid taps' weights, in tap order (the same for every candidate)
};

// does the footprint of a patch at (x, y) with basis (b0, b1) stay inside
// [1, w-3] x [1, h-3] (so every tap's 2x2 texels are in range and no wrap
// applies, since the wrap period is at least the exemplar size)
template <int R>
__device__ __forceinline__ bool footprint_inside(float x, float y, float2 b0, float2 b1, int w, int h) {
    float bx = (float)R * (fabsf(b0.x) + fabsf(b1.x)) + 1.0f;
    float by = (float)R * (fabsf(b0.y) + fabsf(b1.y)) + 1.0f;
    return (x - bx >= 0.0f) && (x + bx <= (float)(w - 2)) && (y - by >= 0.0f) && (y + by <= (float)(h - 2));
}

// Early exit.  When every per-tap term is >= 0 (Params::earlyExit), the
// running sum of a candidate never decreases (each fmaf adds a non-negative
// product and rounding is monotone), and the final energy is that sum divided
// by the pixel's constant tap-weight sum.  Once the running sum reaches
// thr2 = best * sumW rounded up, the energy is >= best whatever the remaining
// taps add, so the reference's strict "<" test rejects the candidate: its
// remaining taps are skipped and it returns +inf, which every caller rejects
// the same way.  A candidate that is still below thr2 at the end returns
// exactly sum / sumW.  A NaN thr2 (no early exit, or best = kNoBest) never
// stops a sum, so the energy is computed in full, NaN and inf included.
constexpr float kNoBest = __builtin_nanf("");
__device__ __forceinline__ float exit_threshold(const Params& P, const PixT& px, float best) {
    return (P.earlyExit && px.sumW >= kEpsilon) ? __fmul_ru(best, px.sumW) : kNoBest;
}

// taps a loop processed before it stopped: the valid taps of its first
// `cols` columns
template <int R>
__device__ __forceinline__ unsigned taps_done(const PixT& px, int cols) {
    const int last = min(-R + cols - 1, px.imax);
    return last < px.imin ? 0u : (unsigned)((last - px.imin + 1) * (px.jmax - px.jmin + 1));
}

__device__ __forceinline__ void count_taps(const Params& P, unsigned taps, bool temporal) {
    unsigned mask = __activemask();
    unsigned tsum = __reduce_add_sync(mask, taps);
    unsigned ttsum = __reduce_add_sync(mask, temporal ? taps : 0u);
    if (lane_id() == (unsigned)(__ffs(mask) - 1)) {
        atomicAdd(&P.counters[1], (unsigned long long)tsum);
        atomicAdd(&P.counters[2], (unsigned long long)ttsum);
    }
}

// One body for both cases: the single-candidate kernels (scatter in
// particular) are instruction-cache bound, and a second, compile-time fast
// copy of this loop measured slower there.  EE: the early-exit test is
// compiled in (false for the residual, which always needs the full sum).
template <int R, int TM, int HW, bool EE>
__device__ __forceinline__ float energy_taps(const Params& P, const TileSmem<R, TM>& T, const PixT& px,
                                             const Cand& c, float2 b0, float2 b1, float sum0, bool fast,
                                             bool fastp, float thr2) {
    constexpr int TW = TileSmem<R, TM>::TW;
    const size_t lsz = (size_t)P.ex.w * P.ex.h;
    const int li = ex_layer(P.ex, c.layer);
    const size_t lo = (size_t)li * lsz;
    const float4* LBO = P.ex.bo + 2 * lo;
    const int lpi = TM ? ex_layer(P.ex, px.prev.layer) : 0;
    const size_t lp = (size_t)lpi * lsz;
    const float hw = (float)P.histW, hh = (float)P.histH;
    const unsigned mask = __activemask();
    float sum = sum0;
    bool act = EE ? !(sum >= thr2) : true;
    int cols = 0;
#pragma unroll 1
    for (int i = -R; i <= R; i++) {
        if (EE && !__any_sync(mask, act)) break;
        cols += act ? 1 : 0;
        if (act) {
#pragma unroll
            for (int j = -R; j <= R; j++) {
                const bool valid = (i >= px.imin) && (i <= px.imax) && (j >= px.jmin) && (j <= px.jmax);
                const int s = px.sidx + j * TW + i;
                float4 base = T.base[s];
                float4 canvas = T.canvas[s];
                float tx = c.x + fmaf((float)i, b0.x, (float)j * b1.x);
                float ty = c.y + fmaf((float)i, b0.y, (float)j * b1.y);
                if (!fast) {
                    if (tx >= hw) tx -= hw; else if (tx < 0) tx += hw;
                    if (ty >= hh) ty -= hh; else if (ty < 0) ty += hh;
                }
                float4 tb, to;
                sample2<true, HW>(P.ex, li, LBO, tx, ty, &tb, &to, fast);
                float res = ssd_ap(base, tb, P.alphaWeight) * P.inputAnalogyWeight;
                if (TM) {
                    if (px.temporal) {
                        float4 pbase = T.pbase[s], pout = T.pout[s];
                        float ptx = px.prev.x + fmaf((float)i, px.pb0.x, (float)j * px.pb1.x);
                        float pty = px.prev.y + fmaf((float)i, px.pb0.y, (float)j * px.pb1.y);
                        float4 peb, peo;
                        sample2<true, HW>(P.ex, lpi, P.ex.bo + 2 * lp, ptx, pty, &peb, &peo, fastp);
                        float r = ssdp(sub4p(base, pbase), sub4p(tb, peb)) * P.tdIn;
                        r = fmaf(ssdp(sub4p(canvas, pout), sub4p(to, peo)), P.tdOut, r);
                        r = fmaf(ssdp(pout, to), P.tc, r);
                        res = (T.prec[s].x > 0) ? res + r : res;
                    }
                }
                if (i == 0 && j == 0) {
                    if (P.distTransWeight > 0.f) {
                        float de = ex_sample_dt(ex_mode<HW>(P.ex), tx, ty, c.layer) / c.sv;
                        float di = lay_texel(P.img.dt[P.img.cur], P, px.x, px.y);
                        float diff = fmaxf(0.0f, fminf(fabsf(de - di), 10.0f));  // clamp(diff, 0, 10): a NaN difference gives 10
                        res = res + diff * P.distTransWeight;
                    }
                    {
                        int Lh = clampi(c.layer, 0, PT_MAX_STYLES - 1);
                        float sh = (float)(P.histH / P.numStyles);
                        int hx = clampi((int)tx, 0, P.histPitch - 1);
                        int hy = clampi((int)(ty + sh * (float)c.layer), 0, P.histRows - 1);
                        float h = __ldg(P.hist + (size_t)hy * P.histPitch + hx);
                        float thr = P.histThreshold[Lh];
                        res = res + ((h > thr) ? (h - thr) * P.histSlope[Lh] : 0.0f);
                    }
                    if (P.styleObjIdWeight > 0.f) {
                        int imgID = lvl_texel(P.img.ids, px.x, px.y);
                        int styleID = ex_point_id(P.ex, tx, ty, c.layer);
                        res = res + ((imgID != styleID) ? P.styleObjIdWeight : 0.0f);
                    }
                } else {
                    res = fmaf(ssd_ap(canvas, to, P.alphaWeight), P.canvasOutputWeight, res);
                }
                const float w = P.gauss[i + R] * P.gauss[j + R];
                sum = valid ? fmaf(res, w, sum) : sum;
            }
            if (EE) act = !(sum >= thr2);
        }
    }
    if (P.counters) count_taps(P, taps_done<R>(px, cols), px.temporal);
    if (px.sumW < kEpsilon) return kBigResidual;
    if (EE && sum >= thr2) return INFINITY;
    return sum / px.sumW;
}

template <int R, int TM, int HW, bool EE>
__device__ __forceinline__ float energy_tiled(const Params& P, const TileSmem<R, TM>& T, const PixT& px,
                                           const Cand& c, float best) {
    float sum0 = 0.0f;
    if (px.hyst_on) sum0 = sum0 - px.hyst;
    float2 b0, b1;
    basis(c.theta, P.scaleWU * c.su, P.scaleWV * c.sv, &b0, &b1);
    const unsigned mask = __activemask();
    bool fast = __all_sync(mask, footprint_inside<R>(c.x, c.y, b0, b1, P.ex.w, P.ex.h));
    bool fastp = TM ? __all_sync(mask, !px.temporal || px.prev_fast) : true;
    return energy_taps<R, TM, HW, EE>(P, T, px, c, b0, b1, sum0, fast, fastp,
                                  EE ? exit_threshold(P, px, best) : kNoBest);
}

// Tensor copies into shared memory (cp.async.bulk.tensor) completing on an
// mbarrier.  Every wait is bounded: kWaitLimit polls of mbarrier.try_wait,
// each of which may suspend the thread for a short hardware time limit.
constexpr int kWaitLimit = 1 << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// box (x, y) of a 2-D tensor map into shared memory at dst, counted on bar
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// waits for the barrier's phase `parity` to complete; false if it did not
// within the limit
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
#pragma unroll 1
    for (int i = 0; i < kWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Stages the tile (and halo) of the pixel-side inputs and fills the
// per-pixel state.  Returns false for threads whose pixel is outside the
// level rectangle (and for the threads of a block of NT > kTileThreads
// threads past the tile's pixels, which only evaluate candidates).  A tile whose halo lies inside the level rectangle, where
// the clamps are no-ops, is copied by tensor copies when the maps are on
// (one thread issues them; the texture mode's flush of subnormal input
// colours follows in shared memory); the others load texel by texel with
// the clamp rules.  *abort is set (for the whole block) when the copies did
// not complete within two bounded waits; the block must then return.
template <int R, int TM, int NT = kTileThreads>
__device__ __forceinline__ bool stage_tile(const Params& P, const TileMaps& M, TileSmem<R, TM>& T, PixT* px,
                                           bool* abort) {
    constexpr int TW = TileSmem<R, TM>::TW, TH = TileSmem<R, TM>::TH, N = TileSmem<R, TM>::N;
    const int tid = threadIdx.x + threadIdx.y * kTileW;
    const int x0 = blockIdx.x * kTileW - R, y0 = blockIdx.y * kTileH - R;
    *abort = false;
    const bool interior = M.on && x0 >= 0 && y0 >= 0 && x0 + TW <= P.lw && y0 + TH <= P.lh;  // (block-uniform)
    if (interior) {
        const uint32_t bar = smem_addr(&T.bar);
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (tid == 0) {
            const uint32_t bytes = (uint32_t)(N * sizeof(float4)) * (TM ? 5u : 2u);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
            // x in FLOAT32 elements: 4 per texel, so x * 4 bytes is a multiple of 16
            tma_load_2d(T.base, &M.base, 4 * x0, y0, bar);
            tma_load_2d(T.canvas, &M.canvas, 4 * x0, y0, bar);
            if (TM) {
                tma_load_2d(T.pbase, &M.pbase, 4 * x0, y0, bar);
                tma_load_2d(T.pout, &M.pout, 4 * x0, y0, bar);
                tma_load_2d(T.prec, &M.prec, 4 * x0, y0, bar);
            }
        }
    } else {
        const Arr<float4>& ib = P.img.base[P.img.cur];
        for (int q = tid; q < N; q += NT) {
            int gx = clampi(x0 + q % TW, 0, P.lw - 1);
            int gy = clampi(y0 + q / TW, 0, P.lh - 1);
            size_t k = (size_t)gy * P.W + gx;
            T.base[q] = lin_texel_of(__ldg(ib.p + (size_t)gy * ib.w + gx), P.hwFilter);
            T.canvas[q] = __ldg(P.canvas + k);
            if (TM) {
                const AdvView& A = P.adv[TM == TM_FWD ? 0 : 1];
                T.pbase[q] = __ldg(A.base + k);
                T.pout[q] = __ldg(A.out + k);
                T.prec[q] = __ldg(A.off.B + k);
            }
        }
    }
    // the per-pixel state reads global memory only: with tensor copies it is
    // computed while they are in flight
    const int x = blockIdx.x * kTileW + threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
    const bool in = tid < kTileThreads && x < P.lw && y < P.lh;  // (threads past the tile's pixels only evaluate)
    if (in) {
        px->x = x;
        px->y = y;
        px->sidx = (threadIdx.y + R) * TW + threadIdx.x + R;
        px->imin = max(-R, -x); px->imax = min(R, P.lw - 1 - x);
        px->jmin = max(-R, -y); px->jmax = min(R, P.lh - 1 - y);
        {
            float sw = 0.0f;
#pragma unroll 1
            for (int i = -R; i <= R; i++)
#pragma unroll
                for (int j = -R; j <= R; j++) {
                    const bool valid = (i >= px->imin) && (i <= px->imax) && (j >= px->jmin) && (j <= px->jmax);
                    const float w = P.gauss[i + R] * P.gauss[j + R];
                    sw = valid ? sw + w : sw;
                }
            px->sumW = sw;
        }
        const size_t k = (size_t)y * P.W + x;
        px->hyst_on = false;
        px->hyst = 0.0f;
        if (P.hysteresisWeight != 0.0f) {
            px->hyst_on = __ldg(&P.adv[0].off.B[k].x) > 0;
            if (px->hyst_on) px->hyst = hysteresis_term(P, x, y);
        }
        px->temporal = false;
        px->prev_fast = false;
        if (TM) {
            px->prev = load_patch(P.adv[TM == TM_FWD ? 0 : 1].off, k);
            bool td = (P.tdIn > 0.f || P.tdOut > 0.f || P.tc > 0.f);
            px->temporal = td && px->prev.hyst > 0;
            if (px->temporal) {
                float a = screen_to_exemplar_angle(P, x, y, px->prev.x, px->prev.y, px->prev.layer);
                basis(a, P.scaleWU * px->prev.su, P.scaleWV * px->prev.sv, &px->pb0, &px->pb1);
                px->prev_fast = footprint_inside<R>(px->prev.x, px->prev.y, px->pb0, px->pb1, P.ex.w, P.ex.h);
            }
        }
    }
    if (interior) {
        const uint32_t bar = smem_addr(&T.bar);
        bool ok = mbar_wait(bar, 0);
        if (!ok) ok = mbar_wait(bar, 0);  // the copies still in flight, once more
        if (__syncthreads_or(!ok)) {
            if (tid == 0 && M.err) atomicExch(M.err, 1);
            *abort = true;
            return false;
        }
        if (P.hwFilter)
            for (int q = tid; q < N; q += NT) T.base[q] = lin_texel_of(T.base[q], 1);
    }
    __syncthreads();
    return in;
}

// the four propagate sources of pixel (x, y), in the reference's order
__device__ __forceinline__ void propagate_source(int cdx, int x, int y, int jump, int* tx, int* ty) {
    *tx = x;
    *ty = y;
    if (cdx == 0) *tx = x + jump;
    else if (cdx == 1) *tx = x - jump;
    else if (cdx == 2) *ty = y + jump;
    else *ty = y - jump;
}

// A block whose pixels need no energy (change tracking skipped all their
// candidates) copies its records and stops before staging its tile.
// (write: the working buffer needs every record written)
__device__ __forceinline__ bool block_idle(const Params& P, PatchPlanes work, bool need, bool in, size_t k,
                                           bool write = true) {
    if (__syncthreads_or(need)) return false;
    if (in) {
        if (write) store_patch(work, k, load_patch(P.off, k));
        P.inc.chg[k] = 0;
    }
    return true;
}

// updateResidualCache_kernel, texSynth_kernel.cu:661-693
template <int R, int TM, int HW>
__global__ void __launch_bounds__(kTileThreads, 2) kt_residual(const Params P, const __grid_constant__ TileMaps M,
                                                                    float* out) {
    __shared__ TileSmem<R, TM> T;
    // Change tracking: only pixels with a changed record in their patch
    // window get a new residual; the others keep theirs (the same inputs give
    // the same value).  The pass stamps are updated here.
    bool need = true;
    if (P.inc.on) {
        constexpr int TW = TileSmem<R, TM>::TW, N = TileSmem<R, TM>::N;
        __shared__ uint8_t C[N];
        const int tid = threadIdx.x + threadIdx.y * kTileW;
        const int x0 = blockIdx.x * kTileW - R, y0 = blockIdx.y * kTileH - R;
        for (int q = tid; q < N; q += kTileThreads) {
            int gx = clampi(x0 + q % TW, 0, P.lw - 1);
            int gy = clampi(y0 + q / TW, 0, P.lh - 1);
            C[q] = P.inc.chg[(size_t)gy * P.W + gx];
        }
        __syncthreads();
        const int x = blockIdx.x * kTileW + threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
        const bool in = x < P.lw && y < P.lh;
        need = false;
        if (in) {
            const int c0 = threadIdx.y * TW + threadIdx.x;  // window corner
            unsigned any = 0;
#pragma unroll
            for (int j = 0; j <= 2 * R; j++)
#pragma unroll
                for (int i = 0; i <= 2 * R; i++) any |= C[c0 + j * TW + i];
            need = any != 0;
            const size_t k = (size_t)y * P.W + x;
            if (C[c0 + R * TW + R]) P.inc.last[k] = P.inc.pi;
            if (need) P.inc.win[k] = P.inc.pi;
        }
        if (!__syncthreads_or(need)) return;
    }
    PixT px;
    bool abort;
    if (!stage_tile<R, TM>(P, M, T, &px, &abort)) return;
    if (!need) return;
    const size_t k = (size_t)px.y * P.W + px.x;
    if (image_culled(P, px.x, px.y)) { out[k] = 0.0f; return; }
    Patch t = load_patch(P.off, k);
    Cand c{t.x, t.y, t.theta, t.su, t.sv, t.layer};
    if (P.counters) count_eval(P, px.x, px.y, px.temporal, false);
    out[k] = energy_tiled<R, TM, HW, false>(P, T, px, c, kNoBest);
}

// ---------------------------------------------------------------------------
// Lane cursors.  In the kernels below every lane evaluates one candidate at
// a time, one column of 2R+1 taps per step, and takes its next candidate as
// soon as the current one is finished or stopped early, instead of waiting
// for the slowest lane of its warp.  Propagate and residual take their
// candidates from a queue in shared memory, so any lane may evaluate any
// pixel of the tile (the pixel-side context is in shared memory too);
// scatter's lanes each follow their own pixel's chain.  A candidate's sum
// still runs over its taps in the reference's order, so every energy is
// bit-identical to a separate evaluation.
// ---------------------------------------------------------------------------

constexpr unsigned kFull = 0xffffffffu;
// (1 -/+ 2^-17): bounds of the rounding of a reference-order sum of <= 81 terms
constexpr float kBoundLo = 1.0f - 1.0f / 131072.0f;
constexpr float kBoundHi = 1.0f + 1.0f / 131072.0f;
// Propagate takes no bound pass: its candidates come from coherent
// neighbours, so their energies are mostly close to the best and a bound
// pass rarely rejects them before its end (measured: 1 or 2 groups of 2R+1
// taps +45-53 %, the full pass +20 % propagate time); scatter's
// random-search candidates are rejected after a few heavy taps (full bound
// pass: -45 % scatter time).

// pixel side of an evaluation
struct LanePix {
    int x, y, sidx;
    int imin, imax, jmin, jmax;
    float sum0, sumW;
    bool temporal, prev_fast;
    float prevx, prevy;
    int prevlayer;  // clamped to the exemplar's layers
    float2 pb0, pb1;
};

// candidate side of an evaluation and its cursor
struct LaneEval {
    float cx, cy, sv;
    int layer;
    float2 b0, b1;
    bool fast;   // footprint inside the exemplar
    bool exact;  // the reference-order pass (else the bound pass)
    int col;     // exact pass: next column, -R..R; bound pass: next position in the weight order
    float sum;   // exact pass: the running sum; bound pass: the lower bound of the weighted taps so far
    float thr2;  // exit threshold (see exit_threshold)
    float s0lo;  // lower bound of the start sum's share of the reference-order sum
};

// The taps of the window by descending weight, with their weights, for the
// bound pass; filled once per block from Params::tapOrder.
template <int R>
struct TapTable {
    uint8_t ij[(2 * R + 1) * (2 * R + 1)];  // (i + R) | (j + R) << 4
    float w[(2 * R + 1) * (2 * R + 1)];
};
template <int R>
__device__ __forceinline__ void load_tap_table(const Params& P, TapTable<R>& TT) {
    constexpr int n = 2 * R + 1, K = n * n;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if (tid < K) {
        const int t = P.tapOrder[tid];
        const int i = t / n, j = t % n;
        TT.ij[tid] = (uint8_t)(i | (j << 4));
        TT.w[tid] = P.gauss[i] * P.gauss[j];
    }
}

template <int R>
__device__ __forceinline__ LanePix lane_pix(const Params& P, const PixT& px) {
    LanePix q;
    q.x = px.x; q.y = px.y; q.sidx = px.sidx;
    q.imin = px.imin; q.imax = px.imax; q.jmin = px.jmin; q.jmax = px.jmax;
    q.sum0 = px.hyst_on ? 0.0f - px.hyst : 0.0f;
    q.sumW = px.sumW;
    q.temporal = px.temporal;
    q.prev_fast = px.prev_fast;
    q.prevx = px.prev.x; q.prevy = px.prev.y;
    q.prevlayer = ex_layer(P.ex, px.prev.layer);
    q.pb0 = px.pb0; q.pb1 = px.pb1;
    return q;
}

// the pixel contexts of a tile in shared memory
struct PixShared {
    float4 a[kTileThreads];  // sum0, sumW, prev x, prev y
    float4 b[kTileThreads];  // prev basis
    int bits[kTileThreads];  // window bounds + R (4 bits each), temporal, prev_fast, prev layer
};

template <int R>
__device__ __forceinline__ void put_pix(PixShared& S, int pid, const LanePix& q) {
    S.a[pid] = make_float4(q.sum0, q.sumW, q.prevx, q.prevy);
    S.b[pid] = make_float4(q.pb0.x, q.pb0.y, q.pb1.x, q.pb1.y);
    S.bits[pid] = (q.imin + R) | ((q.imax + R) << 4) | ((q.jmin + R) << 8) | ((q.jmax + R) << 12) |
                  (q.temporal ? 1 << 16 : 0) | (q.prev_fast ? 1 << 17 : 0) | (q.prevlayer << 18);
}

template <int R, int TM>
__device__ __forceinline__ LanePix get_pix(const Params& P, const PixShared& S, int pid) {
    constexpr int TW = TileSmem<R, TM>::TW;
    LanePix q;
    const int lx = pid % kTileW, ly = pid / kTileW;
    q.x = blockIdx.x * kTileW + lx;
    q.y = blockIdx.y * kTileH + ly;
    q.sidx = (ly + R) * TW + lx + R;
    const float4 a = S.a[pid], b = S.b[pid];
    const int bits = S.bits[pid];
    q.imin = (bits & 15) - R; q.imax = ((bits >> 4) & 15) - R;
    q.jmin = ((bits >> 8) & 15) - R; q.jmax = ((bits >> 12) & 15) - R;
    q.temporal = (bits >> 16) & 1;
    q.prev_fast = (bits >> 17) & 1;
    q.prevlayer = bits >> 18;
    q.sum0 = a.x; q.sumW = a.y; q.prevx = a.z; q.prevy = a.w;
    q.pb0 = make_float2(b.x, b.y); q.pb1 = make_float2(b.z, b.w);
    return q;
}

// best = the energy to beat (kNoBest: none, the energy is computed in full)
template <int R>
__device__ __forceinline__ void lane_start(const Params& P, const LanePix& q, float cx, float cy, float theta,
                                           float su, float sv, int layer, float best, LaneEval* e) {
    e->cx = cx; e->cy = cy; e->sv = sv; e->layer = layer;
    basis(theta, P.scaleWU * su, P.scaleWV * sv, &e->b0, &e->b1);
    e->fast = footprint_inside<R>(cx, cy, e->b0, e->b1, P.ex.w, P.ex.h);
    e->thr2 = (P.earlyExit && q.sumW >= kEpsilon) ? __fmul_ru(best, q.sumW) : kNoBest;
    // With an exit threshold, a bound pass over the taps by descending
    // weight comes first (see lane_step); without one, or with one so small
    // (|thr2| < 2^-100) that subnormal rounding could matter, only the exact
    // pass.
    e->exact = !(fabsf(e->thr2) >= 0x1p-100f);
    e->col = e->exact ? -R : 0;
    e->sum = e->exact ? q.sum0 : 0.0f;
    e->s0lo = q.sum0 >= 0.0f ? __fmul_rd(q.sum0, kBoundLo) : __fmul_rd(q.sum0, kBoundHi);
}

// The exemplar samples of tap (i, j) of candidate e at pixel q (and, for a
// temporal pixel, of its previous offset), with the sample position.
struct TapSample {
    float4 tb, to, peb, peo;
    float tx, ty;
};

template <int R, int TM, int HW>
__device__ __forceinline__ void tap_fetch(const Params& P, const LanePix& q, const LaneEval& e, int i, int j,
                                          bool fast, bool fastp, TapSample* t) {
    const size_t lsz = (size_t)P.ex.w * P.ex.h;
    const int li = ex_layer(P.ex, e.layer);
    const size_t lo = (size_t)li * lsz;
    const float4* LBO = P.ex.bo + 2 * lo;
    const size_t lp = TM ? (size_t)q.prevlayer * lsz : 0;
    const float hw = (float)P.histW, hh = (float)P.histH;
    float tx = e.cx + fmaf((float)i, e.b0.x, (float)j * e.b1.x);
    float ty = e.cy + fmaf((float)i, e.b0.y, (float)j * e.b1.y);
    if (!fast) {
        if (tx >= hw) tx -= hw; else if (tx < 0) tx += hw;
        if (ty >= hh) ty -= hh; else if (ty < 0) ty += hh;
    }
    sample2<true, HW>(P.ex, li, LBO, tx, ty, &t->tb, &t->to, fast);
    t->tx = tx;
    t->ty = ty;
    if (TM && q.temporal) {
        float ptx = q.prevx + fmaf((float)i, q.pb0.x, (float)j * q.pb1.x);
        float pty = q.prevy + fmaf((float)i, q.pb0.y, (float)j * q.pb1.y);
        sample2<true, HW>(P.ex, TM ? q.prevlayer : 0, P.ex.bo + 2 * lp, ptx, pty, &t->peb, &t->peo, fastp);
    }
}

// calculateResidual's value at tap (i, j) of candidate e at pixel q, before
// its Gaussian weight (texSynth_kernel.cu:537-659), from the tap's samples
template <int R, int TM, int HW>
__device__ __forceinline__ float tap_finish(const Params& P, const TileSmem<R, TM>& T, const LanePix& q,
                                            const LaneEval& e, int i, int j, const TapSample& t) {
    constexpr int TW = TileSmem<R, TM>::TW;
    const int s = q.sidx + j * TW + i;
    const float4 base = T.base[s];
    const float4 canvas = T.canvas[s];
    const float4 tb = t.tb, to = t.to;
    const float tx = t.tx, ty = t.ty;
    float res = ssd_ap(base, tb, P.alphaWeight) * P.inputAnalogyWeight;
    if (TM) {
        if (q.temporal) {
            const float4 pbase = T.pbase[s], pout = T.pout[s];
            float r = ssdp(sub4p(base, pbase), sub4p(tb, t.peb)) * P.tdIn;
            r = fmaf(ssdp(sub4p(canvas, pout), sub4p(to, t.peo)), P.tdOut, r);
            r = fmaf(ssdp(pout, to), P.tc, r);
            res = (T.prec[s].x > 0) ? res + r : res;
        }
    }
    if (j == 0 && i == 0) {
        if (P.distTransWeight > 0.f) {
            float de = ex_sample_dt(ex_mode<HW>(P.ex), tx, ty, e.layer) / e.sv;
            float di = lay_texel(P.img.dt[P.img.cur], P, q.x, q.y);
            float diff = fmaxf(0.0f, fminf(fabsf(de - di), 10.0f));  // clamp(diff, 0, 10): a NaN difference gives 10
            res = res + diff * P.distTransWeight;
        }
        {
            int Lh = clampi(e.layer, 0, PT_MAX_STYLES - 1);
            float sh = (float)(P.histH / P.numStyles);
            int hx = clampi((int)tx, 0, P.histPitch - 1);
            int hy = clampi((int)(ty + sh * (float)e.layer), 0, P.histRows - 1);
            float h = __ldg(P.hist + (size_t)hy * P.histPitch + hx);
            float thr = P.histThreshold[Lh];
            res = res + ((h > thr) ? (h - thr) * P.histSlope[Lh] : 0.0f);
        }
        if (P.styleObjIdWeight > 0.f) {
            int imgID = lvl_texel(P.img.ids, q.x, q.y);
            int styleID = ex_point_id(P.ex, tx, ty, e.layer);
            res = res + ((imgID != styleID) ? P.styleObjIdWeight : 0.0f);
        }
    } else {
        res = fmaf(ssd_ap(canvas, to, P.alphaWeight), P.canvasOutputWeight, res);
    }
    return res;
}

// calculateResidual's value at tap (i, j) of candidate e at pixel q, before
// its Gaussian weight; fast / fastp are warp-uniform
template <int R, int TM, int HW>
__device__ __forceinline__ float tap_value(const Params& P, const TileSmem<R, TM>& T, const LanePix& q,
                                           const LaneEval& e, int i, int j, bool fast, bool fastp) {
    TapSample t;
    tap_fetch<R, TM, HW>(P, q, e, i, j, fast, fastp, &t);
    return tap_finish<R, TM, HW>(P, T, q, e, i, j, t);
}

// the taps of column e.col added to e.sum in the reference's order.  ROLL
// keeps the column's taps in a loop (a smaller body: faster for scatter,
// whose chain code competes for the instruction cache; propagate unrolls).
// EE: a lane leaves the column as soon as its sum reaches e.thr2 (the sum
// only grows, so stopping at any tap gives the decision of stopping at the
// column's end), and the loads of its remaining taps are not issued.
// With the texture unit each tap's fetches are issued before the previous
// tap's sum and exit test (one tap ahead), so two taps' fetch latencies
// overlap; a lane that exits has fetched one tap more than it uses.
template <int R, int TM, int HW, bool ROLL, bool EE>
__device__ __forceinline__ float lane_column(const Params& P, const TileSmem<R, TM>& T, const LanePix& q,
                                             const LaneEval& e, bool fast, bool fastp) {
    const int i = e.col;
    const bool cvalid = (i >= q.imin) && (i <= q.imax);
    const float gi = P.gauss[i + R];
    float sum = e.sum;
    if constexpr (HW && !ROLL) {
        TapSample cur, nxt;
        tap_fetch<R, TM, HW>(P, q, e, i, -R, fast, fastp, &cur);
#pragma unroll
        for (int j = -R; j <= R; j++) {
            if (j < R) tap_fetch<R, TM, HW>(P, q, e, i, j + 1, fast, fastp, &nxt);
            const bool valid = cvalid && (j >= q.jmin) && (j <= q.jmax);
            const float res = tap_finish<R, TM, HW>(P, T, q, e, i, j, cur);
            const float w = gi * P.gauss[j + R];
            sum = valid ? fmaf(res, w, sum) : sum;
            if (EE && sum >= e.thr2) break;
            cur = nxt;
        }
        return sum;
    } else {
#pragma unroll(ROLL ? 1 : 2 * R + 1)
        for (int j = -R; j <= R; j++) {
            const bool valid = cvalid && (j >= q.jmin) && (j <= q.jmax);
            const float res = tap_value<R, TM, HW>(P, T, q, e, i, j, fast, fastp);
            const float w = gi * P.gauss[j + R];
            sum = valid ? fmaf(res, w, sum) : sum;
            if (EE && sum >= e.thr2) break;
        }
        return sum;
    }
}

// taps of the first `cols` columns inside the level rectangle
template <int R>
__device__ __forceinline__ unsigned lane_taps(const LanePix& q, int cols) {
    const int last = min(-R + cols - 1, q.imax);
    return last < q.imin ? 0u : (unsigned)((last - q.imin + 1) * (q.jmax - q.jmin + 1));
}

// One step of a lane: the next column (2R+1 taps) of its candidate in the
// reference's order; returns true when the candidate is finished, with its
// energy in *r (kBigResidual where the tap weights sum below kEpsilon, +inf
// where it was rejected early).  The sum is formed as calculateResidual forms
// it (texSynth_kernel.cu:537-659), exiting early on it.  (Propagate's
// candidates come from coherent neighbours and mostly tie with the best, so
// it takes this exact pass alone; scatter's chains take a bound pass first,
// lane_step_uni below.)
template <int R, int TM, int HW, bool EE, bool ROLL>
__device__ __forceinline__ bool lane_step(const Params& P, const TileSmem<R, TM>& T, const LanePix& q, LaneEval& e,
                                          bool fast, bool fastp, float* r) {
    if (!e.exact) {
        e.exact = true;
        e.col = -R;
        e.sum = q.sum0;
    }
    e.sum = lane_column<R, TM, HW, ROLL, EE>(P, T, q, e, fast, fastp);
    e.col++;
    const bool stop = EE && e.sum >= e.thr2;
    if (!stop && e.col <= R) return false;
    if (P.counters) count_taps(P, lane_taps<R>(q, e.col + R), q.temporal);
    *r = (q.sumW < kEpsilon) ? kBigResidual : stop ? INFINITY : e.sum / q.sumW;
    return true;
}

// One step of a lane of scatter's chains: with an exit threshold a
// candidate first takes a bound pass, its taps by descending weight (TT),
// accumulating a lower bound of the weighted sum with round-down products and
// sums.  The reference forms its sum in tap order with round-to-nearest fmaf
// over at most 81 non-negative terms, which is at least (1 - 2^-17) times the
// exact sum of those terms, plus its start sum (the hysteresis term, <= 0)
// scaled by at most (1 + 2^-17).  So once (1 - 2^-17) * bound + that
// start-sum share, rounded down, reaches thr2 = best * sumW rounded up, the
// reference-order energy is >= best and the strict "<" rejects the
// candidate.  The heavy central taps come first, so a rejection needs a few
// taps instead of several columns.  A candidate the bound pass does not
// reject (a winner or a near tie) then takes the exact pass, lane_step's.
// Both passes share one loop body: a step is up to 2R+1 taps, by descending
// weight (bound pass: round-down products and sums, the bound test) or the
// next column in the reference's order (exact pass: fmaf, the exact test),
// chosen per lane by data, so the lanes of a warp in different passes issue
// the same instructions instead of the two passes' code in turn.
template <int R, int TM, int HW>
__device__ __forceinline__ bool lane_step_uni(const Params& P, const TileSmem<R, TM>& T, const TapTable<R>& TT,
                                              const LanePix& q, LaneEval& e, bool fast, bool fastp, float* r) {
    constexpr int K = (2 * R + 1) * (2 * R + 1);
    const bool bound = !e.exact;
    bool hit = false;  // the pass's test reached its threshold
#pragma unroll 1
    for (int k = 0; k < 2 * R + 1; k++) {
        const int pos = e.col + k;
        if (bound && pos >= K) break;
        int i, j;
        float w;
        if (bound) {
            const int ij = TT.ij[pos];
            i = (ij & 15) - R;
            j = (ij >> 4) - R;
            w = TT.w[pos];
        } else {
            i = e.col;
            j = k - R;
            w = P.gauss[i + R] * P.gauss[j + R];
        }
        const bool valid = (i >= q.imin) && (i <= q.imax) && (j >= q.jmin) && (j <= q.jmax);
        const float res = tap_value<R, TM, HW>(P, T, q, e, i, j, fast, fastp);
        const float sb = __fadd_rd(e.sum, __fmul_rd(res, w));
        const float sx = fmaf(res, w, e.sum);
        e.sum = valid ? (bound ? sb : sx) : e.sum;
        hit = bound ? (__fadd_rd(__fmul_rd(e.sum, kBoundLo), e.s0lo) >= e.thr2) : (e.sum >= e.thr2);
        if (hit) break;
    }
    if (bound) {
        e.col += 2 * R + 1;
        if (hit) {
            if (P.counters) count_taps(P, (unsigned)min(e.col, K), q.temporal);
            *r = INFINITY;
            return true;
        }
        if (e.col >= K) {  // not rejected: the exact pass
            if (P.counters) count_taps(P, (unsigned)K, q.temporal);
            e.exact = true;
            e.col = -R;
            e.sum = q.sum0;
        }
        return false;
    }
    e.col++;
    if (!hit && e.col <= R) return false;
    if (P.counters) count_taps(P, lane_taps<R>(q, e.col + R), q.temporal);
    *r = (q.sumW < kEpsilon) ? kBigResidual : hit ? INFINITY : e.sum / q.sumW;
    return true;
}

// a lane's index in a shared queue: warp-aggregated atomic on *next
__device__ __forceinline__ int queue_take(bool want, int* next) {
    const unsigned m = __ballot_sync(kFull, want);
    const int lane = (int)lane_id();
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(next, __popc(m));
    base = __shfl_sync(kFull, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// candidates of a propagate tile
struct PropQueue {
    float4 ca[kTileThreads * 4];     // x, y, theta, su; x holds the energy once evaluated
    float2 cb[kTileThreads * 4];     // sv, layer bits
    uint16_t list[kTileThreads * 4];  // pid * 4 + slot
    float thr[kTileThreads];          // the pixel's residual
    int slots[kTileThreads];          // per candidate (3 bits each): slot + 3, or 0 skipped, 1 repeat, 2 rejected
    int count[kTileH], next[kTileH];  // per warp: its row's candidates (list[128 * warp ...])
};

// propagate_kernel with lane cursors over the tile's candidates.  WIDE
// warps per tile row: with WIDE = 2 the block has twice the tile's threads
// and the second half only takes candidates from the rows' queues (the same
// candidates and results, evaluated by twice the lanes: for the coarse
// levels, whose few tiles leave most of the GPU idle).
template <int R, int TM, int HW, int WIDE>
__global__ void __launch_bounds__(kTileThreads * WIDE, WIDE == 1 ? 2 : 1)
    kt_propagate_q(const Params P, const __grid_constant__ TileMaps M, PatchPlanes work, int jump) {
    const int pid = threadIdx.x + threadIdx.y * kTileW;
    __shared__ TileSmem<R, TM> T;
    __shared__ PixShared S;
    __shared__ PropQueue Q;
    // Change tracking: a candidate whose source record and whose target's
    // patch window are unchanged since the previous pass with this jump was
    // rejected there against the same residual and is skipped (bit cdx of
    // `skip`); a pass without a previous one skips nothing.
    unsigned skip = 0;
    if (P.inc.on) {
        const int x = blockIdx.x * kTileW + threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
        const bool in = pid < kTileThreads && x < P.lw && y < P.lh;
        const size_t k = (size_t)y * P.W + x;
        bool need = in;
        if (in && P.inc.prev != INT_MIN && __ldg(P.inc.win + k) < P.inc.prev) {
#pragma unroll
            for (int cdx = 0; cdx < 4; cdx++) {
                int tx, ty;
                propagate_source(cdx, x, y, jump, &tx, &ty);
                if (__ldg(P.inc.last + pixel_wrap_index(P, tx, ty)) < P.inc.prev) skip |= 1u << cdx;
            }
            need = skip != 0xFu && !image_culled(P, x, y);
        }
        if (block_idle(P, work, need, in, k)) return;
    }
    if (pid < kTileH) { Q.count[pid] = 0; Q.next[pid] = 0; }
    PixT px;
    bool abort;
    const bool in = stage_tile<R, TM, kTileThreads * WIDE>(P, M, T, &px, &abort);  // (synchronises the block)
    if (abort) return;
    // phase 1: each pixel builds its candidates (the reference's order,
    // repeats and test_offset rejections resolved here) and queues them
    int n = 0;
    bool culled = false;
    if (in) {
        const int x = px.x, y = px.y;
        const size_t k = (size_t)y * P.W + x;
        culled = image_culled(P, x, y);
        if (culled) {
            const Patch z = make_patch(0, 0, 0, 0, 0, 1.f, 1.f);
            if (P.inc.on) P.inc.chg[k] = same_record(z, load_patch(P.off, k)) ? 0 : 1;
            store_patch(work, k, z);
        } else {
            const float ia = T.base[px.sidx].w;
            uint32_t kx[4], ky[4], kt[4];
            int kl[4];
            int codes = 0;
#pragma unroll
            for (int cdx = 0; cdx < 4; cdx++) {
                kx[cdx] = ky[cdx] = kt[cdx] = 0u;
                kl[cdx] = 0;
                int code = 2;  // rejected before the energy
                if (skip & (1u << cdx)) {
                    code = 0;
                } else {
                    int tx, ty;
                    propagate_source(cdx, x, y, jump, &tx, &ty);
                    Patch t = propagate_offset(P, tx, ty, x, y);
                    kx[cdx] = __float_as_uint(t.x);
                    ky[cdx] = __float_as_uint(t.y);
                    kt[cdx] = __float_as_uint(t.theta);
                    kl[cdx] = t.layer;
                    bool dup = false;
#pragma unroll
                    for (int q = 0; q < cdx; q++)
                        dup |= !(skip & (1u << q)) && kx[q] == kx[cdx] && ky[q] == ky[cdx] && kt[q] == kt[cdx] &&
                               kl[q] == kl[cdx];
                    if (dup) {
                        code = 1;
                    } else {
                        float dte = ex_texel_dt(ex_mode<HW>(P.ex), (int)t.x, (int)t.y, t.layer);
                        bool ok = !((double)dte > (double)P.distTransCull * 1.25);
                        if (ok && !P.transparencyOk) {
                            float ea = ex_sample_out_alpha(ex_mode<HW>(P.ex), t.x, t.y, t.layer);
                            ok = !(ea < kAlphaThreshold && ia > kAlphaThreshold);
                        }
                        if (ok) {
                            if (P.counters) count_eval(P, x, y, px.temporal, false);
                            Q.ca[pid * 4 + n] = make_float4(t.x, t.y, t.theta, t.su);
                            Q.cb[pid * 4 + n] = make_float2(t.sv, __int_as_float(t.layer));
                            code = n + 3;
                            n++;
                        }
                    }
                }
                codes |= code << (3 * cdx);
            }
            Q.slots[pid] = codes;
            Q.thr[pid] = __ldg(P.res + k);
            put_pix<R>(S, pid, lane_pix<R>(P, px));
        }
    }
    if (pid < kTileThreads) {  // (whole warps)
        // queue this pixel's n candidates
        const unsigned lane = lane_id();
        int incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(kFull, incl, o);
            if ((int)lane >= o) incl += v;
        }
        // each warp queues its own row's candidates, so that its lanes
        // gather from neighbouring exemplar regions (a coherent field maps
        // neighbouring pixels to neighbouring texels)
        const int warp = pid / kTileW;
        if (lane == 31) Q.count[warp] = incl;
        for (int j = 0; j < n; j++) Q.list[warp * 4 * kTileW + incl - n + j] = (uint16_t)(pid * 4 + j);
    }
    __syncthreads();
    // phase 2: lane cursors over the queue
    {
        LanePix q;
        LaneEval e;
        bool act = false, more = true;
        int cur = 0;
        const int warp = (pid / kTileW) % kTileH;  // the row whose queue this warp takes from
        const int count = Q.count[warp];
#pragma unroll 1
        while (true) {
            const bool want = !act && more;
            if (__any_sync(kFull, want)) {
                const int t = queue_take(want, &Q.next[warp]);
                if (want) {
                    if (t < count) {
                        cur = Q.list[warp * 4 * kTileW + t];
                        const int op = cur >> 2;
                        q = get_pix<R, TM>(P, S, op);
                        const float4 a = Q.ca[cur];
                        const float2 b = Q.cb[cur];
                        lane_start<R>(P, q, a.x, a.y, a.z, a.w, b.x, __float_as_int(b.y), Q.thr[op], &e);
                        act = true;
                    } else {
                        more = false;
                    }
                }
            }
            if (!__any_sync(kFull, act)) break;
            const bool fast = __all_sync(kFull, !act || e.fast);
            const bool fastp = TM ? __all_sync(kFull, !act || !q.temporal || q.prev_fast) : true;
            if (act) {
                float r;
                if (lane_step<R, TM, HW, true, false>(P, T, q, e, fast, fastp, &r)) {
                    Q.ca[cur].x = r;
                    act = false;
                }
            }
        }
    }
    __syncthreads();
    // phase 3: each pixel takes the first candidate, in the reference's
    // order, that beats its running best
    if (in && !culled) {
        const int x = px.x, y = px.y;
        const size_t k = (size_t)y * P.W + x;
        const int codes = Q.slots[pid];
        float best = Q.thr[pid];
        int win = -1;
#pragma unroll
        for (int cdx = 0; cdx < 4; cdx++) {
            const int code = (codes >> (3 * cdx)) & 7;
            // a skipped candidate or a repeat is rejected by "<"; one that
            // test_offset rejected before the energy competes with 1e31
            if (code < 2) continue;
            const float r = code == 2 ? kBigResidual : Q.ca[pid * 4 + code - 3].x;
            if (r < best) { best = r; win = cdx; }
        }
        if (win >= 0) {
            int tx, ty;
            propagate_source(win, x, y, jump, &tx, &ty);
            const Patch ow = propagate_offset(P, tx, ty, x, y);
            if (P.inc.on) P.inc.chg[k] = same_record(ow, load_patch(P.off, k)) ? 0 : 1;
            store_patch(work, k, ow);
        } else {
            if (P.inc.on) P.inc.chg[k] = 0;
            store_patch(work, k, load_patch(P.off, k));
        }
    }
}

// scatter_kernel + averageOffset, texSynth_kernel.cu:841-952, each lane
// running its own pixel's chain with a lane cursor
template <int R, int TM, int HW>
__global__ void __launch_bounds__(kTileThreads, 2) kt_scatter_q(const Params P, const __grid_constant__ TileMaps M,
                                                                     PatchPlanes work, int write_all,
                                                               uint32_t pass_id) {
    __shared__ TileSmem<R, TM> T;
    // Change tracking: with the reference's generator a pixel's candidates
    // follow from its own record and its 3x3 neighbours, so a pixel whose
    // patch window is unchanged since the previous scatter of the loop had
    // every candidate rejected there against the same residual, and again now.
    bool stable = false;
    if (P.inc.on) {
        const int x = blockIdx.x * kTileW + threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
        const bool in = x < P.lw && y < P.lh;
        const size_t k = (size_t)y * P.W + x;
        stable = in && P.inc.prev != INT_MIN && __ldg(P.inc.win + k) < P.inc.prev;
        if (block_idle(P, work, in && !stable, in, k, write_all != 0)) return;
    }
    __shared__ TapTable<R> TT;
    load_tap_table<R>(P, TT);
    PixT px;
    bool abort;
    const bool in = stage_tile<R, TM>(P, M, T, &px, &abort);  // (synchronises the block)
    if (abort) return;
    const int x = px.x, y = px.y;
    const size_t k = (size_t)y * P.W + x;
    bool own = false;
    if (in) {
        if (stable || image_culled(P, x, y)) {
            if (write_all) store_patch(work, k, load_patch(P.off, k));
            if (P.inc.on) P.inc.chg[k] = 0;
        } else {
            own = true;
        }
    }
    // chain state (the reference's loop, :896-937)
    const float cached = own ? __ldg(P.res + k) : 0.0f;
    float best = (float)((double)cached + 10e-7);
    float owx = 0.f, owy = 0.f, owt = 0.f;  // running best offset
    int wkind = 0;                           // 0: the pixel's own, 1: a chain candidate, 2: the average
    float ia = 0.f, dist = 0.f;
    float2 sc = make_float2(0.f, 0.f);
    float avgx = 0.f, avgy = 0.f, avgt = 0.f;
    LanePix q;
    if (own) {
        const float4 a = __ldg(P.off.A + k);
        owx = a.x; owy = a.y;
        ia = T.base[px.sidx].w;
        dist = (float)(P.ex.w > P.ex.h ? P.ex.w : P.ex.h);
        sc = lvl_texel_lin(P.img.scale, x, y, P.hwFilter);
        // averageOffset of the base field (:841-861)
        int na = 0;
        for (int i = -1; i <= 1; i++)
            for (int j = -1; j <= 1; j++) {
                if (!in_rect(P, x + i, y + j) || (i == 0 && j == 0)) continue;
                float4 nb = __ldg(P.off.A + (size_t)(y + j) * P.W + (x + i));
                if (__float_as_int(nb.w) != 0) continue;
                avgx = avgx + nb.x;
                avgy = avgy + nb.y;
                na++;
            }
        avgx = avgx / (float)na;
        avgy = avgy / (float)na;
        avgt = screen_to_exemplar_angle(P, x, y, avgx, avgy, 0);
        q = lane_pix<R>(P, px);
    }
    const float closest = 10.f, factor = 0.9f;
    uint32_t lastx = 0xffffffffu, lasty = 0xffffffffu;
    int i = 0;
    bool avg_pending = true;
    LaneEval e;
    bool act = false, more = own;
    bool cur_avg = false;
    float cur_t = 0.f;
#pragma unroll 1
    while (true) {
        if (!act && more) {
            // the next candidate that needs an energy; one that test_offset
            // rejects first competes with 1e31 right here
#pragma unroll 1
            while (true) {
                bool have = false;
                float ex = 0.f, ey = 0.f;
#pragma unroll 1
                while (i < P.scatterSamples && dist * factor >= closest) {
                    float dmin = dist * factor;
                    if (P.rngMode == PT_RNG_COUNTER) {
                        float rr = counter_u01(P.rngSeed, pass_id, x, y, 2 * i);
                        float th = counter_u01(P.rngSeed, pass_id, x, y, 2 * i + 1) * 6.28318530717958647692f;
                        float sn, cs;
                        sincos_poly(th, &sn, &cs);
                        float len = fmaf(rr, dist - dmin, dmin);
                        ex = fmaf(cs, len, owx);
                        ey = fmaf(sn, len, owy);
                    } else {
                        ex = owx + dmin;
                        ey = owy + 0.0f;
                    }
                    clamp_to_exemplar(&ex, &ey, P.ex.w, P.ex.h);
                    i++;
                    dist *= factor;
                    // an exact repeat of the previous candidate has its energy
                    // and is rejected by the strict "<"
                    if (__float_as_uint(ex) == lastx && __float_as_uint(ey) == lasty) continue;
                    lastx = __float_as_uint(ex);
                    lasty = __float_as_uint(ey);
                    have = true;
                    break;
                }
                float cx, cy, ct, csu, csv;
                if (have) {
                    cx = ex; cy = ey; ct = screen_to_exemplar_angle(P, x, y, ex, ey, 0);
                    csu = sc.x; csv = sc.y;
                } else if (avg_pending) {
                    cx = avgx; cy = avgy; ct = avgt; csu = 1.f; csv = 1.f;
                    avg_pending = false;
                } else {
                    more = false;
                    break;
                }
                bool ok = !((double)ex_texel_dt(ex_mode<HW>(P.ex), (int)cx, (int)cy, 0) > (double)P.distTransCull * 1.25);
                if (ok && !P.transparencyOk) {
                    float ea = ex_sample_out_alpha(ex_mode<HW>(P.ex), cx, cy, 0);
                    ok = !(ea < kAlphaThreshold && ia > kAlphaThreshold);
                }
                if (!ok) {
                    if (kBigResidual < best) {
                        best = kBigResidual;
                        owx = cx; owy = cy; owt = ct; wkind = have ? 1 : 2;
                    }
                    continue;
                }
                if (P.counters) count_eval(P, x, y, px.temporal, false);
                lane_start<R>(P, q, cx, cy, ct, csu, csv, 0, best, &e);
                cur_avg = !have;
                cur_t = ct;
                act = true;
                break;
            }
        }
        if (!__any_sync(kFull, act)) break;
        const bool fast = __all_sync(kFull, !act || e.fast);
        const bool fastp = TM ? __all_sync(kFull, !act || !q.temporal || q.prev_fast) : true;
        if (act) {
            float r;
            if (lane_step_uni<R, TM, HW>(P, T, TT, q, e, fast, fastp, &r)) {
                if (r < best) {
                    best = r;
                    owx = e.cx; owy = e.cy; owt = cur_t; wkind = cur_avg ? 2 : 1;
                }
                act = false;
            }
        }
    }
    if (!own) return;
    const Patch off = load_patch(P.off, k);
    Patch ow = off;
    if (wkind == 1) ow = make_patch(owx, owy, owt, 0.0f, 0, sc.x, sc.y);
    else if (wkind == 2) ow = make_patch(owx, owy, owt, 1.f, 0, 1.f, 1.f);
    const bool take = best < cached;
    if (P.inc.on) P.inc.chg[k] = (take && !same_record(ow, off)) ? 1 : 0;
    if (take) store_patch(work, k, ow);
    else if (write_all) store_patch(work, k, off);
}

// updateResidualCache_kernel, texSynth_kernel.cu:661-693, inside a tracked
// propagate/scatter loop.  The residual is the reference-order weighted sum
// of per-tap values; each pixel keeps those values (P.inc.taps).  A tap's
// value changes only when the pixel's own record changed (all taps) or the
// record of the pixel under the tap changed (its canvas), so only those taps
// are recomputed and the sum is then taken again over the stored values:
// the same operations on the same values, so the same bits.  With `fill`
// every tap of every pixel is computed (the loop's first residual).
template <int R, int TM, int HW>
__global__ void __launch_bounds__(kTileThreads, 2) kt_residual_inc(const Params P, const __grid_constant__ TileMaps M,
                                                                        float* out) {
    constexpr int TW = TileSmem<R, TM>::TW, N = TileSmem<R, TM>::N, K = (2 * R + 1) * (2 * R + 1);
    __shared__ TileSmem<R, TM> T;
    __shared__ PixShared S;
    __shared__ float4 CA[kTileThreads];  // own record: x, y, sv, layer bits | fast << 30
    __shared__ float4 CB[kTileThreads];  // its basis
    __shared__ uint16_t list[kTileThreads * K];  // pid << 7 | tap
    __shared__ uint8_t C[N];
    __shared__ int count;
    const int pid = threadIdx.x + threadIdx.y * kTileW;
    const size_t plane = (size_t)P.W * P.H;
    const int x0 = blockIdx.x * kTileW - R, y0 = blockIdx.y * kTileH - R;
    if (!P.inc.fill) {
        for (int q = pid; q < N; q += kTileThreads) {
            int gx = clampi(x0 + q % TW, 0, P.lw - 1);
            int gy = clampi(y0 + q / TW, 0, P.lh - 1);
            C[q] = P.inc.chg[(size_t)gy * P.W + gx];
        }
    }
    if (pid == 0) count = 0;
    __syncthreads();
    // tap mask of this pixel (bit t: recompute tap t) and the pass stamps
    const int x = blockIdx.x * kTileW + threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
    const bool in = x < P.lw && y < P.lh;
    const size_t k = (size_t)y * P.W + x;
    const int c0 = threadIdx.y * TW + threadIdx.x;  // window corner in C
    uint64_t m0 = 0, m1 = 0;                        // taps 0..63, 64..80
    bool own = P.inc.fill != 0;
    if (in && !P.inc.fill) {
        own = C[c0 + R * TW + R] != 0;
#pragma unroll
        for (int t = 0; t < K; t++) {
            const int i = t / (2 * R + 1), j = t % (2 * R + 1);  // column-major (reference order)
            if (C[c0 + j * TW + i]) {
                if (t < 64) m0 |= 1ull << t; else m1 |= 1ull << (t - 64);
            }
        }
        if (own) P.inc.last[k] = P.inc.pi;
        if (m0 | m1) P.inc.win[k] = P.inc.pi;
    }
    const bool need = in && (own || (m0 | m1));
    if (!__syncthreads_or(need)) return;
    PixT px;
    bool abort;
    stage_tile<R, TM>(P, M, T, &px, &abort);  // (synchronises the block)
    if (abort) return;
    bool mine = false;
    int nt = 0;
    if (need) {
        if (image_culled(P, x, y)) {
            out[k] = 0.0f;
        } else {
            mine = true;
            const LanePix q = lane_pix<R>(P, px);
            put_pix<R>(S, pid, q);
            const Patch o = load_patch(P.off, k);
            LaneEval e;
            lane_start<R>(P, q, o.x, o.y, o.theta, o.su, o.sv, o.layer, kNoBest, &e);
            CA[pid] = make_float4(e.cx, e.cy, e.sv, __int_as_float(e.layer | (e.fast ? 1 << 30 : 0)));
            CB[pid] = make_float4(e.b0.x, e.b0.y, e.b1.x, e.b1.y);
            if (own) {  // every tap t < K
                m0 = K >= 64 ? ~0ull : (1ull << K) - 1ull;
                m1 = K > 64 ? (1ull << (K - 64)) - 1ull : 0ull;
            }
            // only taps inside the level rectangle enter the sum
#pragma unroll
            for (int t = 0; t < K; t++) {
                const int i = t / (2 * R + 1) - R, j = t % (2 * R + 1) - R;
                const bool valid = (i >= q.imin) && (i <= q.imax) && (j >= q.jmin) && (j <= q.jmax);
                if (!valid) {
                    if (t < 64) m0 &= ~(1ull << t); else m1 &= ~(1ull << (t - 64));
                }
            }
            nt = __popcll(m0) + __popcll(m1);
            if (P.counters && own) count_eval(P, x, y, px.temporal, false);
        }
    }
    {
        // queue this pixel's nt taps
        const unsigned lane = lane_id();
        int incl = nt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(kFull, incl, o);
            if ((int)lane >= o) incl += v;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        int base = 0;
        if (lane == 31 && total > 0) base = atomicAdd(&count, total);
        base = __shfl_sync(kFull, base, 31);
        int w = base + incl - nt;
        for (int t = 0; t < K; t++) {
            const bool b = t < 64 ? (m0 >> t) & 1 : (m1 >> (t - 64)) & 1;
            if (mine && b && w < kTileThreads * K) list[w++] = (uint16_t)((pid << 7) | t);
        }
    }
    __syncthreads();
    // every lane takes every 256th queued tap
    const int n = count;
#pragma unroll 1
    for (int b = 0; b < n; b += kTileThreads) {
        const int it = b + pid;
        bool act = it < n;
        LanePix q;
        LaneEval e;
        int t = 0, op = 0;
        if (act) {
            const int v = list[it];
            op = v >> 7;
            t = v & 127;
        }
        act = act && t < K && op < kTileThreads;  // (every queued entry satisfies this)
        if (act) {
            q = get_pix<R, TM>(P, S, op);
            const float4 a = CA[op], bb = CB[op];
            const int lb = __float_as_int(a.w);
            e.cx = a.x; e.cy = a.y; e.sv = a.z;
            e.layer = lb & ~(1 << 30);
            e.fast = (lb >> 30) & 1;
            e.b0 = make_float2(bb.x, bb.y);
            e.b1 = make_float2(bb.z, bb.w);
        }
        const bool fast = __all_sync(kFull, !act || e.fast);
        const bool fastp = TM ? __all_sync(kFull, !act || !q.temporal || q.prev_fast) : true;
        if (act) {
            const int i = t / (2 * R + 1) - R, j = t % (2 * R + 1) - R;
            const float v = tap_value<R, TM, HW>(P, T, q, e, i, j, fast, fastp);
            P.inc.taps[(size_t)t * plane + (size_t)q.y * P.W + q.x] = v;
        }
    }
    if (P.counters) count_taps(P, (unsigned)nt, px.temporal);
    __syncthreads();
    // the residual: the stored values summed in the reference's order
    if (mine) {
        const LanePix q = get_pix<R, TM>(P, S, pid);
        float sum = q.sum0;
#pragma unroll 1
        for (int i = -R; i <= R; i++) {
            const float gi = P.gauss[i + R];
            const bool cvalid = (i >= q.imin) && (i <= q.imax);
#pragma unroll
            for (int j = -R; j <= R; j++) {
                const bool valid = cvalid && (j >= q.jmin) && (j <= q.jmax);
                const int t = (i + R) * (2 * R + 1) + (j + R);
                const float v = valid ? P.inc.taps[(size_t)t * plane + k] : 0.0f;
                const float w = gi * P.gauss[j + R];
                sum = valid ? fmaf(v, w, sum) : sum;
            }
        }
        out[k] = (q.sumW < kEpsilon) ? kBigResidual : sum / q.sumW;
    }
}

template <int R>
cudaError_t launch_tiled_r(int kind, int tm, const Params& P, const TileMaps& M, PatchPlanes work, int arg,
                           uint32_t pass_id, float* out, int wide, cudaStream_t s) {
    dim3 b(kTileW, kTileH), bw(kTileW, 2 * kTileH), g((P.lw + kTileW - 1) / kTileW, (P.lh + kTileH - 1) / kTileH);
    // the texture-unit kernels fetch through the exemplar's textures, which
    // must be bound
    if (P.ex.hw && (!P.ex.tbase || !P.ex.tout)) return cudaErrorInvalidValue;
#define PT_TILED_DISPATCH(TMV, HWV)                                                                   \
    if (kind == 0 && wide) kt_propagate_q<R, TMV, HWV, 2><<<g, bw, 0, s>>>(P, M, work, arg);          \
    else if (kind == 0) kt_propagate_q<R, TMV, HWV, 1><<<g, b, 0, s>>>(P, M, work, arg);             \
    else if (kind == 1) kt_scatter_q<R, TMV, HWV><<<g, b, 0, s>>>(P, M, work, arg, pass_id);         \
    else if (P.inc.on || P.inc.fill) kt_residual_inc<R, TMV, HWV><<<g, b, 0, s>>>(P, M, out);        \
    else kt_residual<R, TMV, HWV><<<g, b, 0, s>>>(P, M, out);
    if (P.ex.hw) {
        if (tm == TM_NONE) { PT_TILED_DISPATCH(TM_NONE, 1) }
        else if (tm == TM_FWD) { PT_TILED_DISPATCH(TM_FWD, 1) }
        else { PT_TILED_DISPATCH(TM_BWD, 1) }
    } else {
        if (tm == TM_NONE) { PT_TILED_DISPATCH(TM_NONE, 0) }
        else if (tm == TM_FWD) { PT_TILED_DISPATCH(TM_FWD, 0) }
        else { PT_TILED_DISPATCH(TM_BWD, 0) }
    }
#undef PT_TILED_DISPATCH
    return cudaGetLastError();
}

}  // namespace ptk
