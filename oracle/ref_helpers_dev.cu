// ref_helpers_dev.cu -- the reference's own device helpers
// (src/PaintTweenCUDA/texSynth_util.h) compiled by nvcc with its default
// arithmetic (--fmad=true) into oracle/_ref/ref_helpers.cubin, so that the
// GPU tests can check the oracle's restatement against them on the device.
//
// Test infrastructure only; built by oracle/build.py where the reference
// tree is present, never linked into the product library.  One thread per
// element; every access is guarded by i < n.
#include "texSynth_util.h"

extern "C" __global__ void ref_helpers_batch(const float4* a, const float4* b, const float* alpha,
                                             const float* angle, const float* su, const float* sv,
                                             const float* ij, const float* e, float* ssd_alpha,
                                             float* ssd_plain, float4* basis, float2* coord,
                                             float4* lab, float2* clamped, const float4* packed,
                                             float4* ribbon, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Color4 ca(a[i].x, a[i].y, a[i].z, a[i].w), cb(b[i].x, b[i].y, b[i].z, b[i].w);
    ssd_alpha[i] = sumSquaredDiff(ca, cb, alpha[i]);
    ssd_plain[i] = sumSquaredDiff(ca, cb);
    float2 b0, b1;
    screenToExemplarBasis(angle[i], su[i], sv[i], &b0, &b1);
    basis[i] = make_float4(b0.x, b0.y, b1.x, b1.y);
    float ox, oy;
    calculateNewExemplarCoord(ij[2 * i], ij[2 * i + 1], e[2 * i], e[2 * i + 1], b0, b1, &ox, &oy);
    coord[i] = make_float2(ox, oy);
    Color4 l = RGBtoLAB(ca);
    lab[i] = make_float4(l.r, l.g, l.b, l.a);
    float cx = e[2 * i] - 40.0f, cy = e[2 * i + 1] - 40.0f;
    clampToExemplar(&cx, &cy, 64, 48);
    clamped[i] = make_float2(cx, cy);
    RibbonP r = toRibbonP(packed[i]);
    ribbon[i] = make_float4(r.x, r.y, (float)r.time_step, (float)r.layer);
}
