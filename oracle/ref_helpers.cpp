// ref_helpers.cpp -- C entry points over the reference's own device helpers
// (src/PaintTweenCUDA/texSynth_util.h) and image-buffer addressing
// (cudaImageBuffer.h), compiled for the host from the reference tree by
// oracle/build.py into oracle/_ref/libref_helpers.so.
//
// Test infrastructure only: tests/test_ref_helpers.py checks the oracle's
// restatement of these helpers against the reference's code itself.  The
// header's device-only random generator reads threadIdx, which a host build
// does not declare: a zero index stands in (randFloat is not exported).
#include <cstring>

#include <cuda_runtime.h>
static uint3 threadIdx = {0, 0, 0};
#include "texSynth_util.h"
#include "cudaImageBuffer.h"

extern "C" {

void ref_rgb_to_lab(const float* in, float* out) {
    Color4 c = RGBtoLAB(Color4(in[0], in[1], in[2], in[3]));
    out[0] = c.r; out[1] = c.g; out[2] = c.b; out[3] = c.a;
}

void ref_basis(float angle, float su, float sv, float* out) {
    float2 b0, b1;
    screenToExemplarBasis(angle, su, sv, &b0, &b1);
    out[0] = b0.x; out[1] = b0.y; out[2] = b1.x; out[3] = b1.y;
}

void ref_new_coord(float i, float j, float ex, float ey, const float* basis, float* out) {
    calculateNewExemplarCoord(i, j, ex, ey, make_float2(basis[0], basis[1]), make_float2(basis[2], basis[3]),
                              &out[0], &out[1]);
}

void ref_clamp_to_exemplar(float* x, float* y, int w, int h) { clampToExemplar(x, y, w, h); }

float ref_ssd(const float* a, const float* b, float alpha) {
    return sumSquaredDiff(Color4(a[0], a[1], a[2], a[3]), Color4(b[0], b[1], b[2], b[3]), alpha);
}

float ref_ssd_plain(const float* a, const float* b) {
    return sumSquaredDiff(Color4(a[0], a[1], a[2], a[3]), Color4(b[0], b[1], b[2], b[3]));
}

void ref_ribbon_of(const float* c, float* xy, int* ts_layer) {
    RibbonP r = toRibbonP(make_float4(c[0], c[1], c[2], c[3]));
    xy[0] = r.x; xy[1] = r.y; ts_layer[0] = r.time_step; ts_layer[1] = r.layer;
}

// toPatchXF (texSynth_util.h): the random layer's packed texel as a PatchXF,
// copied out as its 36 bytes.
int ref_to_patchxf(const float* c, unsigned char* out36) {
    PatchXF p = toPatchXF(make_float4(c[0], c[1], c[2], c[3]));
    std::memcpy(out36, &p, sizeof(PatchXF) < 36 ? sizeof(PatchXF) : 36);
    return (int)sizeof(PatchXF);
}

// CudaImageBufferDevice::pixelWrap and inBounds (cudaImageBuffer.h) on a
// w x h image whose pixel i holds i: the wrapped pixel's index comes back.
int ref_pixel_wrap(const int* index_image, int w, int h, int x, int y) {
    CudaImageBufferDevice<int> b(const_cast<int*>(index_image), w * (int)sizeof(int), w, h);
    return b.pixelWrap(x, y);
}

int ref_in_bounds(int w, int h, int x, int y, int level, int border) {
    CudaImageBufferDevice<int> b(nullptr, w * (int)sizeof(int), w, h);
    return b.inBounds(x, y, level, border) ? 1 : 0;
}

}  // extern "C"
