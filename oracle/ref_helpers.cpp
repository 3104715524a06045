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
#include "texSynth_interface.h"
#include "texSynth_kernel.h"

#include <cstddef>

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

// TsParameters (texSynth_interface.h): every field the C ABI's pt_params
// mirrors, in pt_params' order, with its offset and size in the reference's
// struct.  A name missing from TsParameters fails this file's compilation.
#define PT_REF_FIELD(f) {#f, (long)offsetof(TsParameters, f), (long)sizeof(((TsParameters*)0)->f)}
static const struct {
    const char* name;
    long offset, size;
} kParamFields[] = {
    PT_REF_FIELD(residualWindowSize), PT_REF_FIELD(coherenceWeight), PT_REF_FIELD(distTransWeight),
    PT_REF_FIELD(lumShiftWeight), PT_REF_FIELD(lumShiftEnable), PT_REF_FIELD(inputAnalogyWeight),
    PT_REF_FIELD(canvasOutputWeight), PT_REF_FIELD(numStyles), PT_REF_FIELD(offsetsHistogramSlope),
    PT_REF_FIELD(offsetsHistogramThreshold), PT_REF_FIELD(maxDistortion), PT_REF_FIELD(alphaWeight),
    PT_REF_FIELD(transparencyOk), PT_REF_FIELD(styleObjIdWeight), PT_REF_FIELD(orientationEnabled),
    PT_REF_FIELD(colorspace), PT_REF_FIELD(coherenceRatioRange), PT_REF_FIELD(coherenceAngleRange),
    PT_REF_FIELD(levels), PT_REF_FIELD(scatterSamplesCount), PT_REF_FIELD(advectionJitter),
    PT_REF_FIELD(timeDerivativeInputWeight), PT_REF_FIELD(timeDerivativeOutputWeight),
    PT_REF_FIELD(temporalCoherenceWeight), PT_REF_FIELD(hysteresisWeight), PT_REF_FIELD(interpolateKeyFrame),
    PT_REF_FIELD(useGuide), PT_REF_FIELD(currentInterpolationIndex), PT_REF_FIELD(numFrames),
    PT_REF_FIELD(numKeyFrames), PT_REF_FIELD(firstKeyIndex), PT_REF_FIELD(lastKeyIndex),
    PT_REF_FIELD(distTransCull), PT_REF_FIELD(residualWindowScaleU), PT_REF_FIELD(residualWindowScaleV),
    PT_REF_FIELD(direction),
};
#undef PT_REF_FIELD

// TsImageLayer values under the names the C ABI gives them (PT_LAYER_<name>)
#define PT_REF_LAYER(n) {#n, (long)TS_LAYER_##n}
static const struct {
    const char* name;
    long value;
} kLayers[] = {
    PT_REF_LAYER(EXEMPLAR_BASE), PT_REF_LAYER(EXEMPLAR_OUTPUT), PT_REF_LAYER(EXEMPLAR_ORIENTATION),
    PT_REF_LAYER(EXEMPLAR_DIST_TRANS), PT_REF_LAYER(EXEMPLAR_OBJECT_IDS), PT_REF_LAYER(INPUT_COLOR),
    PT_REF_LAYER(INPUT_ORIENTATION), PT_REF_LAYER(INPUT_DIST_TRANS), PT_REF_LAYER(INPUT_SCALE),
    PT_REF_LAYER(INPUT_ID), PT_REF_LAYER(INPUT_SURF_ID), PT_REF_LAYER(INPUT_VEL_B), PT_REF_LAYER(INPUT_VEL_F),
    PT_REF_LAYER(INPUT_VEL_B_PREVIOUS), PT_REF_LAYER(INPUT_VEL_F_PREVIOUS), PT_REF_LAYER(GUIDE_B),
    PT_REF_LAYER(GUIDE_F), PT_REF_LAYER(CUMUL_FIELD_B), PT_REF_LAYER(CUMUL_FIELD_F),
    PT_REF_LAYER(FRAME_TO_KEY_RIBBON_B), PT_REF_LAYER(FRAME_TO_KEY_RIBBON_F), PT_REF_LAYER(RANDOM),
};
#undef PT_REF_LAYER

// i-th entry of the tables above; each returns the table's length
int ref_param_field(int i, const char** name, long* offset, long* size) {
    const int n = (int)(sizeof(kParamFields) / sizeof(kParamFields[0]));
    if (i >= 0 && i < n) {
        *name = kParamFields[i].name;
        *offset = kParamFields[i].offset;
        *size = kParamFields[i].size;
    }
    return n;
}
int ref_layer(int i, const char** name, long* value) {
    const int n = (int)(sizeof(kLayers) / sizeof(kLayers[0]));
    if (i >= 0 && i < n) {
        *name = kLayers[i].name;
        *value = kLayers[i].value;
    }
    return n;
}
// TexSynth's syncBuffers / merge and advect flags (texSynth_kernel.h):
// DONT_COPY_OFFSETS, DONT_UPDATE_RESIDUAL, MERGE_FALLBACK_RANDOM,
// MERGE_FALLBACK_LAST_PASS, ADVECT_IGNORE_RANDOM, ADVECT_DO_NOT_CHECK_PREVIOUS,
// ADVECT_CHECK_FRAME_TO_KEY, ADVECT_UPDATE_RESIDUAL
void ref_flags(long* out8) {
    out8[0] = TexSynth::DONT_COPY_OFFSETS;
    out8[1] = TexSynth::DONT_UPDATE_RESIDUAL;
    out8[2] = TexSynth::MERGE_FALLBACK_RANDOM;
    out8[3] = TexSynth::MERGE_FALLBACK_LAST_PASS;
    out8[4] = TexSynth::ADVECT_IGNORE_RANDOM;
    out8[5] = TexSynth::ADVECT_DO_NOT_CHECK_PREVIOUS;
    out8[6] = TexSynth::ADVECT_CHECK_FRAME_TO_KEY;
    out8[7] = TexSynth::ADVECT_UPDATE_RESIDUAL;
}

// PatchXF's and RibbonP's layouts (types.h): sizeof, then the offsets of
// x, y, theta, hysteresis, layer, scaleU, scaleV, luminanceShift.y,
// luminanceShift.a; then sizeof(RibbonP) and the offsets of x, y,
// time_step, layer
void ref_record_layouts(long* out15) {
    out15[0] = (long)sizeof(PatchXF);
    out15[1] = (long)offsetof(PatchXF, x);
    out15[2] = (long)offsetof(PatchXF, y);
    out15[3] = (long)offsetof(PatchXF, theta);
    out15[4] = (long)offsetof(PatchXF, hysteresis);
    out15[5] = (long)offsetof(PatchXF, layer);
    out15[6] = (long)offsetof(PatchXF, scaleU);
    out15[7] = (long)offsetof(PatchXF, scaleV);
    out15[8] = (long)(offsetof(PatchXF, luminanceShift) + offsetof(Luminance, y));
    out15[9] = (long)(offsetof(PatchXF, luminanceShift) + offsetof(Luminance, a));
    out15[10] = (long)sizeof(RibbonP);
    out15[11] = (long)offsetof(RibbonP, x);
    out15[12] = (long)offsetof(RibbonP, y);
    out15[13] = (long)offsetof(RibbonP, time_step);
    out15[14] = (long)offsetof(RibbonP, layer);
}

// NUM_MAX_STYLES, sizeof(TsParameters), and PassDirection's FORWARD,
// BACKWARD, BIDIRECTIONAL
void ref_param_constants(long* out5) {
    out5[0] = NUM_MAX_STYLES;
    out5[1] = (long)sizeof(TsParameters);
    out5[2] = FORWARD;
    out5[3] = BACKWARD;
    out5[4] = BIDIRECTIONAL;
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
