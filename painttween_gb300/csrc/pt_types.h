// pt_types.h -- plain data structures shared by host and device code.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>

#include "painttween.h"

namespace ptk {

constexpr int kMaxRadius = 15;  // taps per axis <= 31
constexpr int kTileW = 32;      // pixel tile of the tiled kernels
constexpr int kTileH = 8;

// Offset field in three planes (SoA of the 36-byte PatchXF):
//   A = (x, y, theta, layer as int bits), B = (hysteresis, scaleU, scaleV,
//   lumShift.y), C = lumShift.a.  Full-resolution, pitch = image width.
struct Patch {
    float x, y, theta, hyst;
    int layer;
    float su, sv, lumy, luma;
};

struct PatchPlanes {
    float4* A;
    float4* B;
    float* C;
};

// One exemplar pyramid level: ns styles of w x h texels, base and output
// colours in two planes (16-byte texels), so that the gathers of neighbouring
// pixels, which sample neighbouring texels, share cache lines.
struct ExView {
    const float4* base;
    const float4* out;
    const float4* bo;  // the same texels interleaved: bo[2t] = base[t], bo[2t + 1] = out[t] (32-byte records)
    const float* orient;
    const float* dt;
    const int* ids;
    int w, h, ns;
    // PT_FILTER_TEXTURE: the linearly filtered inputs are read with the
    // texture unit's arithmetic (hw); base and output are also bound as
    // layered textures (linear filter, clamp, unnormalised coordinates) that
    // the tiled kernels fetch through
    int hw;
    cudaTextureObject_t tbase, tout;
};

// A 2-D array of one pyramid level.  Image-side "layered" inputs (colour,
// DT, velocities) are addressed with clamp at the level-0 size and read zero
// outside the level rectangle, like the reference's full-resolution layered
// textures holding the level in the top-left corner; the other inputs clamp
// at their own size.
template <class T>
struct Arr {
    const T* p;
    int w, h;
};

struct ImgView {
    Arr<float4> base[2];
    Arr<float> dt[2];
    Arr<float2> velf[2];
    Arr<float2> velb[2];
    Arr<float> orient;
    Arr<float2> scale;
    Arr<int> ids;
    Arr<float4> rnd;
    Arr<float4> f2k[2];  // frame-to-key ribbons of the level, [0] = backward, [1] = forward
    int cur;
};

struct AdvView {
    PatchPlanes off;
    float4* base;
    float4* out;
    float* res;
    int* ts;
};

// Keyframe interpolation inputs: the key-to-key cumulative fields
// [0] = backward, [1] = forward (n key layers of w x h RGBA texels, RibbonP
// packed as (time_step, y, x, layer), linear filter).
struct KeyView {
    const float4* cumul[2];
    int w, h, n;
    int hw;  // PT_FILTER_TEXTURE
};
// RibbonP (types.h:111-126) in the ribbon field buffers; layer < 0 = invalid
struct Ribbon {
    float x, y;
    int time_step, layer;
};

// Change tracking across the passes of one propagate/scatter loop.  A pass
// sets chg[k] = 1 where it changed pixel k's offset record (any of its 36
// bytes); the sync after it stamps last[k] (the last pass that changed k's
// record) and win[k] (the last pass that changed a record inside k's patch
// window).  Pass indices grow monotonically over the context's life, so a
// stamp from an earlier loop reads as "unchanged since before this loop".
struct IncView {
    uint8_t* chg;
    int* last;
    int* win;
    int on;    // this pass is tracked (chg written, stamps updated)
    int pi;    // its index
    int prev;  // index of the previous pass of this loop with the same candidates, INT_MIN if none
    // per-tap values of every pixel's residual, (2r+1)^2 planes at level-0
    // pitch, tap t = (i + r) * (2r + 1) + (j + r); `fill` recomputes all
    float* taps;
    int fill;
};

struct Params {
    int W, H;            // level-0 image size == buffer pitch / height
    int level, lw, lh;   // level and its size
    int r;               // patch radius
    float gauss[2 * kMaxRadius + 1];
    float scaleWU, scaleWV;
    float alphaWeight, inputAnalogyWeight, canvasOutputWeight;
    float distTransWeight, styleObjIdWeight, coherenceWeight;
    float coherenceRatioRange, coherenceAngleRange;
    float tdIn, tdOut, tc;
    float maxDistortion, hysteresisWeight;
    float histThreshold[PT_MAX_STYLES], histSlope[PT_MAX_STYLES];
    float jitter;
    int numStyles;
    int transparencyOk, orientationEnabled, lumShiftEnable;
    int distTransCull;
    int direction;
    int scatterSamples;
    int firstKey, lastKey;     // first and last keyframe layer (keyframe interpolation)
    int colorspace;            // 1: the energy compares Lab colours
    int rngMode;
    uint32_t rngSeed;
    int hwFilter;              // PT_FILTER_TEXTURE: texture-unit arithmetic for the linearly filtered inputs
    int histW, histH;          // histogram level size (style w, style h * ns) >> level
    int histPitch, histRows;   // histogram buffer size at level 0
    const float* hist;
    ExView ex;
    ImgView img;
    PatchPlanes off;           // offsets base
    const float* res;          // residual base
    const float4* canvas;
    AdvView adv[2];            // [0] = forward, [1] = backward
    unsigned long long* counters;  // profiling: energy evaluations, taps, temporal taps (null = off)
    int earlyExit;             // every per-tap term is >= 0 (all weights >= 0): candidates may stop early
    // the taps of a patch window of radius <= 4 by descending weight (ties in
    // the reference's order), tap t = (i + r) * (2r + 1) + (j + r)
    uint8_t tapOrder[81];
    IncView inc;
};

struct ConvKernel {
    int r;
    float w[2 * kMaxRadius + 1];
};

// Tensor maps of the pixel-side planes a tiled kernel stages (each a float4
// plane read as a FLOAT32 tensor of 4 * level width x level height, boxes of
// one tile with its halo): the input colour, the canvas and, for temporal
// passes, the advected colours and the advected records' B plane.  With
// `on`, blocks whose tile and halo lie inside the level rectangle stage them
// with tensor copies; the others (and every block without `on`) load them
// with the clamp rules.  `err` is set when a block's wait for its copies
// runs out.
struct TileMaps {
    CUtensorMap base, canvas, pbase, pout, prec;
    int* err;
    int on;
};

}  // namespace ptk
