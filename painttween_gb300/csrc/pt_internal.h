// pt_internal.h -- launchers shared by the kernel and host translation units.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "pt_types.h"

namespace pt {

// Gaussian weights of radius r, sigma = r / 3, as allocateGaussianKernel
// (src/PaintTweenCUDA/convolution.cu:37-60) forms them: the exponential in
// float, and with `normalize` the division by sqrt(2*pi)*sigma in double
// (M_PI promotes the expression) rounded back to float.  w has 2r+1 entries.
inline void gaussian_weights(int r, bool normalize, float* w) {
    float sigma = (float)r / 3.0f, s2 = sigma * sigma;
    for (int i = 0; i <= r; i++) {
        float v = expf(-(float)(i * i) / (2.f * s2));
        if (normalize) v = (float)((double)v / (std::sqrt(2.0 * M_PI) * (double)sigma));
        w[r + i] = v;
        w[r - i] = v;
    }
}

using ptk::Arr;
using ptk::ConvKernel;
using ptk::ExView;
using ptk::Params;
using ptk::PatchPlanes;
using ptk::TileMaps;

using ptk::KeyView;
using ptk::Ribbon;

cudaError_t launch_propagate(const Params& P, PatchPlanes work, int jump, int key, cudaStream_t s);
cudaError_t launch_scatter(const Params& P, PatchPlanes work, int write_all, uint32_t pass_id, int key,
                           cudaStream_t s);
// keyframe interpolation (pt_keys.cu)
cudaError_t launch_propagate_keys(const Params& P, PatchPlanes work, int jump, int key, const KeyView& K,
                                  cudaStream_t s);
cudaError_t launch_scatter_keys(const Params& P, PatchPlanes work, int write_all, int key, const KeyView& K,
                                cudaStream_t s);
cudaError_t launch_accumulate_ribbon(const Params& P, int forwards, Ribbon* dest, const Ribbon* src, int time_step,
                                     int overwrite, cudaStream_t s);
cudaError_t launch_ribbon_output(const Params& P, const Ribbon* rib, const float4* canvas, float4* out,
                                 cudaStream_t s);
cudaError_t launch_frame_to_key(const Params& P, PatchPlanes work, int look_forwards, const KeyView& K,
                                cudaStream_t s);
cudaError_t launch_merge_advected(const Params& P, int fallback, PatchPlanes work, cudaStream_t s);
cudaError_t launch_fill_ribbons(Ribbon* r, size_t n, int layer, cudaStream_t s);
cudaError_t launch_ribbon_pack(const Ribbon* src, int w, int h, float4* dst, cudaStream_t s);
cudaError_t launch_ribbon_down(const float4* src, int sw, float4* dst, int w, int h, cudaStream_t s);
cudaError_t launch_residual(const Params& P, float* out, cudaStream_t s);
cudaError_t launch_canvas(const Params& P, float4* canvas, cudaStream_t s);
cudaError_t launch_random_offsets(const Params& P, PatchPlanes work, cudaStream_t s);
cudaError_t launch_upsample(const Params& P, PatchPlanes work, PatchPlanes border_src, int copy_border,
                            float* res_out, cudaStream_t s);
cudaError_t launch_advect(const Params& P, int d, int forwards, int time_step, int flags, cudaStream_t s);
cudaError_t launch_merge_random(const Params& P, int d, int forwards, float weight, int force, PatchPlanes work,
                                cudaStream_t s);
cudaError_t launch_merge_residual(const Params& P, int d, PatchPlanes work, cudaStream_t s);
cudaError_t launch_conv(const float* src, float* dst, int w, int h, int pitch, int rows, const ConvKernel& kw,
                        cudaStream_t s);
cudaError_t launch_copy_patch(const Params& P, PatchPlanes dst, PatchPlanes src, cudaStream_t s);
cudaError_t launch_copy_float(const Params& P, float* dst, const float* src, cudaStream_t s);
cudaError_t launch_unpack_patch(const Params& P, const pt_patchxf* src, PatchPlanes dst, cudaStream_t s);
cudaError_t launch_pack_patch(const Params& P, PatchPlanes src, pt_patchxf* dst, cudaStream_t s);
cudaError_t launch_load_residual(const Params& P, const float* src, float* dst, cudaStream_t s);
cudaError_t launch_gather_level(const Params& P, const float* src, int ch, float* dst, cudaStream_t s);
cudaError_t launch_down_avg(const float* src, int w, int h, int ch, int vel, float* dst, cudaStream_t s);
cudaError_t launch_down_vote(const int* src, int w, int h, int* dst, cudaStream_t s);
cudaError_t launch_tensor_angle(const float* t3, int n, float* out, cudaStream_t s);
cudaError_t launch_random_level_keys(int w, int h, int mx, int my, int transparencyOk, int orientationEnabled,
                                     Arr<float4> img, Arr<float> iorient, ExView ex, float4* out,
                                     const uint32_t* state31, int nk, int first_key, cudaStream_t s);
cudaError_t launch_random_level(int mode, int w, int h, int mx, int my, int transparencyOk, int orientationEnabled,
                                Arr<float4> img, Arr<float> iorient, ExView ex, float4* out,
                                const uint32_t* states, uint32_t seed, cudaStream_t s);
cudaError_t launch_any_transparent(const float4* out, size_t n, int* flag, cudaStream_t s);
cudaError_t launch_interleave_texels(const float4* base, const float4* out, float4* bo, size_t n, cudaStream_t s);

// tiled patch-distance kernels for patch radius 2, 3, 4 (pt_tiled_r*.cu):
// kind 0 = propagate (arg = jump), 1 = scatter (arg = write_all),
// 2 = residual (into out); tm 0 = no temporal terms, 1 = forward, 2 = backward;
// M: the tensor maps of the staged planes (M.on = 0: staged by plain loads);
// wide: propagate with two warps per tile row (same results)
cudaError_t launch_tiled_2(int kind, int tm, const Params& P, const TileMaps& M, PatchPlanes work, int arg,
                           uint32_t pass_id, float* out, int wide, cudaStream_t s);
cudaError_t launch_tiled_3(int kind, int tm, const Params& P, const TileMaps& M, PatchPlanes work, int arg,
                           uint32_t pass_id, float* out, int wide, cudaStream_t s);
cudaError_t launch_tiled_4(int kind, int tm, const Params& P, const TileMaps& M, PatchPlanes work, int arg,
                           uint32_t pass_id, float* out, int wide, cudaStream_t s);
}  // namespace pt
