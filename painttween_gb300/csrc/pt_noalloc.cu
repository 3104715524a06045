// pt_noalloc.cu -- an allocation-free separable Gaussian blur.
//
// Some callers cannot allocate device memory at the time they need this
// operation: a host application (a compositing or render plugin host, for
// instance) that owns the GPU's memory through its own pool and forbids
// cudaMalloc/cudaFree inside its per-frame callbacks, or a process whose
// device memory is entirely held by another framework's caching allocator.
// pt_convolve_separable needs a context, whose scratch buffer for the
// row-pass result is allocated on demand.  This entry point instead keeps
// that intermediate image in a fixed array in the library's own device
// memory, so a call allocates nothing: the caller passes its own input and
// output buffers and a stream.
#include <cmath>
#include <mutex>

#include <cuda_runtime.h>

#include "painttween.h"
#include "pt_internal.h"

// The intermediate (row-convolved) image.  It is part of the library's
// module image: every GPU that loads the library holds these
// PT_NOALLOC_MAX_PIXELS floats (4 MiB) until the process exits.
static __device__ __align__(256) float g_noalloc_scratch[PT_NOALLOC_MAX_PIXELS];

namespace {

// Device address of g_noalloc_scratch per device ordinal, looked up once per
// device.  In host code the array's name is only a host-side stand-in, so a
// kernel must be given this address, never the name.
constexpr int kMaxDevices = 64;
float* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

cudaError_t scratch_address(int device, float** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        float* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);  // with `device` current
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = ptr;
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace

pt_status pt_convolve_separable_noalloc(const float* src_dev, float* dst_dev, int w, int h, int pitch, int radius,
                                        void* stream) {
    if (!src_dev || !dst_dev || w < 1 || h < 1 || pitch < w || radius < 1 || radius > ptk::kMaxRadius)
        return PT_ERR_INVALID;
    if ((size_t)pitch * (size_t)h > (size_t)PT_NOALLOC_MAX_PIXELS) return PT_ERR_INVALID;  // beyond the fixed array
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return PT_ERR_CUDA;
    float* scratch = nullptr;
    if (scratch_address(device, &scratch) != cudaSuccess) return PT_ERR_CUDA;
    // normalised Gaussian, sigma = radius / 3 (convolution.cu:37-60)
    ptk::ConvKernel k;
    k.r = radius;
    float sigma = (float)radius / 3.0f, s2 = sigma * sigma;
    for (int i = 0; i <= radius; i++) {
        float wgt = expf(-(float)(i * i) / (2.f * s2));
        wgt = wgt / (sqrtf(2.f * (float)M_PI) * sigma);
        k.w[radius + i] = wgt;
        k.w[radius - i] = wgt;
    }
    // every scratch element the column pass reads is written by the row pass
    // first, so nothing has to be cleared between calls
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (pt::launch_conv(src_dev, scratch, w, h, pitch, 1, k, s) != cudaSuccess) return PT_ERR_CUDA;
    if (pt::launch_conv(scratch, dst_dev, w, h, pitch, 0, k, s) != cudaSuccess) return PT_ERR_CUDA;
    return PT_OK;
}
