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
#include <cuda_runtime.h>

#include "painttween.h"
#include "pt_internal.h"

// The intermediate (row-convolved) image.  It is part of the library's
// module image: every GPU that loads the library holds these
// PT_NOALLOC_MAX_PIXELS floats (4 MiB) until the process exits.
static __device__ __align__(256) float g_noalloc_scratch[PT_NOALLOC_MAX_PIXELS];

pt_status pt_convolve_separable_noalloc(const float* src_dev, float* dst_dev, int w, int h, int pitch, int radius,
                                        void* stream) {
    if (!src_dev || !dst_dev || w < 1 || h < 1 || pitch < w || radius < 1 || radius > ptk::kMaxRadius)
        return PT_ERR_INVALID;
    if ((size_t)pitch * (size_t)h > (size_t)PT_NOALLOC_MAX_PIXELS) return PT_ERR_INVALID;  // beyond the fixed array
    // An error left pending on this thread by earlier work is not ours to
    // report or to clear: refuse the call and leave it for the caller.
    if (cudaPeekAtLastError() != cudaSuccess) return PT_ERR_CUDA;
    // Device address of the array in the current device's context.  In host
    // code the array's name is only a host-side stand-in, so the kernels are
    // given this address.  It is looked up on every call (cheap once the
    // module is loaded), so it stays valid after the caller resets the device
    // and the module is loaded again.
    float* scratch = nullptr;
    if (cudaGetSymbolAddress((void**)&scratch, g_noalloc_scratch) != cudaSuccess || !scratch) return PT_ERR_CUDA;
    ptk::ConvKernel k;
    k.r = radius;
    pt::gaussian_weights(radius, true, k.w);  // normalised, sigma = radius / 3
    // every scratch element the column pass reads is written by the row pass
    // first, so nothing has to be cleared between calls
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (pt::launch_conv(src_dev, scratch, w, h, pitch, 1, k, s) != cudaSuccess) return PT_ERR_CUDA;
    if (pt::launch_conv(scratch, dst_dev, w, h, pitch, 0, k, s) != cudaSuccess) return PT_ERR_CUDA;
    return PT_OK;
}
