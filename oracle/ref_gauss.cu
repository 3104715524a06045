// ref_gauss.cu -- the reference's allocateGaussianKernel
// (src/PaintTweenCUDA/convolution.cu:37-60), compiled from its own source for
// the host, so that a CPU test can compare the Gaussian weights of the oracle
// and of the library with the reference's bit for bit.
//
// Test infrastructure only; built by oracle/build.py into oracle/_ref/ where
// the reference tree is present, never linked into the product library.
// allocateGaussianKernel ends by copying its host array to a __constant__
// symbol; here that copy is redirected into a host buffer, so the function
// runs without a GPU.  No kernel of convolution.cu is launched.
#include <cuda_runtime.h>

#include <cstring>

static float g_captured[64];
static int g_captured_n = 0;

static cudaError_t capture_weights(const float* src, size_t bytes) {
    g_captured_n = (int)(bytes / sizeof(float));
    if (g_captured_n > 64) g_captured_n = 64;
    std::memcpy(g_captured, src, (size_t)g_captured_n * sizeof(float));
    return cudaSuccess;
}

#define cudaMemcpyToSymbol(symbol, src, bytes) capture_weights((const float*)(src), (bytes))
#include "convolution.cu"
#undef cudaMemcpyToSymbol

void checkCUDAError(const char*) {}
void checkCUDAError(const char*, const char*) {}

// Weights of radius r (2r+1 floats into out) as the reference computes them;
// returns the number written.
extern "C" int ref_gaussian_kernel(int radius, int normalize, float* out) {
    g_captured_n = 0;
    allocateGaussianKernel(nullptr, radius, normalize != 0);
    std::memcpy(out, g_captured, (size_t)g_captured_n * sizeof(float));
    return g_captured_n;
}
