// refport_compat.h -- force-included into every translation unit of the
// reference-kernel port (test and baseline infrastructure only).
//
// cudaThreadSynchronize was removed in CUDA 13; cudaDeviceSynchronize is its
// documented replacement with the same effect.
#pragma once
#include <cuda_runtime.h>
#define cudaThreadSynchronize cudaDeviceSynchronize
