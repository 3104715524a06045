// pt_measure.cu -- ceilings for the roofline of the patch-distance kernels.
//
// The kernels gather 32-byte exemplar records (both colours of a texel) from
// an exemplar level that stays resident in L2, so their ceiling is the rate
// of such gathers, not the HBM copy rate.  This measures it on the running
// GPU: 32-byte records from an L2-resident buffer, gathered at random by
// every lane (the worst case) or at random per warp with the warp's lanes on
// consecutive records (the coherent case the kernels approach when
// neighbouring pixels take neighbouring exemplar positions).
#include <cuda_runtime.h>

#include <cstdint>

#include "painttween.h"

namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// every lane reads `iters` records; rec holds (mask + 1) records of 32 bytes
__global__ void k_gather32(const float4* __restrict__ rec, uint32_t mask, int iters, int coherent, float* sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.0f;
    for (int k = 0; k < iters; k++) {
        uint32_t r = coherent ? (mix32((tid >> 5) * 977u + (uint32_t)k) + (threadIdx.x & 31u)) & mask
                              : mix32(tid * 7919u + (uint32_t)k) & mask;
        const float4 a = __ldg(rec + 2 * (size_t)r), b = __ldg(rec + 2 * (size_t)r + 1);
        acc += a.x + a.y + a.z + a.w + b.x + b.y + b.z + b.w;
    }
    if (acc == 1234.5f) sink[tid] = acc;  // keeps the loads; never true for the zeroed buffer
}

}  // namespace

pt_status pt_measure_gather(int device, int coherent, double* out_gbs) {
    if (!out_gbs) return PT_ERR_INVALID;
    *out_gbs = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return PT_ERR_CUDA;
    const uint32_t nrec = 1u << 20;  // 32 MiB of 32-byte records: L2-resident
    float4* rec = nullptr;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    pt_status st = PT_ERR_CUDA;
    int sms = 0;
    const int threads = 256, iters = 256;
    int blocks = 0;
    float ms = 0.0f;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) goto done;
    blocks = sms * 8;
    if (cudaMalloc(&rec, (size_t)nrec * 32) != cudaSuccess) goto done;
    if (cudaMalloc(&sink, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) goto done;
    if (cudaMemset(rec, 0, (size_t)nrec * 32) != cudaSuccess) goto done;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto done;
    for (int w = 0; w < 3; w++) k_gather32<<<blocks, threads>>>(rec, nrec - 1, iters, coherent, sink);
    if (cudaEventRecord(e0) != cudaSuccess) goto done;
    for (int rep = 0; rep < 10; rep++) k_gather32<<<blocks, threads>>>(rec, nrec - 1, iters, coherent, sink);
    if (cudaEventRecord(e1) != cudaSuccess) goto done;
    if (cudaEventSynchronize(e1) != cudaSuccess) goto done;
    if (cudaGetLastError() != cudaSuccess) goto done;
    if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f) goto done;
    *out_gbs = 10.0 * blocks * threads * (double)iters * 32.0 / (ms * 1e6);
    st = PT_OK;
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rec) cudaFree(rec);
    if (sink) cudaFree(sink);
    return st;
}
