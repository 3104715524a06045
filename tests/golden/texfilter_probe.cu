// texfilter_probe.cu -- records the texture unit's bilinear fetches on the
// GPU it runs on, for the fixture tests/golden/texfilter_gb300.npz that pins
// the oracle's emulation of that filtering (make_texfilter.py builds and runs
// this program; see there).
//
// Each case is a float texture (1, 2 or 4 channels; a layered cudaArray, or
// pitched linear memory) with clamp addressing, linear filtering and
// unnormalised coordinates, and a list of (x, y, layer) coordinates passed to
// tex2D / tex2DLayered as given.  Output per case: a file
// <dir>/<name>.bin holding int32 W, H, L, C, n, then the texels (float32,
// W*H*L*C), the coordinates (float32, 3n) and the fetched values (float32,
// C*n).  Every kernel thread reads q[i] and writes out[i] for i < n only.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#define CK(x)                                                                             \
    do {                                                                                  \
        cudaError_t e_ = (x);                                                             \
        if (e_ != cudaSuccess) {                                                          \
            fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_));    \
            exit(1);                                                                      \
        }                                                                                 \
    } while (0)

template <class T> __device__ void put(float* o, T v);
template <> __device__ void put<float>(float* o, float v) { o[0] = v; }
template <> __device__ void put<float2>(float* o, float2 v) { o[0] = v.x; o[1] = v.y; }
template <> __device__ void put<float4>(float* o, float4 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }

template <class T>
__global__ void fetch_layered(cudaTextureObject_t t, const float* q, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) put<T>(out + (size_t)i * (sizeof(T) / 4), tex2DLayered<T>(t, q[3 * i], q[3 * i + 1], (int)q[3 * i + 2]));
}
template <class T>
__global__ void fetch_pitch(cudaTextureObject_t t, const float* q, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) put<T>(out + (size_t)i * (sizeof(T) / 4), tex2D<T>(t, q[3 * i], q[3 * i + 1]));
}

template <class T>
static void run(const std::string& dir, const char* name, const std::vector<float>& texels, int W, int H, int L,
                const std::vector<float>& q, bool pitch) {
    const int C = sizeof(T) / 4;
    const int n = (int)(q.size() / 3);
    cudaChannelFormatDesc d = cudaCreateChannelDesc<T>();
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof rd);
    cudaArray_t arr = nullptr;
    void* lin = nullptr;
    if (!pitch) {
        CK(cudaMalloc3DArray(&arr, &d, make_cudaExtent(W, H, L), cudaArrayLayered));
        cudaMemcpy3DParms p;
        memset(&p, 0, sizeof p);
        p.srcPtr = make_cudaPitchedPtr((void*)texels.data(), (size_t)W * sizeof(T), W, H);
        p.dstArray = arr;
        p.extent = make_cudaExtent(W, H, L);
        p.kind = cudaMemcpyHostToDevice;
        CK(cudaMemcpy3D(&p));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
    } else {
        size_t pitchb = 0;
        CK(cudaMallocPitch(&lin, &pitchb, (size_t)W * sizeof(T), H));
        CK(cudaMemcpy2D(lin, pitchb, texels.data(), (size_t)W * sizeof(T), (size_t)W * sizeof(T), H,
                        cudaMemcpyHostToDevice));
        rd.resType = cudaResourceTypePitch2D;
        rd.res.pitch2D.devPtr = lin;
        rd.res.pitch2D.desc = d;
        rd.res.pitch2D.width = W;
        rd.res.pitch2D.height = H;
        rd.res.pitch2D.pitchInBytes = pitchb;
    }
    cudaTextureDesc td;
    memset(&td, 0, sizeof td);
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t obj;
    CK(cudaCreateTextureObject(&obj, &rd, &td, nullptr));
    float *dq = nullptr, *dout = nullptr;
    CK(cudaMalloc(&dq, q.size() * sizeof(float)));
    CK(cudaMalloc(&dout, (size_t)n * C * sizeof(float)));
    CK(cudaMemcpy(dq, q.data(), q.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (pitch)
        fetch_pitch<T><<<(n + 255) / 256, 256>>>(obj, dq, n, dout);
    else
        fetch_layered<T><<<(n + 255) / 256, 256>>>(obj, dq, n, dout);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    std::vector<float> out((size_t)n * C);
    CK(cudaMemcpy(out.data(), dout, out.size() * sizeof(float), cudaMemcpyDeviceToHost));
    std::string fn = dir + "/" + name + ".bin";
    FILE* f = fopen(fn.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", fn.c_str()); exit(1); }
    int hdr[5] = {W, H, L, C, n};
    fwrite(hdr, 4, 5, f);
    fwrite(texels.data(), sizeof(float), (size_t)W * H * L * C, f);
    fwrite(q.data(), sizeof(float), q.size(), f);
    fwrite(out.data(), sizeof(float), out.size(), f);
    fclose(f);
    CK(cudaDestroyTextureObject(obj));
    if (arr) CK(cudaFreeArray(arr));
    if (lin) CK(cudaFree(lin));
    CK(cudaFree(dq));
    CK(cudaFree(dout));
    printf("%s: %d fetches\n", fn.c_str(), n);
}

int main(int argc, char** argv) {
    std::string dir = argc > 1 ? argv[1] : ".";
    CK(cudaSetDevice(0));
    std::mt19937 rng(20261204);
    std::uniform_real_distribution<float> U(0.f, 1.f);
    auto coord = [&](std::vector<float>& q, float x, float y, int layer) {
        q.push_back(x); q.push_back(y); q.push_back((float)layer);
    };
    {   // unit texels: the four weights, along each axis and over the square
        int W = 8, H = 8;
        std::vector<float> t((size_t)W * H * 4, 0.f);
        t[(3 * W + 3) * 4 + 0] = 1; t[(3 * W + 4) * 4 + 1] = 1; t[(4 * W + 3) * 4 + 2] = 1; t[(4 * W + 4) * 4 + 3] = 1;
        std::vector<float> q;
        for (int k = 0; k < 2048; k++) coord(q, 3.5f + k / 2048.f, 3.5f, 0);
        for (int k = 0; k < 2048; k++) coord(q, 3.5f, 3.5f + k / 2048.f, 0);
        for (int k = 0; k < 8192; k++) coord(q, 3.5f + U(rng), 3.5f + U(rng), 0);
        run<float4>(dir, "weights", t, W, H, 1, q, false);
    }
    {   // uniform texels in [0, 1), four channels, coordinates across and beyond the edges
        int W = 32, H = 32, L = 2;
        std::vector<float> t((size_t)W * H * L * 4);
        for (auto& v : t) v = U(rng);
        std::vector<float> q;
        for (int k = 0; k < 6000; k++) coord(q, U(rng) * 38.f - 3.f, U(rng) * 38.f - 3.f, k & 1);
        run<float4>(dir, "unit4", t, W, H, L, q, false);
    }
    {   // signed values over twelve decades, zeros, signed zeros, subnormals, ties of the fraction
        int W = 32, H = 32, L = 2;
        std::normal_distribution<float> N(0.f, 1.f);
        auto special = [&]() -> float {
            float r = U(rng);
            if (r < 0.20f) return 0.f;
            if (r < 0.25f) return -0.f;
            if (r < 0.32f) return 1.f;
            if (r < 0.40f) return U(rng) * 1e-3f;
            if (r < 0.45f) return U(rng) * 1e-30f;
            if (r < 0.48f) return U(rng) * 1e-39f;
            if (r < 0.55f) return -U(rng);
            return N(rng) * powf(10.f, U(rng) * 12.f - 6.f);
        };
        std::vector<float> t((size_t)W * H * L * 4);
        for (auto& v : t) v = special();
        std::vector<float> q;
        for (int k = 0; k < 6000; k++) coord(q, U(rng) * 36.f - 2.f, U(rng) * 36.f - 2.f, k & 1);
        for (int k = 0; k < 3000; k++) {
            float fx = (floorf(U(rng) * 256.f) + 0.5f) / 256.f, fy = (floorf(U(rng) * 256.f) + 0.5f) / 256.f;
            coord(q, floorf(U(rng) * 30.f) + 0.5f + fx, floorf(U(rng) * 30.f) + 0.5f + fy, k & 1);
        }
        run<float4>(dir, "special4", t, W, H, L, q, false);
        std::vector<float> t1((size_t)W * H * L), t2((size_t)W * H * L * 2);
        for (size_t i = 0; i < t1.size(); i++) t1[i] = t[i * 4];
        for (size_t i = 0; i < t1.size(); i++) { t2[2 * i] = t[i * 4 + 1]; t2[2 * i + 1] = t[i * 4 + 2]; }
        run<float>(dir, "special1", t1, W, H, L, q, false);
        run<float2>(dir, "special2", t2, W, H, L, q, false);
        std::vector<float> q0;
        for (size_t i = 0; i < q.size(); i += 3) coord(q0, q[i], q[i + 1], 0);
        std::vector<float> tl0(t.begin(), t.begin() + (size_t)W * H * 4);
        run<float4>(dir, "special4_pitch", tl0, W, H, 1, q0, true);
    }
    {   // coordinates that are not finite or far outside: NaN, +-inf, +-1e30
        int W = 8, H = 6, L = 2;
        std::vector<float> t((size_t)W * H * L * 4);
        for (auto& v : t) v = U(rng);
        const float odd[] = {NAN, -NAN, INFINITY, -INFINITY, 1e30f, -1e30f, 3.25f, 0.5f, 7.75f, -100.f};
        std::vector<float> q;
        for (float x : odd)
            for (float y : odd) coord(q, x, y, 1);
        run<float4>(dir, "nonfinite4", t, W, H, L, q, false);
    }
    {   // large coordinates: fraction resolution at x near 3000
        int W = 4096, H = 4;
        std::vector<float> t((size_t)W * H, 0.f);
        std::vector<float> q;
        for (int i = 0; i < W * H; i++) t[i] = U(rng);
        for (int k = 0; k < 2048; k++) coord(q, 3000.5f + k / 2048.f, 1.5f + U(rng), 0);
        run<float>(dir, "far1", t, W, H, 1, q, false);
    }
    return 0;
}
