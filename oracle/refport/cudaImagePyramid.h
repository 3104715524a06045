// cudaImagePyramid.h -- replacement of the reference's header of the same
// name (src/PaintTweenCUDA/cudaImagePyramid.h:56-108) for the reference-kernel
// port, which is test and baseline infrastructure only.
//
// The reference binds each image pyramid to a file-scope texture<>
// reference.  Texture references were removed in CUDA 13, so this header
// keeps the reference's class interface and macro names but binds each
// pyramid to a texture object instead: the macros declare a __constant__
// handle beside the host object, the host object creates the texture object
// with the filter mode the reference asks for (clamp addressing,
// unnormalised coordinates, element reads, as cudaImagePyramid.cpp:96-106
// sets on the reference) and writes the handle there, and the fetch macros
// read through it.  Coordinates are passed exactly as the reference's fetch
// macros form them ((X) + 0.5, converted to float), so every fetch goes
// through the same texture-unit filtering as in the reference.
#ifndef REFPORT_CUDA_IMAGE_PYRAMID_H
#define REFPORT_CUDA_IMAGE_PYRAMID_H

#include <cuda_runtime.h>

#include <vector>

// a texture handle typed by its texel and its dimensionality, so that a 2D
// fetch of a layered pyramid (or the converse) does not compile, as with the
// reference's typed texture references
template <class T, int Layered>
struct RefportTex {
    cudaTextureObject_t obj;
};

template <class T>
__device__ __forceinline__ T refport_fetch(const RefportTex<T, 0>& t, float x, float y) {
    return tex2D<T>(t.obj, x, y);
}
template <class T>
__device__ __forceinline__ T refport_fetch_layer(const RefportTex<T, 1>& t, float x, float y, int layer) {
    return tex2DLayered<T>(t.obj, x, y, layer);
}

class CudaImagePyramidHost {
public:
    CudaImagePyramidHost(int textureType, int typeSize, const char* name, cudaChannelFormatDesc desc,
                         const void* handle_symbol);
    ~CudaImagePyramidHost();

    void initialize(int width, int height, cudaTextureFilterMode filter_mode, int depth = 1);

    void clear();
    static void clearAllInstances();

    void copyFromHost(const void* source);
    void copyFromHost(int width, int height, const void* source, int layer);
    void copyFromHost(int width, int height, cudaTextureFilterMode filter_mode, const void* source);
    void copyTo(CudaImagePyramidHost& target);

    bool isInitialized() const { return _storage != nullptr; }

    int width() { return _baseWidth; }
    int height() { return _baseHeight; }

    // port additions: bind every pyramid that holds no array to a 1x1 zero
    // texture (a fetch through a handle that was never created is undefined),
    // and release every texture and array
    static cudaError_t bindEmptyInstances();
    static void releaseAll();

protected:
    cudaError_t bindTexture();
    cudaError_t bindEmpty();
    void destroyTexture();

    cudaArray_t _storage = nullptr;
    cudaArray_t _empty = nullptr;
    cudaTextureObject_t _tex = 0;
    int _typeSize;
    int _textureType;
    int _baseWidth = 0, _baseHeight = 0, _numLayers = 0;
    cudaTextureFilterMode _filterMode = cudaFilterModePoint;
    cudaChannelFormatDesc _desc;
    const void* _symbol;
    const char* _name;

    static std::vector<CudaImagePyramidHost*>& instances();
};

#define CUDA_IMAGE_PYRAMID(TYPE, NAME)                                            \
    __constant__ RefportTex<TYPE, 0> NAME##_TEXTURE_PYRAMID;                     \
    CudaImagePyramidHost NAME(cudaTextureType2D, sizeof(TYPE), #NAME, cudaCreateChannelDesc<TYPE>(), \
                              &NAME##_TEXTURE_PYRAMID);
#define PYRAMID_FETCH(NAME, X, Y) refport_fetch(NAME##_TEXTURE_PYRAMID, (X) + 0.5, (Y) + 0.5)

#define CUDA_IMAGE_PYRAMID_LAYERED(TYPE, NAME)                                    \
    __constant__ RefportTex<TYPE, 1> NAME##_TEXTURE_PYRAMID;                     \
    CudaImagePyramidHost NAME(cudaTextureType2DLayered, sizeof(TYPE), #NAME, cudaCreateChannelDesc<TYPE>(), \
                              &NAME##_TEXTURE_PYRAMID);

#define PYRAMID_FETCH_LAYER(NAME, X, Y, LAYER) \
    refport_fetch_layer(NAME##_TEXTURE_PYRAMID, (X) + 0.5, (Y) + 0.5, (LAYER))

#endif
