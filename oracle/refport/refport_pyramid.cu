// refport_pyramid.cu -- CudaImagePyramidHost over texture objects, for the
// reference-kernel port (test and baseline infrastructure only).
//
// Same behaviour as the reference's src/PaintTweenCUDA/cudaImagePyramid.cpp
// (initialize keeps an existing array of the same size and filter; layered
// uploads write one layer's top-left rectangle; 2D uploads re-create the
// array at the upload's size; copyTo duplicates the whole array), with the
// texture reference replaced by a texture object whose handle is written to
// the pyramid's __constant__ slot.  Two choices of the port: a new array is
// filled with zeros (the reference leaves cudaMalloc3DArray's contents
// unspecified), and a pyramid without an array is bound to a 1x1 zero
// texture so that no kernel fetches through a handle that was never made.
#include "cudaImagePyramid.h"

#include <cstdio>
#include <cstring>
#include <vector>

void refport_record_error(const char* where, cudaError_t e);

#define RP_CHECK(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) {                         \
            refport_record_error(_name, e_);             \
            return e_;                                   \
        }                                                \
    } while (0)

std::vector<CudaImagePyramidHost*>& CudaImagePyramidHost::instances() {
    static std::vector<CudaImagePyramidHost*> v;
    return v;
}

CudaImagePyramidHost::CudaImagePyramidHost(int textureType, int typeSize, const char* name,
                                           cudaChannelFormatDesc desc, const void* handle_symbol)
    : _typeSize(typeSize), _textureType(textureType), _desc(desc), _symbol(handle_symbol), _name(name) {
    instances().push_back(this);
}

// no CUDA calls at process exit: releaseAll() frees everything explicitly
CudaImagePyramidHost::~CudaImagePyramidHost() {}

void CudaImagePyramidHost::destroyTexture() {
    if (_tex) cudaDestroyTextureObject(_tex);
    _tex = 0;
}

static cudaTextureObject_t make_texture(cudaArray_t arr, cudaTextureFilterMode filter, cudaError_t* err) {
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof td);
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = filter;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t t = 0;
    *err = cudaCreateTextureObject(&t, &rd, &td, nullptr);
    return t;
}

cudaError_t CudaImagePyramidHost::bindTexture() {
    destroyTexture();
    cudaError_t e;
    _tex = make_texture(_storage, _filterMode, &e);
    RP_CHECK(e);
    RP_CHECK(cudaMemcpyToSymbol(_symbol, &_tex, sizeof(_tex)));
    return cudaSuccess;
}

cudaError_t CudaImagePyramidHost::bindEmpty() {
    destroyTexture();
    if (!_empty) {
        if (_textureType == cudaTextureType2DLayered)
            RP_CHECK(cudaMalloc3DArray(&_empty, &_desc, make_cudaExtent(1, 1, 1), cudaArrayLayered));
        else
            RP_CHECK(cudaMallocArray(&_empty, &_desc, 1, 1));
        std::vector<char> zero(_typeSize, 0);
        cudaMemcpy3DParms p;
        std::memset(&p, 0, sizeof p);
        p.srcPtr = make_cudaPitchedPtr(zero.data(), _typeSize, 1, 1);
        p.dstArray = _empty;
        p.extent = make_cudaExtent(1, 1, 1);
        p.kind = cudaMemcpyHostToDevice;
        RP_CHECK(cudaMemcpy3D(&p));
    }
    cudaError_t e;
    _tex = make_texture(_empty, cudaFilterModePoint, &e);
    RP_CHECK(e);
    RP_CHECK(cudaMemcpyToSymbol(_symbol, &_tex, sizeof(_tex)));
    return cudaSuccess;
}

void CudaImagePyramidHost::initialize(int width, int height, cudaTextureFilterMode filter_mode, int depth) {
    if (isInitialized() && width == _baseWidth && height == _baseHeight && filter_mode == _filterMode) return;
    clear();
    _baseWidth = width;
    _baseHeight = height;
    _filterMode = filter_mode;
    _numLayers = depth;
    cudaError_t e;
    if (_textureType == cudaTextureType2DLayered)
        e = cudaMalloc3DArray(&_storage, &_desc, make_cudaExtent(width, height, depth), cudaArrayLayered);
    else
        e = cudaMallocArray(&_storage, &_desc, width, height);
    if (e != cudaSuccess) {
        refport_record_error(_name, e);
        _storage = nullptr;
        return;
    }
    int layers = _textureType == cudaTextureType2DLayered ? depth : 1;
    std::vector<char> zero((size_t)width * height * layers * _typeSize, 0);
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof p);
    p.srcPtr = make_cudaPitchedPtr(zero.data(), (size_t)width * _typeSize, width, height);
    p.dstArray = _storage;
    p.extent = make_cudaExtent(width, height, _textureType == cudaTextureType2DLayered ? depth : 0);
    if (_textureType != cudaTextureType2DLayered) p.extent.depth = 1;
    p.kind = cudaMemcpyHostToDevice;
    e = cudaMemcpy3D(&p);
    if (e != cudaSuccess) refport_record_error(_name, e);
    bindTexture();
}

void CudaImagePyramidHost::clear() {
    if (!isInitialized()) return;
    destroyTexture();
    cudaFreeArray(_storage);
    _storage = nullptr;
    _baseWidth = _baseHeight = 0;
    bindEmpty();
}

void CudaImagePyramidHost::clearAllInstances() {
    for (CudaImagePyramidHost* p : instances()) p->clear();
}

void CudaImagePyramidHost::copyFromHost(const void* source) {
    if (!isInitialized() || _textureType != cudaTextureType2D) {
        refport_record_error(_name, cudaErrorInvalidValue);
        return;
    }
    size_t row = (size_t)_baseWidth * _typeSize;
    cudaError_t e = cudaMemcpy2DToArray(_storage, 0, 0, source, row, row, _baseHeight, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) refport_record_error(_name, e);
}

void CudaImagePyramidHost::copyFromHost(int width, int height, const void* source, int layer) {
    if (!isInitialized() || _textureType != cudaTextureType2DLayered || layer < 0 || layer >= _numLayers ||
        width > _baseWidth || height > _baseHeight) {
        refport_record_error(_name, cudaErrorInvalidValue);
        return;
    }
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof p);
    p.srcPtr = make_cudaPitchedPtr((void*)source, (size_t)width * _typeSize, width, height);
    p.srcPos = make_cudaPos(0, 0, 0);
    p.dstArray = _storage;
    p.dstPos = make_cudaPos(0, 0, layer);
    p.extent = make_cudaExtent(width, height, 1);
    p.kind = cudaMemcpyHostToDevice;
    cudaError_t e = cudaMemcpy3D(&p);
    if (e != cudaSuccess) refport_record_error(_name, e);
}

void CudaImagePyramidHost::copyFromHost(int width, int height, cudaTextureFilterMode filter_mode, const void* source) {
    initialize(width, height, filter_mode);
    copyFromHost(source);
}

void CudaImagePyramidHost::copyTo(CudaImagePyramidHost& target) {
    if (target._typeSize != _typeSize || target._textureType != _textureType || !isInitialized()) {
        refport_record_error(_name, cudaErrorInvalidValue);
        return;
    }
    target.initialize(_baseWidth, _baseHeight, _filterMode, _numLayers);
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof p);
    p.srcArray = _storage;
    p.dstArray = target._storage;
    p.extent = make_cudaExtent(_baseWidth, _baseHeight, _textureType == cudaTextureType2DLayered ? _numLayers : 1);
    p.kind = cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpy3D(&p);
    if (e != cudaSuccess) refport_record_error(_name, e);
}

cudaError_t CudaImagePyramidHost::bindEmptyInstances() {
    for (CudaImagePyramidHost* p : instances())
        if (!p->isInitialized() && !p->_tex) {
            cudaError_t e = p->bindEmpty();
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

void CudaImagePyramidHost::releaseAll() {
    for (CudaImagePyramidHost* p : instances()) {
        p->destroyTexture();
        if (p->_storage) cudaFreeArray(p->_storage);
        if (p->_empty) cudaFreeArray(p->_empty);
        p->_storage = p->_empty = nullptr;
        p->_baseWidth = p->_baseHeight = 0;
    }
}
