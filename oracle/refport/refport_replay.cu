// refport_replay.cu -- host driver of the reference-kernel port: the
// reference's own TexSynth host wrappers and kernels
// (src/PaintTweenCUDA/texSynth_kernel.cu, convolution.cu, advectedBuffers.cpp,
// compiled unchanged), driven through a small C interface with the same step
// surface as the CPU oracle, so that tests and the benchmark can run the
// reference's synthesis on the GPU on the same inputs as this library.
//
// Test and baseline infrastructure only: nothing in the product links it.
//
// What the reference's Qt/OpenEXR host code did around the kernels is done
// here instead:
//  - WorkingBuffers::initialize (workingBuffers.cpp:48-94) with the image and
//    style sizes passed to rp_create instead of read from DataAccess;
//  - ImagePyramid uploads (TexSynth::uploadImage_*, texSynth_kernel.cu:
//    2143-2253) of one level held in a one-level pyramid object;
//  - WorkingBuffers::loadOffsets / loadResidual / getOutput
//    (workingBuffers.cpp:125-207) as copies to and from caller memory (the
//    caller applies the half-precision rounding of the residual file);
//  - checkCUDAError (cudaHostUtil.cpp:46-66) records the first error instead
//    of exiting the process.
#include <cstdio>
#include <cstring>
#include <string>

#include "texSynth_kernel.h"
#include "convolution.h"
#include "cudaHostUtil.h"
#include "cudaImagePyramid.h"

#include "painttween.h"

// ---- error recording (replaces checkCUDAError's exit) -------------------------

static std::string g_error;
static int g_error_count = 0;

void refport_record_error(const char* where, cudaError_t e) {
    if (e == cudaSuccess) return;
    if (g_error_count++ == 0) g_error = std::string(where) + ": " + cudaGetErrorString(e);
}

void checkCUDAError(const char* msg) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) refport_record_error(msg, e);
}
void checkCUDAError(const char* msg, const char* name) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::string w = std::string(msg) + " " + name;
        refport_record_error(w.c_str(), e);
    }
}

// ---- the pieces of WorkingBuffers and ImagePyramid that live in Qt-bound files

static int g_image_w = 0, g_image_h = 0, g_style_w = 0, g_style_h = 0, g_num_styles = 1;

void WorkingBuffers::initialize() {
    int styleHeight = g_style_h * g_num_styles;
    if (_is_initialized && g_image_w == _image_width && g_image_h == _image_height && g_style_w == _style_width &&
        styleHeight == _style_height)
        return;
    offsets.initialize(g_image_w, g_image_h);
    residualCache.initialize(g_image_w, g_image_h);
    canvasOutputCache.initialize(g_image_w, g_image_h);
    canvasVelFCache.initialize(g_image_w, g_image_h);
    canvasVelBCache.initialize(g_image_w, g_image_h);
    distTransCache.initialize(g_image_w, g_image_h);
    ribbonField.initialize(g_image_w, g_image_h);
    advectedF.initialize(g_image_w, g_image_h);
    advectedB.initialize(g_image_w, g_image_h);
    tempOutput.initialize(g_image_w, g_image_h);
    offsetsHistogram.initialize(g_style_w, styleHeight);
    _is_initialized = true;
    _style_width = g_style_w;
    _style_height = styleHeight;
    _image_width = g_image_w;
    _image_height = g_image_h;
    _current_level = 0;
}

void WorkingBuffers::clear() {
    if (!_is_initialized) return;
    offsets.clear();
    residualCache.clear();
    canvasOutputCache.clear();
    canvasVelFCache.clear();
    canvasVelBCache.clear();
    distTransCache.clear();
    ribbonField.clear();
    offsetsHistogram.clear();
    tempOutput.clear();
    tempOutputHistogram.clear();
    advectedF.clear();
    advectedB.clear();
    _is_initialized = false;
}

void WorkingBuffers::resetAdvectedBuffers() {
    advectedF.reset();
    advectedB.reset();
}

template <class T>
void ImagePyramid<T>::clear() {
    _storage.clear();
    _baseWidth = _baseHeight = 0;
    _initialized = false;
}

// one level of caller memory as the level-0 image of a pyramid
template <class T>
class OneLevelPyramid : public ImagePyramid<T> {
public:
    OneLevelPyramid(const void* data, int w, int h) {
        QVector<T> level(w * h);
        std::memcpy(level.data(), data, sizeof(T) * (size_t)w * h);
        this->_storage.append(level);
        this->_baseWidth = w;
        this->_baseHeight = h;
        this->_initialized = true;
    }
};

// ---- the C interface ---------------------------------------------------------

static WorkingBuffers* g_buffers = nullptr;
static int g_flip_parity = 0;  // TexSynth's current anim buffer (file-scope in texSynth_kernel.cu)

static TsParameters to_ts(const pt_params* p) {
    TsParameters t;
    std::memset(&t, 0, sizeof t);
    t.residualWindowSize = p->residualWindowSize;
    t.coherenceWeight = p->coherenceWeight;
    t.distTransWeight = p->distTransWeight;
    t.lumShiftWeight = p->lumShiftWeight;
    t.lumShiftEnable = p->lumShiftEnable != 0;
    t.inputAnalogyWeight = p->inputAnalogyWeight;
    t.canvasOutputWeight = p->canvasOutputWeight;
    t.numStyles = p->numStyles;
    for (int i = 0; i < NUM_MAX_STYLES; i++) {
        t.offsetsHistogramSlope[i] = p->offsetsHistogramSlope[i];
        t.offsetsHistogramThreshold[i] = p->offsetsHistogramThreshold[i];
    }
    t.maxDistortion = p->maxDistortion;
    t.alphaWeight = p->alphaWeight;
    t.transparencyOk = p->transparencyOk != 0;
    t.styleObjIdWeight = p->styleObjIdWeight;
    t.orientationEnabled = p->orientationEnabled != 0;
    t.colorspace = p->colorspace;
    t.coherenceRatioRange = p->coherenceRatioRange;
    t.coherenceAngleRange = p->coherenceAngleRange;
    t.levels = p->levels;
    t.scatterSamplesCount = p->scatterSamplesCount;
    t.advectionJitter = p->advectionJitter;
    t.timeDerivativeInputWeight = p->timeDerivativeInputWeight;
    t.timeDerivativeOutputWeight = p->timeDerivativeOutputWeight;
    t.temporalCoherenceWeight = p->temporalCoherenceWeight;
    t.hysteresisWeight = p->hysteresisWeight;
    t.interpolateKeyFrame = p->interpolateKeyFrame != 0;
    t.useGuide = p->useGuide != 0;
    t.currentInterpolationIndex = p->currentInterpolationIndex;
    t.numFrames = p->numFrames;
    t.numKeyFrames = p->numKeyFrames;
    t.firstKeyIndex = p->firstKeyIndex;
    t.lastKeyIndex = p->lastKeyIndex;
    t.distTransCull = p->distTransCull;
    t.residualWindowScaleU = p->residualWindowScaleU;
    t.residualWindowScaleV = p->residualWindowScaleV;
    t.direction = (PassDirection)p->direction;
    return t;
}

template <class T>
static void to_host(CudaImageBufferHost<T>& b, int level, void* out) {
    QVector<T> v;
    b.copyToHost(v, level);
    std::memcpy(out, v.data(), sizeof(T) * (size_t)v.size());
}
template <class T>
static void from_host(CudaImageBufferHost<T>& b, int level, const void* in) {
    QVector<T> v(b.width(level) * b.height(level));
    std::memcpy(v.data(), in, sizeof(T) * (size_t)v.size());
    b.copyFromHost(v, level);
}

extern "C" {

int rp_error_count() { return g_error_count; }
const char* rp_last_error() { return g_error.c_str(); }

// The reference runs one synthesis per process (file-scope texture pyramids
// and constant parameters); so does the port: rp_create replaces any
// previous state.
int rp_create(int W, int H, int SW, int SH, int NS) {
    g_error.clear();
    g_error_count = 0;
    if (g_buffers) {
        g_buffers->clear();
        delete g_buffers;
        g_buffers = nullptr;
    }
    CudaImagePyramidHost::releaseAll();
    if (g_flip_parity) {  // a new run starts on anim buffer 0
        TexSynth::flipAnimBuffers();
        g_flip_parity = 0;
    }
    g_image_w = W;
    g_image_h = H;
    g_style_w = SW;
    g_style_h = SH;
    g_num_styles = NS;
    g_buffers = new WorkingBuffers();
    g_buffers->initialize();
    TexSynth::initialize_images(W, H);
    refport_record_error("bindEmptyInstances", CudaImagePyramidHost::bindEmptyInstances());
    checkCUDAError("rp_create");
    return g_error_count;
}

void rp_destroy() {
    if (g_buffers) {
        g_buffers->clear();
        delete g_buffers;
        g_buffers = nullptr;
    }
    CudaImagePyramidHost::releaseAll();
}

// TexSynth::setup (and the WorkingBuffers copy of the parameters that
// syncBuffers reads)
void rp_set_params(const pt_params* p) {
    TsParameters t = to_ts(p);
    g_buffers->setParams(t);
    TexSynth::setup(t);
}

void rp_init_exemplars(int w, int h, int n) { TexSynth::initialize_exemplars(w, h, n); }
void rp_init_cumulative_fields(int w, int h, int n) { TexSynth::initialize_cumulativeFields(w, h, n); }

// kind 0 = Color4, 1 = float, 2 = float2, 3 = int
void rp_upload(int kind, int layer, const void* data, int w, int h, int style) {
    TsImageLayer L = (TsImageLayer)layer;
    switch (kind) {
    case 0: { OneLevelPyramid<Color4> p(data, w, h); TexSynth::uploadImage_Color4(0, L, p, style); break; }
    case 1: { OneLevelPyramid<float> p(data, w, h); TexSynth::uploadImage_float(0, L, p, style); break; }
    case 2: { OneLevelPyramid<float2> p(data, w, h); TexSynth::uploadImage_float2(0, L, p); break; }
    case 3: { OneLevelPyramid<int> p(data, w, h); TexSynth::uploadImage_int(0, L, p, style); break; }
    default: refport_record_error("rp_upload", cudaErrorInvalidValue);
    }
}

void rp_flip() {
    TexSynth::flipAnimBuffers();
    g_flip_parity ^= 1;
}
void rp_reset_advected() { g_buffers->resetAdvectedBuffers(); }
void rp_copy_base_to_working() { g_buffers->offsets.copyBaseToWorking(); }
// synthesisProcessor.cpp:987-988 (FBMO's merge pass)
void rp_copy_base_to_advected(int forwards) {
    AdvectedBuffersHost& a = forwards ? g_buffers->advectedF : g_buffers->advectedB;
    g_buffers->offsets.base().copyTo(a.offsets());
    g_buffers->residualCache.base().copyTo(a.residual());
}

void rp_randomize(int level) { TexSynth::randomizeOffsets(g_buffers, level); }
void rp_propagate(int level, int jump, int key) { TexSynth::propagate(g_buffers, level, jump, key); }
void rp_scatter(int level, int key) { TexSynth::scatter(g_buffers, level, key); }
void rp_upsample(int level) { TexSynth::upsample(g_buffers, level); }
void rp_advect(int level, int ts, int fwd, int flags) { TexSynth::advectOffsets(g_buffers, level, ts, fwd != 0, flags); }
void rp_merge_randomly(int level, int fwd, float w, int force) {
    TexSynth::mergeRandomly(g_buffers, level, fwd != 0, w, force != 0);
}
void rp_merge_using_residual(int level, int fwd) { TexSynth::mergeUsingResidual(g_buffers, level, fwd != 0); }
void rp_merge_advected(int level, int fallback) { TexSynth::mergeAdvectedBuffers(g_buffers, level, fallback); }
void rp_update_residual(int level) { TexSynth::updateResidualCache(g_buffers, level); }
void rp_sync(int level, int flags) { TexSynth::syncBuffers(g_buffers, level, flags); }
void rp_accumulate_ribbon(int level, int fwd, int ts, int overwrite) {
    TexSynth::accumulateRibbonField(g_buffers, level, fwd != 0, ts, overwrite != 0);
}
void rp_frame_to_key_ribbon(int level, int look_fwd) {
    TexSynth::offsetsFromFrameToKeyRibbon(g_buffers, level, look_fwd != 0);
}

void rp_get_offsets(int level, void* out) { to_host(g_buffers->offsets.base(), level, out); }
void rp_get_residual(int level, void* out) { to_host(g_buffers->residualCache.base(), level, out); }
void rp_get_output(int level, void* out) { to_host(g_buffers->canvasOutputCache, level, out); }
void rp_get_ribbon(int level, void* out) { to_host(g_buffers->ribbonField.base(), level, out); }
void rp_get_advected_output(int fwd, int level, void* out) {
    to_host(fwd ? g_buffers->advectedF.output() : g_buffers->advectedB.output(), level, out);
}
void rp_load_offsets(int level, const void* in) { from_host(g_buffers->offsets.base(), level, in); }
void rp_load_residual(int level, const void* in) { from_host(g_buffers->residualCache.base(), level, in); }
void rp_load_ribbon(int level, const void* in) { from_host(g_buffers->ribbonField.base(), level, in); }
void rp_load_canvas(int level, const void* in) { from_host(g_buffers->canvasOutputCache, level, in); }

// every launch in the TexSynth wrappers is followed by a device synchronise,
// so this only reports
int rp_synchronize() {
    checkCUDAError("rp_synchronize");
    return g_error_count;
}

}  // extern "C"
