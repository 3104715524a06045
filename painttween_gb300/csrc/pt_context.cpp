// pt_context.cpp -- host side of libpainttween_gb300: the context, device
// buffers, the C ABI of include/painttween.h and the per-frame driver.
//
// Buffer model.  As in the reference (src/PaintTweenCUDA/cudaImageBuffer.h,
// workingBuffers.cpp:48-94) the image-size buffers are full resolution and a
// level uses the top-left (W>>L) x (H>>L) rectangle.  The reference keeps a
// base/working pair for the offsets and copies working -> base after every
// Jacobi pass (copyWorkingToBase, :332-334).  Here the pair is two physical
// buffers with a copy-on-write alias: after a sync the logical base and
// working buffers are the same physical buffer, and the next writer of
// "working" takes the other one (writing every level pixel it would otherwise
// have left unchanged).  This removes the per-pass full-buffer copy while
// keeping the reference's observable state.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <climits>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "painttween.h"
#include "pt_internal.h"

using ptk::AdvView;
using ptk::Arr;
using ptk::ConvKernel;
using ptk::ExView;
using ptk::ImgView;
using ptk::Params;
using ptk::PatchPlanes;

namespace {

int level_count(int w, int h) {
    // ImagePyramid level count, imagePyramid.cpp:86
    return (int)std::min(std::floor(std::log2((float)w)), std::floor(std::log2((float)h)));
}

// A layered float4 array (one layer per style) bound to a texture object
// with the reference's sampling state (linear filter, clamp, unnormalised
// coordinates).  Its extent is a capacity: a level of w x h texels occupies
// the corner [0, w) x [0, h), its last column and row repeated once beyond
// (where the capacity allows), and the kernels clamp coordinates to
// [0, w-1] x [0, h-1] before a fetch that may leave the level.  That gives
// the texels and weights of clamp addressing on an array of exactly w x h:
// a clamped coordinate has fraction 0 at the edge, where the array's clamp
// would blend the edge texel with itself, and the texel beyond the edge that
// a fraction-0 fetch still addresses holds the edge's value.  Arrays are
// therefore reused across exemplars of different sizes without cudaFreeArray,
// which would wait for the whole device.
struct TexArray {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    int cw = 0, ch = 0, layers = 0;
    size_t bytes = 0;
};

struct ExLevel {  // one exemplar pyramid level, all styles (base and output planes)
    float4* base = nullptr;
    float4* out = nullptr;
    float4* bo = nullptr;   // base and output interleaved per texel, rebuilt when stale
    bool bo_stale = true;
    // PT_FILTER_TEXTURE: base and output as textures, refreshed when stale
    TexArray ta[2];
    bool tex_stale = true;
    float* orient = nullptr;
    float* dt = nullptr;
    int* ids = nullptr;
    int w = 0, h = 0;
    int transparent = -1;  // -1 unknown, 0/1
};

struct FrameLevel {
    float4* rgba = nullptr;
    float* orient = nullptr;
    float* dt = nullptr;
    int* ids = nullptr;
    float2* velf = nullptr;
    float2* velb = nullptr;
    float2* scale = nullptr;
    int w = 0, h = 0;
};

struct StoreEntry {
    pt_patchxf* offs = nullptr;
    float* res = nullptr;
    float4* canvas = nullptr;
    int w = 0, h = 0;
};

}  // namespace

constexpr int kSpanNone = 1 << 20;  // a level coarser than any image has

struct pt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t budget = 0, allocated = 0;
    std::string err;
    std::map<void*, size_t> allocs;
    std::multimap<size_t, void*> cache;  // freed blocks by size
    size_t cached = 0;
    std::vector<TexArray> tex_free;  // texture arrays not bound to a level (bytes counted in `cached`)

    pt_params params{};
    bool have_params = false;
    float gauss[2 * ptk::kMaxRadius + 1] = {0};
    ConvKernel hist_kernel{};

    int W = 0, H = 0, SW = 0, SH = 0, NS = 0;
    bool initialized = false;

    PatchPlanes off[2]{};
    int base_i = 0, work_i = 0;
    // The two offset buffers hold the same records outside the rectangle of
    // level `off_span` (kSpanNone: everywhere).  Kernels write only inside
    // their level's rectangle, so when a coarser level follows a finer one
    // (the IND scheme's next frame) the buffer that becomes the working one
    // must first be made whole: propagate reads records outside a coarse
    // rectangle, and upsample keeps the working buffer's border.
    int off_span = 0;
    float* res[2] = {nullptr, nullptr};
    int res_i = 0;
    float4* canvas = nullptr;
    float* hist[2] = {nullptr, nullptr};  // [0] base, [1] working
    bool hist_zero = false;                // both histogram buffers hold zeros
    AdvView adv[2]{};

    // storage behind the step-wise uploads
    float4* up_base[2] = {nullptr, nullptr};
    float* up_dt[2] = {nullptr, nullptr};
    float2* up_velf[2] = {nullptr, nullptr};
    float2* up_velb[2] = {nullptr, nullptr};
    bool slot_copy = false;  // driver binds copy into the layered arrays (IND)
    // keyframe interpolation: cumulative fields (B, F), frame-to-key ribbons
    // (B, F) and the ribbon field pair ([0] base, [1] working)
    float4* cumul[2] = {nullptr, nullptr};
    int cf_w = 0, cf_h = 0, cf_n = 0;
    float4* f2k_buf[2] = {nullptr, nullptr};
    ptk::Ribbon* rib[2] = {nullptr, nullptr};
    // keyframe interpolation driver: style i is the key of frame
    // key_frames[i] (DataAccess::keyFrameIndices); key_sub is the run's key
    // subrange (Style::keyFrameSubrange); keyed is set while a run
    // interpolates keys.  keyFramesPreprocess leaves per frame its
    // frame-to-key ribbon pyramid and per key (full index) its key-to-key
    // ribbon pyramid, [0] backward, [1] forward, as RGBA levels.
    std::vector<int> key_frames, key_sub;
    bool keyed = false;
    int run_first = 0, run_last = 0;
    std::map<int, std::vector<float4*>> f2k_pyr[2], k2k_pyr[2];
    float* up_orient = nullptr;
    float2* up_scale = nullptr;
    int* up_ids = nullptr;
    float4* rnd = nullptr;
    ImgView img{};

    ExLevel up_ex;     // exemplar storage of the step-wise API
    ExLevel* ex = nullptr;
    size_t ex_cap = 0;  // texels (w*h*ns) allocated in up_ex

    // staging
    void* stage = nullptr;
    size_t stage_bytes = 0;
    float* conv_scratch = nullptr;
    size_t conv_scratch_elems = 0;
    uint32_t* states = nullptr;
    size_t states_cap = 0;
    int* flag = nullptr;

    // resident working set
    std::vector<ExLevel> style_levels;
    std::vector<int> style_set;
    std::map<int, std::vector<FrameLevel>> frames;
    // ribbon inputs: (frame, time step) -> per level forward and backward
    // velocities over that many frames (getRibbonF/B, nlDataAccess.cpp:
    // 160-205); time step 1 is the frame's own velocities
    std::map<std::pair<int, int>, std::vector<std::pair<float2*, float2*>>> ribbons;
    std::map<std::tuple<int, int, int>, StoreEntry> store;
    // SynthesisFrame::_last_saved_pass: (frame, level) -> last pass saved
    // through saveImages
    std::map<std::pair<int, int>, int> last_saved;
    int out_level = 0, out_pass = 0;  // where the last run's final output was saved

    uint64_t launches = 0;
    uint32_t pass_counter = 0;
    void* cb_stage = nullptr;  // page-locked staging of the animation callback
    size_t cb_stage_bytes = 0;
    bool adv_written[2] = {false, false};  // advected F/B written since the last reset
    bool use_tiled = true;                 // tiled kernels where an instantiation exists

    // change tracking of the driver's propagate/scatter loops
    bool use_incremental = true;
    uint8_t* chg = nullptr;
    int* stamp_last = nullptr;
    int* stamp_win = nullptr;
    int inc_seq = 0;        // index of the last tracked pass
    int inc_on = 0, inc_pi = 0, inc_prev = INT_MIN;
    int inc_fill = 0;       // the next residual computes and stores every tap value
    float* tap_cache = nullptr;  // per-tap residual values, (2r+1)^2 planes
    int tap_cache_k = 0;         // planes allocated

    // measurement
    cudaEvent_t timers[PT_TIMER_SLOTS] = {};
    int profiling = 0;  // PT_PROFILE_* flags
    unsigned long long* counters = nullptr;  // [kernel][evals, taps, temporal taps]
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pairs[PT_KERNEL_COUNT];
    std::map<int, std::vector<uint32_t>> jump_cache;  // M^(4w)
};

// ---------------------------------------------------------------------------
// errors and allocation
// ---------------------------------------------------------------------------

static pt_status fail(pt_ctx* c, pt_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
    return s;
}

#define CU(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(c, PT_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define LN(call)              \
    do {                              \
        CU(call);                     \
        c->launches++;                \
    } while (0)

#define TRY(expr)                      \
    do {                               \
        pt_status s_ = (expr);         \
        if (s_ != PT_OK) return s_;    \
    } while (0)

// Device memory of a context.  Freed blocks are kept in a per-context cache
// and handed out again (all of a context's work is ordered on its stream, so
// a block's next user runs after its previous one): in steady state no
// cudaFree runs, which would wait for the whole device and stall the other
// contexts working beside this one.  The cache is released when an
// allocation would exceed the budget or cudaMalloc fails.
static void destroy_tex_array(TexArray& t) {
    if (t.tex) cudaDestroyTextureObject(t.tex);
    if (t.arr) cudaFreeArray(t.arr);
    t = TexArray();
}

static void release_cache(pt_ctx* c) {
    if (c->cache.empty() && c->tex_free.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto& kv : c->cache) cudaFree(kv.second);
    c->cache.clear();
    for (auto& t : c->tex_free) destroy_tex_array(t);
    c->tex_free.clear();
    c->cached = 0;
}
// Block sizes are rounded up to classes of 1/8 of a power of two (at most
// 12.5 % larger than asked); a request takes the smallest cached block that
// fits if it is at most twice its size, so blocks are reused across requests
// of different sizes.
static size_t size_class(size_t bytes) {
    if (bytes <= 4096) return (bytes + 255) & ~(size_t)255;
    size_t top = 1;
    while ((top << 1) <= bytes) top <<= 1;  // highest power of two <= bytes
    const size_t step = top / 8;
    return (bytes + step - 1) / step * step;
}
static pt_status dalloc(pt_ctx* c, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    bytes = size_class(bytes);
    auto it = c->cache.lower_bound(bytes);  // the smallest cached block that fits, if at most twice the size
    if (it != c->cache.end() && it->first <= 2 * bytes) {
        const size_t sz = it->first;
        *p = it->second;
        c->cache.erase(it);
        c->cached -= sz;
        c->allocated += sz;
        c->allocs[*p] = sz;
    } else {
        if (c->budget && c->allocated + c->cached + bytes > c->budget) release_cache(c);
        if (c->budget && c->allocated + bytes > c->budget)
            return fail(c, PT_ERR_BUDGET, "allocation of %zu bytes exceeds the HBM budget (%zu of %zu used)", bytes,
                        c->allocated, c->budget);
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            release_cache(c);
            e = cudaMalloc(p, bytes);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            *p = nullptr;
            return fail(c, PT_ERR_OOM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        }
        c->allocated += bytes;
        c->allocs[*p] = bytes;
    }
    cudaError_t e = cudaMemsetAsync(*p, 0, bytes, c->stream);
    if (e != cudaSuccess) return fail(c, PT_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    return PT_OK;
}
template <class T>
static pt_status dalloc_t(pt_ctx* c, T** p, size_t count) {
    void* v = nullptr;
    pt_status s = dalloc(c, &v, count * sizeof(T));
    *p = (T*)v;
    return s;
}
static void dfree(pt_ctx* c, void* p) {
    if (!p) return;
    auto it = c->allocs.find(p);
    if (it == c->allocs.end()) {
        cudaFree(p);
        return;
    }
    c->allocated -= it->second;
    c->cached += it->second;
    c->cache.insert(std::make_pair(it->second, p));
    c->allocs.erase(it);
}
template <class T>
static void dfree_t(pt_ctx* c, T*& p) {
    dfree(c, (void*)p);
    p = nullptr;
}

static pt_status ensure_stage(pt_ctx* c, size_t bytes) {
    if (c->stage_bytes >= bytes) return PT_OK;
    dfree(c, c->stage);
    c->stage = nullptr;
    c->stage_bytes = 0;
    TRY(dalloc(c, &c->stage, bytes));
    c->stage_bytes = bytes;
    return PT_OK;
}

// ---------------------------------------------------------------------------
// kernel parameters
// ---------------------------------------------------------------------------

static PatchPlanes base_planes(pt_ctx* c) { return c->off[c->base_i]; }

static Params make_params(pt_ctx* c, int level) {
    Params P;
    memset(&P, 0, sizeof(P));
    const pt_params& p = c->params;
    P.W = c->W;
    P.H = c->H;
    P.level = level;
    P.lw = c->W >> level;
    P.lh = c->H >> level;
    P.r = p.residualWindowSize;
    for (int i = 0; i < 2 * P.r + 1; i++) P.gauss[i] = c->gauss[i];
    P.scaleWU = p.residualWindowScaleU;
    P.scaleWV = p.residualWindowScaleV;
    P.alphaWeight = p.alphaWeight;
    P.inputAnalogyWeight = p.inputAnalogyWeight;
    P.canvasOutputWeight = p.canvasOutputWeight;
    P.distTransWeight = p.distTransWeight;
    P.styleObjIdWeight = p.styleObjIdWeight;
    P.coherenceWeight = p.coherenceWeight;
    P.coherenceRatioRange = p.coherenceRatioRange;
    P.coherenceAngleRange = p.coherenceAngleRange;
    P.tdIn = p.timeDerivativeInputWeight;
    P.tdOut = p.timeDerivativeOutputWeight;
    P.tc = p.temporalCoherenceWeight;
    P.maxDistortion = p.maxDistortion;
    P.hysteresisWeight = p.hysteresisWeight;
    for (int i = 0; i < PT_MAX_STYLES; i++) {
        P.histThreshold[i] = p.offsetsHistogramThreshold[i];
        P.histSlope[i] = p.offsetsHistogramSlope[i];
    }
    // A candidate's partial patch sum can only grow when every weight that
    // scales a per-tap term is non-negative (NaN weights fail the test).
    {
        bool nonneg = P.alphaWeight >= 0.f && P.inputAnalogyWeight >= 0.f && P.canvasOutputWeight >= 0.f &&
                      P.tdIn >= 0.f && P.tdOut >= 0.f && P.tc >= 0.f;
        for (int i = 0; i < PT_MAX_STYLES; i++) nonneg = nonneg && P.histSlope[i] >= 0.f;
        for (int i = 0; i < 2 * P.r + 1; i++) nonneg = nonneg && P.gauss[i] >= 0.f;
        P.earlyExit = nonneg ? 1 : 0;
    }
    if (P.r <= 4) {
        // taps by descending weight (the weights as the kernels form them)
        const int n = 2 * P.r + 1, K = n * n;
        std::vector<std::pair<float, int>> order;
        for (int t = 0; t < K; t++) order.push_back(std::make_pair(P.gauss[t / n] * P.gauss[t % n], t));
        std::stable_sort(order.begin(), order.end(),
                         [](const std::pair<float, int>& a, const std::pair<float, int>& b) { return a.first > b.first; });
        for (int k = 0; k < K; k++) P.tapOrder[k] = (uint8_t)order[k].second;
    }
    P.jitter = p.advectionJitter;
    P.numStyles = p.numStyles > 0 ? p.numStyles : 1;
    P.transparencyOk = p.transparencyOk;
    P.orientationEnabled = p.orientationEnabled;
    P.lumShiftEnable = p.lumShiftEnable;
    P.distTransCull = p.distTransCull;
    P.direction = p.direction;
    P.scatterSamples = p.scatterSamplesCount;
    P.colorspace = p.colorspace;
    P.firstKey = p.firstKeyIndex;
    P.lastKey = p.lastKeyIndex;
    P.rngMode = p.rngMode;
    P.rngSeed = p.rngSeed;
    P.histPitch = c->SW;
    P.histRows = c->SH * c->NS;
    P.histW = c->SW >> level;
    P.histH = (c->SH * c->NS) >> level;
    P.hist = c->hist[0];
    if (c->ex) {
        P.ex.base = c->ex->base;
        P.ex.out = c->ex->out;
        P.ex.bo = c->ex->bo;
        P.ex.orient = c->ex->orient;
        P.ex.dt = c->ex->dt;
        P.ex.ids = c->ex->ids;
        P.ex.w = c->ex->w;
        P.ex.h = c->ex->h;
        P.ex.ns = c->NS;
        P.ex.hw = p.filterMode == PT_FILTER_TEXTURE;
        if (P.ex.hw && !c->ex->tex_stale) {
            P.ex.tbase = c->ex->ta[0].tex;
            P.ex.tout = c->ex->ta[1].tex;
        }
    }
    P.hwFilter = p.filterMode == PT_FILTER_TEXTURE;
    P.img = c->img;
    P.off = base_planes(c);
    P.res = c->res[c->res_i];
    P.canvas = c->canvas;
    P.adv[0] = c->adv[0];
    P.adv[1] = c->adv[1];
    P.inc = ptk::IncView{c->chg, c->stamp_last, c->stamp_win, c->inc_on, c->inc_pi, c->inc_prev,
                         c->tap_cache, c->inc_fill};
    return P;
}

// a level's texture arrays back to the context's free list
static void free_textures(pt_ctx* c, ExLevel* L) {
    for (int k = 0; k < 2; k++) {
        if (L->ta[k].arr) {
            c->allocated -= L->ta[k].bytes;
            c->cached += L->ta[k].bytes;
            c->tex_free.push_back(L->ta[k]);
        }
        L->ta[k] = TexArray();
    }
    L->tex_stale = true;
}

// a free texture array of at least w x h texels and `layers` layers (the
// smallest that fits), else a new one with its extent rounded up to 64
static pt_status take_tex_array(pt_ctx* c, int w, int h, int layers, TexArray* out) {
    int best = -1;
    for (int i = 0; i < (int)c->tex_free.size(); i++) {
        const TexArray& t = c->tex_free[i];
        if (t.layers != layers || t.cw < w || t.ch < h) continue;
        if (best < 0 || t.bytes < c->tex_free[best].bytes) best = i;
    }
    if (best >= 0 && c->tex_free[best].bytes <= 4 * (size_t)w * h * layers * sizeof(float4) + (1u << 20)) {
        *out = c->tex_free[best];
        c->tex_free.erase(c->tex_free.begin() + best);
        c->cached -= out->bytes;
        c->allocated += out->bytes;
        return PT_OK;
    }
    TexArray t;
    t.cw = (w + 1 + 63) / 64 * 64;  // room for the repeated edge column and row
    t.ch = (h + 1 + 63) / 64 * 64;
    t.layers = layers;
    t.bytes = (size_t)t.cw * t.ch * layers * sizeof(float4);
    if (c->budget && c->allocated + c->cached + t.bytes > c->budget) release_cache(c);
    cudaChannelFormatDesc d = cudaCreateChannelDesc<float4>();
    cudaError_t e = cudaMalloc3DArray(&t.arr, &d, make_cudaExtent(t.cw, t.ch, layers), cudaArrayLayered);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release_cache(c);
        e = cudaMalloc3DArray(&t.arr, &d, make_cudaExtent(t.cw, t.ch, layers), cudaArrayLayered);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, PT_ERR_OOM, "cudaMalloc3DArray(%dx%dx%d) failed: %s", t.cw, t.ch, layers,
                    cudaGetErrorString(e));
    }
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = t.arr;
    cudaTextureDesc td;
    memset(&td, 0, sizeof td);
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    e = cudaCreateTextureObject(&t.tex, &rd, &td, nullptr);
    if (e != cudaSuccess) {
        destroy_tex_array(t);
        return fail(c, PT_ERR_CUDA, "cudaCreateTextureObject: %s", cudaGetErrorString(e));
    }
    c->allocated += t.bytes;
    *out = t;
    return PT_OK;
}

// one copy of the w x h x layers block at (sx, sy) of layered planes
// (pitch_texels x plane_rows texels per layer) into an array at (dx, dy):
// the source pointer is offset to the block, whose rows and layers keep the
// planes' strides
static cudaError_t copy_to_array(const float4* src, int pitch_texels, int plane_rows, int sx, int sy, cudaArray_t dst,
                                 int dx, int dy, int w, int h, int layers, cudaStream_t st) {
    cudaMemcpy3DParms cp;
    memset(&cp, 0, sizeof cp);
    const size_t pitch = (size_t)pitch_texels * sizeof(float4);
    cp.srcPtr = make_cudaPitchedPtr((void*)(src + (size_t)sy * pitch_texels + sx), pitch, pitch, plane_rows);
    cp.dstArray = dst;
    cp.dstPos = make_cudaPos(dx, dy, 0);
    cp.extent = make_cudaExtent(w, h, layers);
    cp.kind = cudaMemcpyDeviceToDevice;
    return cudaMemcpy3DAsync(&cp, st);
}

// the textures of an exemplar level (PT_FILTER_TEXTURE), copied from its
// planes after they were written: the level into the array's corner, then
// its last column, last row and corner texel once more beyond them
static pt_status refresh_textures(pt_ctx* c, ExLevel* L) {
    if (!L->base) return PT_OK;
    const int w = L->w, h = L->h, ns = c->NS;
    if (L->ta[0].arr && (L->ta[0].cw < w + 1 || L->ta[0].ch < h + 1 || L->ta[0].layers != ns)) free_textures(c, L);
    if (!L->tex_stale && L->ta[0].arr) return PT_OK;
    for (int k = 0; k < 2; k++) {
        if (!L->ta[k].arr) TRY(take_tex_array(c, w + 1, h + 1, ns, &L->ta[k]));
        const float4* src = k ? L->out : L->base;
        cudaArray_t a = L->ta[k].arr;
        CU(copy_to_array(src, w, h, 0, 0, a, 0, 0, w, h, ns, c->stream));
        CU(copy_to_array(src, w, h, w - 1, 0, a, w, 0, 1, h, ns, c->stream));
        CU(copy_to_array(src, w, h, 0, h - 1, a, 0, h, w, 1, ns, c->stream));
        CU(copy_to_array(src, w, h, w - 1, h - 1, a, w, h, 1, 1, ns, c->stream));
    }
    L->tex_stale = false;
    return PT_OK;
}

// the copies of an exemplar level that the tiled kernels gather from (the
// interleaved records, and with PT_FILTER_TEXTURE the textures), rebuilt
// after its planes were written
static pt_status refresh_interleaved(pt_ctx* c, ExLevel* L) {
    if (L->bo_stale && L->bo && L->base) {
        LN(pt::launch_interleave_texels(L->base, L->out, L->bo, (size_t)L->w * L->h * c->NS, c->stream));
        L->bo_stale = false;
    }
    if (c->params.filterMode == PT_FILTER_TEXTURE) TRY(refresh_textures(c, L));
    return PT_OK;
}

template <class T>
static pt_status zero_layer(pt_ctx* c, T** buf, Arr<T>* bind) {
    if (bind->p) return PT_OK;
    const size_t n = (size_t)c->W * c->H;
    if (!*buf) TRY(dalloc_t(c, buf, n));
    CU(cudaMemsetAsync(*buf, 0, n * sizeof(T), c->stream));
    *bind = Arr<T>{*buf, c->W, c->H};
    return PT_OK;
}
static pt_status bind_unwritten_layers(pt_ctx* c) {
    for (int i = 0; i < 2; i++) {
        TRY(zero_layer(c, &c->up_base[i], &c->img.base[i]));
        TRY(zero_layer(c, &c->up_dt[i], &c->img.dt[i]));
        TRY(zero_layer(c, &c->up_velf[i], &c->img.velf[i]));
        TRY(zero_layer(c, &c->up_velb[i], &c->img.velb[i]));
    }
    return PT_OK;
}

static pt_status check_ready(pt_ctx* c, int level, bool need_ex = true, bool need_img = true) {
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    if (!c->have_params) return fail(c, PT_ERR_STATE, "pt_set_params has not been called");
    if (level < 0 || (c->W >> level) < 1 || (c->H >> level) < 1)
        return fail(c, PT_ERR_INVALID, "level %d out of range", level);
    if (need_ex && (!c->ex || !c->ex->base)) return fail(c, PT_ERR_STATE, "no exemplar level loaded");
    if (need_ex) TRY(refresh_interleaved(c, c->ex));
    if (need_img) {
        // A layered input holds whatever level was last written into it, as
        // the reference's layered textures do (a kernel at another level
        // reads that level's texels, and zero outside them); a layer never
        // written reads zero (a zeroed full-size array is bound to it).
        TRY(bind_unwritten_layers(c));
        const ImgView& I = c->img;
        if (!I.orient.p || !I.scale.p || !I.ids.p)
            return fail(c, PT_ERR_STATE, "input orientation/scale/ids not uploaded");
    }
    return PT_OK;
}

// copy-on-write helpers for the offsets pair
static pt_status copy_planes_full(pt_ctx* c, PatchPlanes dst, PatchPlanes src) {
    size_t n = (size_t)c->W * c->H;
    CU(cudaMemcpyAsync(dst.A, src.A, n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(dst.B, src.B, n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(dst.C, src.C, n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    return PT_OK;
}
// The shared buffer of an aliased pair is about to be split for a write
// inside the rectangle of `level`: the other buffer is taken as it is when
// it already holds the same records outside that rectangle, else after a
// full copy.
static pt_status split_aliased(pt_ctx* c, int level) {
    const int other = 1 - c->base_i;
    if (c->off_span < level) {
        TRY(copy_planes_full(c, c->off[other], c->off[c->base_i]));
        c->off_span = kSpanNone;
    }
    c->off_span = std::min(c->off_span, level);
    return PT_OK;
}
static pt_status writable_work(pt_ctx* c, int level, PatchPlanes* out, bool* was_aliased = nullptr) {
    if (was_aliased) *was_aliased = (c->work_i == c->base_i);
    if (c->work_i == c->base_i) {
        TRY(split_aliased(c, level));
        c->work_i = 1 - c->base_i;
    }
    c->off_span = std::min(c->off_span, level);
    *out = c->off[c->work_i];
    return PT_OK;
}
// base about to be partly overwritten: give it its own buffer first
static pt_status base_for_partial_write(pt_ctx* c, int level, PatchPlanes* out) {
    if (c->base_i == c->work_i) {
        int nb = 1 - c->work_i;
        TRY(copy_planes_full(c, c->off[nb], c->off[c->work_i]));
        c->base_i = nb;
        c->off_span = kSpanNone;
    }
    c->off_span = std::min(c->off_span, level);
    *out = c->off[c->base_i];
    return PT_OK;
}

// ---------------------------------------------------------------------------
// syncBuffers and friends
// ---------------------------------------------------------------------------

static bool histogram_on(pt_ctx* c) {
    for (int i = 0; i < c->params.numStyles && i < PT_MAX_STYLES; i++)
        if (c->params.offsetsHistogramSlope[i] > 0.0f) return true;
    return false;
}

// ---------------------------------------------------------------------------
// profiled launches: an event pair around the launch and the kernel's own
// evaluation counters
// ---------------------------------------------------------------------------

static cudaEvent_t pool_event(pt_ctx* c) {
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

template <class F>
static pt_status profiled(pt_ctx* c, int kernel, Params& P, F&& launch) {
    if (c->profiling & PT_PROFILE_COUNTERS) P.counters = c->counters + 3 * kernel;
    if (!(c->profiling & PT_PROFILE_TIMING)) {
        LN(launch(P));
        return PT_OK;
    }
    cudaEvent_t a = pool_event(c), b = pool_event(c);
    if (!a || !b) return fail(c, PT_ERR_CUDA, "cudaEventCreate failed");
    CU(cudaEventRecord(a, c->stream));
    LN(launch(P));
    CU(cudaEventRecord(b, c->stream));
    c->ev_pairs[kernel].push_back(std::make_pair(a, b));
    return PT_OK;
}

// Temporal mode of the tiled kernels: which advected buffer can make the
// temporal terms of calculateResidual active (texSynth_kernel.cu:610-627).
// Returns -1 when both can (bidirectional), which the tiled kernels do not
// cover.
static int temporal_mode(pt_ctx* c) {
    const pt_params& p = c->params;
    bool td = p.timeDerivativeInputWeight > 0.f || p.timeDerivativeOutputWeight > 0.f ||
              p.temporalCoherenceWeight > 0.f;
    bool f = td && c->adv_written[0] && (p.direction == PT_FORWARD || p.direction == PT_BIDIRECTIONAL);
    bool b = td && c->adv_written[1] && (p.direction == PT_BACKWARD || p.direction == PT_BIDIRECTIONAL);
    if (f && b) return -1;
    return f ? 1 : (b ? 2 : 0);
}

// whether the tiled kernels cover the current configuration
static bool tiled_usable(pt_ctx* c) {
    int r = c->params.residualWindowSize;
    return c->use_tiled && !c->params.interpolateKeyFrame && c->params.colorspace == 0 &&
           c->params.coherenceWeight <= 0.f &&
           temporal_mode(c) >= 0 && r >= 2 && r <= 4;
}

// launches the tiled kernel of `kind` if one is instantiated for this
// configuration; *done = false otherwise (the generic kernel is used)
static cudaError_t launch_tiled(pt_ctx* c, int kind, const Params& P, PatchPlanes work, int arg, uint32_t pass_id,
                                float* out, bool* done) {
    *done = false;
    if (!tiled_usable(c)) return cudaSuccess;
    int tm = temporal_mode(c);
    *done = true;
    switch (P.r) {
        case 2: return pt::launch_tiled_2(kind, tm, P, work, arg, pass_id, out, c->stream);
        case 3: return pt::launch_tiled_3(kind, tm, P, work, arg, pass_id, out, c->stream);
        case 4: return pt::launch_tiled_4(kind, tm, P, work, arg, pass_id, out, c->stream);
        default: *done = false; return cudaSuccess;
    }
}

static pt_status do_residual(pt_ctx* c, int level) {
    Params P = make_params(c, level);
    float* out = c->res[c->res_i];
    return profiled(c, PT_KERNEL_RESIDUAL, P, [&](const Params& Q) {
        bool done = false;
        cudaError_t e = launch_tiled(c, 2, Q, PatchPlanes{}, 0, 0, out, &done);
        return done ? e : pt::launch_residual(Q, out, c->stream);
    });
}

// TexSynth::syncBuffers, texSynth_kernel.cu:1240-1303
static pt_status do_sync(pt_ctx* c, int level, int flags) {
    if (!(flags & PT_DONT_COPY_OFFSETS)) c->base_i = c->work_i;
    // calculateOffsetsHistogram adds nothing (its atomicAdd is commented out
    // at :258), so the histogram is zeroed and its blur (rows base ->
    // working, columns working -> base) of zeros is zeros again: once both
    // buffers hold zeros there is nothing left to recompute.
    if (histogram_on(c) && !c->hist_zero) {
        size_t hn = (size_t)c->SW * c->SH * c->NS * sizeof(float);
        CU(cudaMemsetAsync(c->hist[0], 0, hn, c->stream));
        CU(cudaMemsetAsync(c->hist[1], 0, hn, c->stream));
        int hw = c->SW >> level, hh = (c->SH * c->NS) >> level;
        LN(pt::launch_conv(c->hist[0], c->hist[1], hw, hh, c->SW, 1, c->hist_kernel, c->stream));
        LN(pt::launch_conv(c->hist[1], c->hist[0], hw, hh, c->SW, 0, c->hist_kernel, c->stream));
        c->hist_zero = true;
    }
    Params P = make_params(c, level);
    TRY(profiled(c, PT_KERNEL_CANVAS, P, [&](const Params& Q) { return pt::launch_canvas(Q, c->canvas, c->stream); }));
    if (!(flags & PT_DONT_UPDATE_RESIDUAL)) TRY(do_residual(c, level));
    return PT_OK;
}

// ---------------------------------------------------------------------------
// glibc random(): seeding and jump-ahead (row-parallel random levels)
// ---------------------------------------------------------------------------

// state of the TYPE_3 generator after srand(seed): the 31 values
// r[313..343] that produce the first output r[344] >> 1
static void glibc_state(uint32_t seed, uint32_t out[31]) {
    int32_t word = (int32_t)seed;
    if (seed == 0) word = 1;
    std::vector<uint32_t> r(344);
    r[0] = (uint32_t)word;
    for (int i = 1; i < 31; i++) {
        int32_t hi = word / 127773, lo = word % 127773;
        word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        r[i] = (uint32_t)word;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 34; i < 344; i++) r[i] = r[i - 31] + r[i - 3];
    for (int i = 0; i < 31; i++) out[i] = r[313 + i];
}

// 31x31 matrices over Z/2^32, row-major
static void matmul31(const uint32_t* a, const uint32_t* b, uint32_t* out) {
    for (int i = 0; i < 31; i++)
        for (int j = 0; j < 31; j++) {
            uint32_t s = 0;
            for (int k = 0; k < 31; k++) s += a[i * 31 + k] * b[k * 31 + j];
            out[i * 31 + j] = s;
        }
}
static std::vector<uint32_t> step_power(uint64_t n) {
    // one step: s'[i] = s[i+1] (i < 30), s'[30] = s[0] + s[28]
    std::vector<uint32_t> M(961, 0), R(961, 0), T(961);
    for (int i = 0; i < 30; i++) M[i * 31 + i + 1] = 1;
    M[30 * 31 + 0] = 1;
    M[30 * 31 + 28] += 1;
    for (int i = 0; i < 31; i++) R[i * 31 + i] = 1;
    while (n) {
        if (n & 1) { matmul31(R.data(), M.data(), T.data()); R.swap(T); }
        matmul31(M.data(), M.data(), T.data());
        M.swap(T);
        n >>= 1;
    }
    return R;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

// The public functions below take their C linkage from the declarations in
// painttween.h.

int pt_abi_version(void) { return PT_ABI_VERSION; }

const char* pt_status_string(pt_status s) {
    switch (s) {
        case PT_OK: return "PT_OK";
        case PT_ERR_INVALID: return "PT_ERR_INVALID";
        case PT_ERR_CUDA: return "PT_ERR_CUDA";
        case PT_ERR_OOM: return "PT_ERR_OOM";
        case PT_ERR_STATE: return "PT_ERR_STATE";
        case PT_ERR_UNSUPPORTED: return "PT_ERR_UNSUPPORTED";
        case PT_ERR_TIMEOUT: return "PT_ERR_TIMEOUT";
        case PT_ERR_BUDGET: return "PT_ERR_BUDGET";
    }
    return "PT_ERR_UNKNOWN";
}

const char* pt_last_error(const pt_ctx* c) { return c ? c->err.c_str() : "null context"; }
size_t pt_device_bytes(const pt_ctx* c) { return c ? c->allocated + c->cached : 0; }
uint64_t pt_kernel_launches(const pt_ctx* c) { return c ? c->launches : 0; }

void pt_default_params(pt_params* p) {
    memset(p, 0, sizeof(*p));
    p->residualWindowSize = 4;
    p->inputAnalogyWeight = 1.0f;
    p->canvasOutputWeight = 1.0f;
    p->orientationEnabled = 1;
    p->numStyles = 1;
    p->maxDistortion = 4.0f;
    p->alphaWeight = 1.0f;
    p->coherenceRatioRange = 2.0f;
    p->coherenceAngleRange = 0.25f;
    p->levels = 4;
    p->scatterSamplesCount = 25;
    p->timeDerivativeInputWeight = 1.f;
    p->timeDerivativeOutputWeight = 1.f;
    p->temporalCoherenceWeight = 0.2f;
    p->distTransCull = 50;
    p->residualWindowScaleU = 1;
    p->residualWindowScaleV = 1;
    p->firstKeyIndex = -1;
    p->lastKeyIndex = -1;
    p->direction = PT_BIDIRECTIONAL;
    p->iterations = 3;
    p->fixupPasses = 1;
    p->scheme = PT_S_FMBM_RM;
    p->finalLevel = 0;
    p->rngMode = PT_RNG_REFERENCE;
    p->filterMode = PT_FILTER_TEXTURE;  // the reference's texture-unit sampling
}

pt_status pt_create(int device, size_t budget, pt_ctx** out) {
    if (!out) return PT_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return PT_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return PT_ERR_CUDA;
    pt_ctx* c = new pt_ctx();
    c->device = device;
    c->budget = budget;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return PT_ERR_CUDA;
    }
    pt_default_params(&c->params);
    if (dalloc_t(c, &c->flag, 4) != PT_OK) {
        cudaStreamDestroy(c->stream);
        delete c;
        return PT_ERR_OOM;
    }
    *out = c;
    return PT_OK;
}

static void free_frames(pt_ctx* c) {
    for (auto& kv : c->frames)
        for (auto& L : kv.second) {
            dfree_t(c, L.rgba); dfree_t(c, L.orient); dfree_t(c, L.dt); dfree_t(c, L.ids);
            dfree_t(c, L.velf); dfree_t(c, L.velb); dfree_t(c, L.scale);
        }
    c->frames.clear();
    for (auto& kv : c->ribbons)
        for (auto& L : kv.second) {
            dfree_t(c, L.first); dfree_t(c, L.second);
        }
    c->ribbons.clear();
}
static void free_store(pt_ctx* c) {
    for (auto& kv : c->store) {
        dfree_t(c, kv.second.offs);
        dfree_t(c, kv.second.res);
        dfree_t(c, kv.second.canvas);
    }
    c->store.clear();
    c->last_saved.clear();
}

pt_status pt_destroy(pt_ctx* c) {
    if (!c) return PT_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& e : c->timers)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->ev_pool) cudaEventDestroy(e);
    for (auto& v : c->ev_pairs)
        for (auto& pr : v) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    free_textures(c, &c->up_ex);
    for (auto& L : c->style_levels) free_textures(c, &L);
    for (auto& t : c->tex_free) destroy_tex_array(t);
    c->tex_free.clear();
    for (auto& kv : c->allocs) cudaFree(kv.first);
    c->allocs.clear();
    for (auto& kv : c->cache) cudaFree(kv.second);
    c->cache.clear();
    if (c->cb_stage) cudaFreeHost(c->cb_stage);
    cudaStreamDestroy(c->stream);
    delete c;
    return PT_OK;
}

pt_status pt_synchronize(pt_ctx* c) {
    if (!c) return PT_ERR_INVALID;
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

pt_status pt_set_params(pt_ctx* c, const pt_params* p) {
    if (!c || !p) return PT_ERR_INVALID;
    if (p->residualWindowSize < 0 || p->residualWindowSize > ptk::kMaxRadius)
        return fail(c, PT_ERR_INVALID, "residualWindowSize %d outside [0, %d]", p->residualWindowSize,
                    ptk::kMaxRadius);
    if (p->colorspace != 0 && p->colorspace != 1) return fail(c, PT_ERR_INVALID, "colorspace must be 0 (RGB) or 1 (Lab)");
    if (p->numStyles < 1 || p->numStyles > PT_MAX_STYLES) return fail(c, PT_ERR_INVALID, "numStyles out of range");
    if (p->rngMode != PT_RNG_REFERENCE && p->rngMode != PT_RNG_COUNTER)
        return fail(c, PT_ERR_INVALID, "unknown rngMode");
    if (p->filterMode != PT_FILTER_EXACT && p->filterMode != PT_FILTER_TEXTURE)
        return fail(c, PT_ERR_INVALID, "unknown filterMode");
    c->params = *p;
    c->have_params = true;
    if (c->ex) TRY(refresh_interleaved(c, c->ex));
    // TexSynth::setup: unnormalised Gaussian with sigma = r/3
    // (allocateGaussianKernel(..., normalize=false), convolution.cu:37-60)
    int r = p->residualWindowSize;
    pt::gaussian_weights(r, false, c->gauss);
    c->hist_kernel.r = r;  // normalised copy for the histogram smoothing
    pt::gaussian_weights(r, true, c->hist_kernel.w);
    return PT_OK;
}

pt_status pt_get_params(const pt_ctx* c, pt_params* out) {
    if (!c || !out) return PT_ERR_INVALID;
    *out = c->params;
    return PT_OK;
}

static pt_status alloc_planes(pt_ctx* c, PatchPlanes* p, size_t n) {
    TRY(dalloc_t(c, &p->A, n));
    TRY(dalloc_t(c, &p->B, n));
    TRY(dalloc_t(c, &p->C, n));
    return PT_OK;
}
static void free_planes(pt_ctx* c, PatchPlanes* p) {
    dfree_t(c, p->A);
    dfree_t(c, p->B);
    dfree_t(c, p->C);
}

pt_status pt_initialize(pt_ctx* c, int iw, int ih, int sw, int sh, int ns) {
    if (!c) return PT_ERR_INVALID;
    if (iw < 2 || ih < 2 || sw < 2 || sh < 2 || ns < 1 || ns > PT_MAX_STYLES)
        return fail(c, PT_ERR_INVALID, "bad sizes %dx%d style %dx%dx%d", iw, ih, sw, sh, ns);
    // pixel and texel ids are 32-bit in the kernels
    if ((long long)iw * ih > INT32_MAX || (long long)sw * sh * ns > INT32_MAX)
        return fail(c, PT_ERR_INVALID, "sizes too large: %dx%d image, %dx%dx%d styles (at most 2^31-1 pixels each)",
                    iw, ih, sw, sh, ns);
    CU(cudaSetDevice(c->device));
    if (c->initialized && iw == c->W && ih == c->H && sw == c->SW && sh == c->SH && ns == c->NS) return PT_OK;
    // release the image-size state
    for (int i = 0; i < 2; i++) {
        free_planes(c, &c->off[i]);
        dfree_t(c, c->res[i]);
        dfree_t(c, c->hist[i]);
        free_planes(c, &c->adv[i].off);
        dfree_t(c, c->adv[i].base); dfree_t(c, c->adv[i].out); dfree_t(c, c->adv[i].res); dfree_t(c, c->adv[i].ts);
        dfree_t(c, c->up_base[i]); dfree_t(c, c->up_dt[i]); dfree_t(c, c->up_velf[i]); dfree_t(c, c->up_velb[i]);
    }
    dfree_t(c, c->canvas); dfree_t(c, c->up_orient); dfree_t(c, c->up_scale); dfree_t(c, c->up_ids);
    dfree_t(c, c->rnd);
    for (int i = 0; i < 2; i++) {
        dfree_t(c, c->cumul[i]); dfree_t(c, c->f2k_buf[i]); dfree_t(c, c->rib[i]);
    }
    c->cf_w = c->cf_h = c->cf_n = 0;
    dfree_t(c, c->chg); dfree_t(c, c->stamp_last); dfree_t(c, c->stamp_win);
    dfree_t(c, c->tap_cache);
    c->tap_cache_k = 0;
    free_store(c);
    c->initialized = false;
    c->W = iw; c->H = ih; c->SW = sw; c->SH = sh; c->NS = ns;
    size_t n = (size_t)iw * ih;
    for (int i = 0; i < 2; i++) {
        TRY(alloc_planes(c, &c->off[i], n));
        TRY(dalloc_t(c, &c->res[i], n));
        TRY(dalloc_t(c, &c->hist[i], (size_t)sw * sh * ns));
        c->hist_zero = false;
        TRY(alloc_planes(c, &c->adv[i].off, n));
        TRY(dalloc_t(c, &c->adv[i].base, n));
        TRY(dalloc_t(c, &c->adv[i].out, n));
        TRY(dalloc_t(c, &c->adv[i].res, n));
        TRY(dalloc_t(c, &c->adv[i].ts, n));
    }
    TRY(dalloc_t(c, &c->canvas, n));
    TRY(dalloc_t(c, &c->chg, n));
    TRY(dalloc_t(c, &c->stamp_last, n));
    TRY(dalloc_t(c, &c->stamp_win, n));
    CU(cudaMemsetAsync(c->stamp_last, 0, n * sizeof(int), c->stream));
    CU(cudaMemsetAsync(c->stamp_win, 0, n * sizeof(int), c->stream));
    c->inc_seq = 0;
    c->base_i = c->work_i = 0;
    c->off_span = 0;  // fresh buffers: nothing known to agree
    c->res_i = 0;
    memset(&c->img, 0, sizeof(c->img));
    c->initialized = true;
    return PT_OK;
}

// zero the working state (the reference starts each synthesis from freshly
// memset buffers, cudaImageBuffer.h:154-162)
static pt_status reset_working(pt_ctx* c) {
    size_t n = (size_t)c->W * c->H;
    for (int i = 0; i < 2; i++) {
        CU(cudaMemsetAsync(c->off[i].A, 0, n * sizeof(float4), c->stream));
        CU(cudaMemsetAsync(c->off[i].B, 0, n * sizeof(float4), c->stream));
        CU(cudaMemsetAsync(c->off[i].C, 0, n * sizeof(float), c->stream));
        CU(cudaMemsetAsync(c->res[i], 0, n * sizeof(float), c->stream));
        CU(cudaMemsetAsync(c->hist[i], 0, (size_t)c->SW * c->SH * c->NS * sizeof(float), c->stream));
    }
    c->hist_zero = true;
    CU(cudaMemsetAsync(c->canvas, 0, n * sizeof(float4), c->stream));
    c->base_i = c->work_i = 0;
    c->off_span = kSpanNone;  // both buffers all zero
    c->res_i = 0;
    c->pass_counter = 0;
    return pt_reset_advected_buffers(c);
}

pt_status pt_reset_advected_buffers(pt_ctx* c) {
    if (!c || !c->initialized) return PT_ERR_STATE;
    c->adv_written[0] = c->adv_written[1] = false;
    size_t n = (size_t)c->W * c->H;
    for (int i = 0; i < 2; i++) {
        CU(cudaMemsetAsync(c->adv[i].off.A, 0, n * sizeof(float4), c->stream));
        CU(cudaMemsetAsync(c->adv[i].off.B, 0, n * sizeof(float4), c->stream));
        CU(cudaMemsetAsync(c->adv[i].off.C, 0, n * sizeof(float), c->stream));
        CU(cudaMemsetAsync(c->adv[i].base, 0, n * sizeof(float4), c->stream));
        CU(cudaMemsetAsync(c->adv[i].out, 0, n * sizeof(float4), c->stream));
        CU(cudaMemsetAsync(c->adv[i].res, 0, n * sizeof(float), c->stream));
        CU(cudaMemsetAsync(c->adv[i].ts, 0, n * sizeof(int), c->stream));
    }
    return PT_OK;
}

pt_status pt_initialize_exemplars(pt_ctx* c, int w, int h, int ns) {
    if (!c) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    if (w < 2 || h < 2 || ns != c->NS || (long long)w * h * ns > INT32_MAX)
        return fail(c, PT_ERR_INVALID, "bad exemplar size %dx%dx%d", w, h, ns);
    size_t n = (size_t)w * h * ns;
    if (n > c->ex_cap) {
        dfree_t(c, c->up_ex.base); dfree_t(c, c->up_ex.out); dfree_t(c, c->up_ex.bo);
        dfree_t(c, c->up_ex.orient); dfree_t(c, c->up_ex.dt); dfree_t(c, c->up_ex.ids);
        TRY(dalloc_t(c, &c->up_ex.base, n));
        TRY(dalloc_t(c, &c->up_ex.out, n));
        TRY(dalloc_t(c, &c->up_ex.bo, 2 * n));
        TRY(dalloc_t(c, &c->up_ex.orient, n));
        TRY(dalloc_t(c, &c->up_ex.dt, n));
        TRY(dalloc_t(c, &c->up_ex.ids, n));
        c->ex_cap = n;
    }
    c->up_ex.w = w;
    c->up_ex.h = h;
    c->up_ex.transparent = -1;
    c->up_ex.bo_stale = true;
    c->up_ex.tex_stale = true;
    c->ex = &c->up_ex;
    return PT_OK;
}

// Host-to-device copy that has finished reading `src` on return, so callers
// may reuse or free their host buffer at once (the reference's uploads are
// synchronous as well).
// a level rectangle between a host array and a full-pitch device buffer
static pt_status rect_copy(pt_ctx* c, void* dst, size_t dpitch, const void* src, size_t spitch, size_t row_bytes,
                           int rows, cudaMemcpyKind kind) {
    CU(cudaMemcpy2DAsync(dst, dpitch, src, spitch, row_bytes, rows, kind, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

static pt_status h2d(pt_ctx* c, void* dst, const void* src, size_t bytes) {
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

// A layered input image (colour, distance transform, velocities) as the
// reference keeps it (cudaImageBuffer.h layered copyFromHost): one
// full-size array per layer, which an upload of a level overwrites on that
// level's rectangle only, so texels outside the rectangle keep what a finer
// level left there.  Allocated zeroed; bound with the full width as pitch.
template <class T>
static pt_status slot_write(pt_ctx* c, T** slot, Arr<T>* bind, const void* src, int w, int h, cudaMemcpyKind kind) {
    const size_t n = (size_t)c->W * c->H;
    if (!*slot) {
        TRY(dalloc_t(c, slot, n));
        CU(cudaMemsetAsync(*slot, 0, n * sizeof(T), c->stream));
    }
    CU(cudaMemcpy2DAsync(*slot, (size_t)c->W * sizeof(T), src, (size_t)w * sizeof(T), (size_t)w * sizeof(T), h, kind,
                         c->stream));
    if (kind == cudaMemcpyHostToDevice) CU(cudaStreamSynchronize(c->stream));
    *bind = Arr<T>{*slot, c->W, c->H};
    return PT_OK;
}

// A fresh run: no input image or random level bound, the layered arrays all
// zero.
static pt_status reset_image_slots(pt_ctx* c) {
    const size_t n = (size_t)c->W * c->H;
    c->img.rnd = Arr<float4>{};
    for (int i = 0; i < 2; i++) {
        c->img.base[i] = Arr<float4>{};
        c->img.dt[i] = Arr<float>{};
        c->img.velf[i] = Arr<float2>{};
        c->img.velb[i] = Arr<float2>{};
        if (c->up_base[i]) CU(cudaMemsetAsync(c->up_base[i], 0, n * sizeof(float4), c->stream));
        if (c->up_dt[i]) CU(cudaMemsetAsync(c->up_dt[i], 0, n * sizeof(float), c->stream));
        if (c->up_velf[i]) CU(cudaMemsetAsync(c->up_velf[i], 0, n * sizeof(float2), c->stream));
        if (c->up_velb[i]) CU(cudaMemsetAsync(c->up_velb[i], 0, n * sizeof(float2), c->stream));
    }
    c->img.cur = 0;
    return PT_OK;
}

pt_status pt_upload_image_color4(pt_ctx* c, int level, int layer, const float* rgba, int w, int h, int style) {
    if (!c || !rgba) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    size_t n = (size_t)w * h;
    if (layer == PT_LAYER_EXEMPLAR_BASE || layer == PT_LAYER_EXEMPLAR_OUTPUT) {
        if (!c->ex || c->ex != &c->up_ex || w != c->up_ex.w || h != c->up_ex.h || style < 0 || style >= c->NS)
            return fail(c, PT_ERR_INVALID, "exemplar upload %dx%d style %d does not match pt_initialize_exemplars", w,
                        h, style);
        float4* plane = (layer == PT_LAYER_EXEMPLAR_OUTPUT) ? c->up_ex.out : c->up_ex.base;
        TRY(h2d(c, plane + n * style, rgba, n * sizeof(float4)));
        if (layer == PT_LAYER_EXEMPLAR_OUTPUT) c->up_ex.transparent = -1;
        c->up_ex.bo_stale = true;
        c->up_ex.tex_stale = true;
        return PT_OK;
    }
    if (layer == PT_LAYER_CUMUL_FIELD_B || layer == PT_LAYER_CUMUL_FIELD_F) {
        const int d = layer == PT_LAYER_CUMUL_FIELD_F ? 1 : 0;
        if (!c->cumul[d] || style < 0 || style >= c->cf_n || w > c->cf_w || h > c->cf_h)
            return fail(c, PT_ERR_INVALID, "cumulative field %dx%d layer %d does not fit pt_initialize_cumulative_fields",
                        w, h, style);
        float4* dst = c->cumul[d] + (size_t)style * c->cf_w * c->cf_h;
        return rect_copy(c, dst, (size_t)c->cf_w * sizeof(float4), rgba, (size_t)w * sizeof(float4),
                         (size_t)w * sizeof(float4), h, cudaMemcpyHostToDevice);
    }
    if (level < 0 || w != (c->W >> level) || h != (c->H >> level))
        return fail(c, PT_ERR_INVALID, "image upload %dx%d does not match level %d", w, h, level);
    int cur = c->img.cur;
    if (layer == PT_LAYER_INPUT_COLOR)
        return slot_write(c, &c->up_base[cur], &c->img.base[cur], rgba, w, h, cudaMemcpyHostToDevice);
    if (layer == PT_LAYER_FRAME_TO_KEY_RIBBON_B || layer == PT_LAYER_FRAME_TO_KEY_RIBBON_F) {
        const int d = layer == PT_LAYER_FRAME_TO_KEY_RIBBON_F ? 1 : 0;
        if (!c->f2k_buf[d]) TRY(dalloc_t(c, &c->f2k_buf[d], (size_t)c->W * c->H));
        TRY(h2d(c, c->f2k_buf[d], rgba, n * sizeof(float4)));
        c->img.f2k[d] = Arr<float4>{c->f2k_buf[d], w, h};
        return PT_OK;
    }
    if (layer == PT_LAYER_RANDOM) {
        if (!c->rnd) TRY(dalloc_t(c, &c->rnd, (size_t)c->W * c->H));
        TRY(h2d(c, c->rnd, rgba, n * sizeof(float4)));
        c->img.rnd = Arr<float4>{c->rnd, w, h};
        return PT_OK;
    }
    // the keyframe guides: uploaded by loadAnimImages with
    // guidedInterpolation, read by no kernel (texSynth_kernel.cu:85-86)
    if (layer == PT_LAYER_GUIDE_B || layer == PT_LAYER_GUIDE_F) return PT_OK;
    return fail(c, PT_ERR_UNSUPPORTED, "colour layer %d not supported", layer);
}

pt_status pt_upload_image_float(pt_ctx* c, int level, int layer, const float* data, int w, int h, int style) {
    if (!c || !data) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    size_t n = (size_t)w * h;
    if (layer == PT_LAYER_EXEMPLAR_ORIENTATION || layer == PT_LAYER_EXEMPLAR_DIST_TRANS) {
        if (!c->ex || c->ex != &c->up_ex || w != c->up_ex.w || h != c->up_ex.h || style < 0 || style >= c->NS)
            return fail(c, PT_ERR_INVALID, "exemplar upload does not match pt_initialize_exemplars");
        float* dst = (layer == PT_LAYER_EXEMPLAR_ORIENTATION ? c->up_ex.orient : c->up_ex.dt) + n * style;
        return h2d(c, dst, data, n * sizeof(float));
    }
    if (level < 0 || w != (c->W >> level) || h != (c->H >> level))
        return fail(c, PT_ERR_INVALID, "image upload %dx%d does not match level %d", w, h, level);
    int cur = c->img.cur;
    if (layer == PT_LAYER_INPUT_ORIENTATION) {
        if (!c->up_orient) TRY(dalloc_t(c, &c->up_orient, (size_t)c->W * c->H));
        TRY(h2d(c, c->up_orient, data, n * sizeof(float)));
        c->img.orient = Arr<float>{c->up_orient, w, h};
        return PT_OK;
    }
    if (layer == PT_LAYER_INPUT_DIST_TRANS)
        return slot_write(c, &c->up_dt[cur], &c->img.dt[cur], data, w, h, cudaMemcpyHostToDevice);
    return fail(c, PT_ERR_UNSUPPORTED, "float layer %d not supported", layer);
}

pt_status pt_upload_image_float2(pt_ctx* c, int level, int layer, const float* xy, int w, int h) {
    if (!c || !xy) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    if (level < 0 || w != (c->W >> level) || h != (c->H >> level))
        return fail(c, PT_ERR_INVALID, "image upload %dx%d does not match level %d", w, h, level);
    size_t n = (size_t)w * h;
    int cur = c->img.cur, prev = 1 - c->img.cur;
    float2** store = nullptr;
    Arr<float2>* slot = nullptr;
    switch (layer) {
        case PT_LAYER_INPUT_VEL_B: store = &c->up_velb[cur]; slot = &c->img.velb[cur]; break;
        case PT_LAYER_INPUT_VEL_F: store = &c->up_velf[cur]; slot = &c->img.velf[cur]; break;
        case PT_LAYER_INPUT_VEL_B_PREVIOUS: store = &c->up_velb[prev]; slot = &c->img.velb[prev]; break;
        case PT_LAYER_INPUT_VEL_F_PREVIOUS: store = &c->up_velf[prev]; slot = &c->img.velf[prev]; break;
        case PT_LAYER_INPUT_SCALE: store = &c->up_scale; slot = &c->img.scale; break;
        // surface ids: uploaded by loadAnimImages, read by no kernel
        case PT_LAYER_INPUT_SURF_ID: return PT_OK;
        default: return fail(c, PT_ERR_UNSUPPORTED, "float2 layer %d not supported", layer);
    }
    if (layer != PT_LAYER_INPUT_SCALE) return slot_write(c, store, slot, xy, w, h, cudaMemcpyHostToDevice);
    if (!*store) TRY(dalloc_t(c, store, (size_t)c->W * c->H));
    TRY(h2d(c, *store, xy, n * sizeof(float2)));
    *slot = Arr<float2>{*store, w, h};
    return PT_OK;
}

pt_status pt_upload_image_int(pt_ctx* c, int level, int layer, const int32_t* data, int w, int h, int style) {
    if (!c || !data) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    size_t n = (size_t)w * h;
    if (layer == PT_LAYER_EXEMPLAR_OBJECT_IDS) {
        if (!c->ex || c->ex != &c->up_ex || w != c->up_ex.w || h != c->up_ex.h || style < 0 || style >= c->NS)
            return fail(c, PT_ERR_INVALID, "exemplar upload does not match pt_initialize_exemplars");
        return h2d(c, c->up_ex.ids + n * style, data, n * sizeof(int));
    }
    if (layer == PT_LAYER_INPUT_ID) {
        if (level < 0 || w != (c->W >> level) || h != (c->H >> level))
            return fail(c, PT_ERR_INVALID, "image upload %dx%d does not match level %d", w, h, level);
        if (!c->up_ids) TRY(dalloc_t(c, &c->up_ids, (size_t)c->W * c->H));
        TRY(h2d(c, c->up_ids, data, n * sizeof(int)));
        c->img.ids = Arr<int>{c->up_ids, w, h};
        return PT_OK;
    }
    return fail(c, PT_ERR_UNSUPPORTED, "int layer %d not supported", layer);
}

pt_status pt_flip_anim_buffers(pt_ctx* c) {
    if (!c) return PT_ERR_INVALID;
    c->img.cur = 1 - c->img.cur;
    return PT_OK;
}

// --- per-step compute --------------------------------------------------------

static pt_status ensure_transparency_known(pt_ctx* c) {
    if (c->ex->transparent >= 0) return PT_OK;
    CU(cudaMemsetAsync(c->flag, 0, sizeof(int), c->stream));
    LN(pt::launch_any_transparent(c->ex->out, (size_t)c->ex->w * c->ex->h, c->flag, c->stream));
    int f = 0;
    CU(cudaMemcpyAsync(&f, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->ex->transparent = f ? 1 : 0;
    return PT_OK;
}

// SynthesisFrame::createRandomPyramid, synthesisFrame.cpp:66-150, over the
// frame's colour (transparency) and orientation of `level`
static pt_status random_level(pt_ctx* c, int level, int frame, Arr<float4> rgba, Arr<float> orient);

pt_status pt_create_random_level(pt_ctx* c, int level, int frame) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    return random_level(c, level, frame, c->img.base[c->img.cur], c->img.orient);
}

static pt_status random_level(pt_ctx* c, int level, int frame, Arr<float4> rgba, Arr<float> orient) {
    int lw = c->W >> level, lh = c->H >> level;
    int mx = (c->SW >> level) - 1, my = (c->SH >> level) - 1;
    if (mx < 1 || my < 1) return fail(c, PT_ERR_INVALID, "style too small for level %d", level);
    if (!c->rnd) TRY(dalloc_t(c, &c->rnd, (size_t)c->W * c->H));
    ExView ex{c->ex->base, c->ex->out, c->ex->bo, c->ex->orient, c->ex->dt, c->ex->ids, c->ex->w, c->ex->h, c->NS};
    int mode;
    uint32_t seed = (uint32_t)(frame * level);
    if (c->params.rngMode == PT_RNG_COUNTER) {
        mode = 2;
        seed = c->params.rngSeed ^ (0x9E3779B9u * (uint32_t)(frame + 1)) ^ (0x85EBCA6Bu * (uint32_t)(level + 1));
    } else {
        TRY(ensure_transparency_known(c));
        mode = (c->params.transparencyOk || !c->ex->transparent) ? 0 : 1;
        uint32_t s0[31];
        glibc_state(seed, s0);
        size_t need = mode == 0 ? (size_t)lh * 31 : 31;
        if (need > c->states_cap) {
            dfree_t(c, c->states);
            TRY(dalloc_t(c, &c->states, need));
            c->states_cap = need;
        }
        std::vector<uint32_t> host(need);
        if (mode == 0) {
            auto it = c->jump_cache.find(lw);
            if (it == c->jump_cache.end()) it = c->jump_cache.emplace(lw, step_power(4ull * (uint64_t)lw)).first;
            const std::vector<uint32_t>& A = it->second;
            std::vector<uint32_t> s(s0, s0 + 31), t(31);
            for (int y = 0; y < lh; y++) {
                memcpy(&host[(size_t)y * 31], s.data(), 31 * sizeof(uint32_t));
                for (int i = 0; i < 31; i++) {
                    uint32_t acc = 0;
                    for (int k = 0; k < 31; k++) acc += A[i * 31 + k] * s[k];
                    t[i] = acc;
                }
                s.swap(t);
            }
        } else {
            memcpy(host.data(), s0, sizeof(s0));
        }
        CU(cudaMemcpyAsync(c->states, host.data(), need * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
        CU(cudaStreamSynchronize(c->stream));  // host vector goes out of scope
    }
    LN(pt::launch_random_level(mode, lw, lh, mx, my, c->params.transparencyOk, c->params.orientationEnabled,
                               rgba, orient, ex, c->rnd, c->states, seed, c->stream));
    c->img.rnd = Arr<float4>{c->rnd, lw, lh};
    return PT_OK;
}

pt_status pt_randomize_offsets(pt_ctx* c, int level) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (!c->img.rnd.p) return fail(c, PT_ERR_STATE, "no random level");
    PatchPlanes work;
    TRY(writable_work(c, level, &work));
    Params P = make_params(c, level);
    LN(pt::launch_random_offsets(P, work, c->stream));
    return do_sync(c, level, 0);
}

static ptk::KeyView key_view(const pt_ctx* c) {
    ptk::KeyView K{};
    K.cumul[0] = c->cumul[0];
    K.cumul[1] = c->cumul[1];
    K.w = c->cf_w;
    K.h = c->cf_h;
    K.n = c->cf_n;
    K.hw = c->params.filterMode == PT_FILTER_TEXTURE;
    return K;
}

// one propagate pass into the working buffer; a keyframe layer (key >= 0)
// or keyframe interpolation takes the generic kernels
static pt_status propagate_pass(pt_ctx* c, int level, int jump, int key = -1) {
    PatchPlanes work;
    TRY(writable_work(c, level, &work));
    Params P = make_params(c, level);
    const bool keys = c->params.interpolateKeyFrame != 0;
    return profiled(c, PT_KERNEL_PROPAGATE, P, [&](const Params& Q) {
        if (keys) return pt::launch_propagate_keys(Q, work, jump, key, key_view(c), c->stream);
        bool done = false;
        cudaError_t e = key >= 0 ? cudaSuccess : launch_tiled(c, 0, Q, work, jump, 0, nullptr, &done);
        return done ? e : pt::launch_propagate(Q, work, jump, key, c->stream);
    });
}

static pt_status scatter_pass(pt_ctx* c, int level, int key = -1) {
    bool aliased = false;
    PatchPlanes work;
    TRY(writable_work(c, level, &work, &aliased));
    Params P = make_params(c, level);
    uint32_t pass_id = c->pass_counter++;
    const bool keys = c->params.interpolateKeyFrame != 0;
    return profiled(c, PT_KERNEL_SCATTER, P, [&](const Params& Q) {
        if (keys) return pt::launch_scatter_keys(Q, work, aliased ? 1 : 0, key, key_view(c), c->stream);
        bool done = false;
        cudaError_t e = key >= 0 ? cudaSuccess : launch_tiled(c, 1, Q, work, aliased ? 1 : 0, pass_id, nullptr, &done);
        return done ? e : pt::launch_scatter(Q, work, aliased ? 1 : 0, pass_id, key, c->stream);
    });
}

pt_status pt_propagate(pt_ctx* c, int level, int jump, int key_index) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (key_index >= c->NS) return fail(c, PT_ERR_INVALID, "key index %d outside the %d style layers", key_index, c->NS);
    TRY(propagate_pass(c, level, jump, key_index));
    return do_sync(c, level, 0);
}

pt_status pt_scatter(pt_ctx* c, int level, int key_index) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (key_index >= c->NS) return fail(c, PT_ERR_INVALID, "key index %d outside the %d style layers", key_index, c->NS);
    TRY(scatter_pass(c, level, key_index));
    return do_sync(c, level, 0);
}

// --- keyframe interpolation -----------------------------------------------------

// TexSynth::initialize_cumulativeFields, texSynth_kernel.cu:2138-2142: the
// key-to-key fields, `layers` layers of w x h, zeroed
pt_status pt_initialize_cumulative_fields(pt_ctx* c, int w, int h, int layers) {
    if (!c) return PT_ERR_INVALID;
    if (w < 1 || h < 1 || layers < 1 || (long long)w * h * layers > INT32_MAX)
        return fail(c, PT_ERR_INVALID, "bad cumulative field size %dx%dx%d", w, h, layers);
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    const size_t n = (size_t)w * h * layers;
    for (int d = 0; d < 2; d++) {
        dfree_t(c, c->cumul[d]);
        TRY(dalloc_t(c, &c->cumul[d], n));
        CU(cudaMemsetAsync(c->cumul[d], 0, n * sizeof(float4), c->stream));
    }
    c->cf_w = w;
    c->cf_h = h;
    c->cf_n = layers;
    return PT_OK;
}

static pt_status ensure_ribbons(pt_ctx* c) {
    const size_t n = (size_t)c->W * c->H;
    for (int i = 0; i < 2; i++) {
        if (c->rib[i]) continue;
        TRY(dalloc_t(c, &c->rib[i], n));
        LN(pt::launch_fill_ribbons(c->rib[i], n, -1, c->stream));
    }
    return PT_OK;
}

// TexSynth::accumulateRibbonField, texSynth_kernel.cu:1830-1853
pt_status pt_accumulate_ribbon_field(pt_ctx* c, int level, int forwards, int time_step, int overwrite) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));  // unbound layers read as zero
    TRY(ensure_ribbons(c));
    Params P = make_params(c, level);
    LN(pt::launch_accumulate_ribbon(P, forwards ? 1 : 0, c->rib[1], c->rib[0], time_step, overwrite ? 1 : 0,
                                    c->stream));
    // ribbonField.copyWorkingToBase
    CU(cudaMemcpyAsync(c->rib[0], c->rib[1], (size_t)c->W * c->H * sizeof(ptk::Ribbon), cudaMemcpyDeviceToDevice,
                       c->stream));
    LN(pt::launch_ribbon_output(P, c->rib[0], c->canvas, c->adv[0].out, c->stream));
    return PT_OK;
}

// TexSynth::mergeAdvectedBuffers, texSynth_kernel.cu:2025-2042
pt_status pt_merge_advected_buffers(pt_ctx* c, int level, int merge_fallback) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (!c->img.rnd.p) return fail(c, PT_ERR_STATE, "no random level");
    PatchPlanes work;
    TRY(writable_work(c, level, &work));
    Params P = make_params(c, level);
    LN(pt::launch_merge_advected(P, merge_fallback, work, c->stream));
    return do_sync(c, level, 0);
}

// TexSynth::offsetsFromFrameToKeyRibbon, texSynth_kernel.cu:2111-2118
pt_status pt_offsets_from_frame_to_key_ribbon(pt_ctx* c, int level, int look_forwards) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (!c->img.rnd.p) return fail(c, PT_ERR_STATE, "no random level");
    PatchPlanes work;
    TRY(writable_work(c, level, &work));
    Params P = make_params(c, level);
    LN(pt::launch_frame_to_key(P, work, look_forwards ? 1 : 0, key_view(c), c->stream));
    return do_sync(c, level, 0);
}

// ribbonField.base().copyFromHost / copyToHost, workingBuffers.cpp
pt_status pt_load_ribbon_field(pt_ctx* c, int level, const pt_ribbon* rib) {
    if (!c || !rib) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    TRY(ensure_ribbons(c));
    const size_t lw = (size_t)(c->W >> level), rb = sizeof(pt_ribbon);
    return rect_copy(c, c->rib[0], c->W * rb, rib, lw * rb, lw * rb, c->H >> level, cudaMemcpyHostToDevice);
}
pt_status pt_get_ribbon_field(pt_ctx* c, int level, pt_ribbon* out) {
    if (!c || !out) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    TRY(ensure_ribbons(c));
    const size_t lw = (size_t)(c->W >> level), rb = sizeof(pt_ribbon);
    return rect_copy(c, out, lw * rb, c->rib[0], c->W * rb, lw * rb, c->H >> level, cudaMemcpyDeviceToHost);
}
// canvasOutputCache.copyFromHost (accumulateRibbon puts a keyframe there)
pt_status pt_load_canvas(pt_ctx* c, int level, const float* rgba) {
    if (!c || !rgba) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    const size_t lw = (size_t)(c->W >> level), px = sizeof(float4);
    return rect_copy(c, c->canvas, c->W * px, rgba, lw * px, lw * px, c->H >> level, cudaMemcpyHostToDevice);
}
// advectedF/B.output().copyToHost (the guide colours of accumulateRibbon)
pt_status pt_get_advected_output(pt_ctx* c, int forwards, int level, float* out) {
    if (!c || !out) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    const size_t lw = (size_t)(c->W >> level), px = sizeof(float4);
    return rect_copy(c, out, lw * px, c->adv[forwards ? 0 : 1].out, c->W * px, lw * px, c->H >> level,
                     cudaMemcpyDeviceToHost);
}

pt_status pt_upsample(pt_ctx* c, int fine_level) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, fine_level));
    bool aliased = false;
    PatchPlanes old_base = base_planes(c);
    PatchPlanes work;
    TRY(writable_work(c, fine_level, &work, &aliased));
    Params P = make_params(c, fine_level);
    float* res_out = c->res[1 - c->res_i];
    LN(pt::launch_upsample(P, work, old_base, aliased ? 1 : 0, res_out, c->stream));
    c->res_i = 1 - c->res_i;
    c->base_i = c->work_i;  // copyWorkingToBase for offsets and residual
    return PT_OK;
}

// A run that advects before any random level was drawn (TCTF's keyframe
// initialisation) reads the never-uploaded random texture: zero.
static pt_status ensure_random(pt_ctx* c) {
    if (c->img.rnd.p) return PT_OK;
    if (!c->rnd) TRY(dalloc_t(c, &c->rnd, (size_t)c->W * c->H));
    CU(cudaMemsetAsync(c->rnd, 0, sizeof(float4), c->stream));
    c->img.rnd = Arr<float4>{c->rnd, 1, 1};
    return PT_OK;
}

pt_status pt_advect_offsets(pt_ctx* c, int level, int time_step, int forwards, int flags) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (!c->img.rnd.p) return fail(c, PT_ERR_STATE, "no random level");
    int d = forwards ? 0 : 1;
    Params P = make_params(c, level);
    LN(pt::launch_advect(P, d, forwards ? 1 : 0, time_step, flags, c->stream));
    c->adv_written[d] = true;
    // dest->offsets().copyTo(offsets.base()) copies the whole buffer: outside
    // the level rectangle the base then holds the advected buffer's texels
    // (zero after a reset), which propagate's wrap can read before the next
    // full sync
    if (c->base_i == c->work_i) c->base_i = 1 - c->work_i;
    TRY(copy_planes_full(c, c->off[c->base_i], c->adv[d].off));
    c->off_span = 0;  // the two buffers may now differ anywhere
    P = make_params(c, level);
    TRY(do_sync(c, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
    if (flags & PT_ADVECT_UPDATE_RESIDUAL) TRY(do_residual(c, level));
    P = make_params(c, level);
    LN(pt::launch_copy_float(P, c->adv[d].res, c->res[c->res_i], c->stream));
    return PT_OK;
}

pt_status pt_merge_randomly(pt_ctx* c, int level, int forwards, float weight, int force_valid) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    if (!c->img.rnd.p) return fail(c, PT_ERR_STATE, "no random level");
    PatchPlanes work;
    TRY(writable_work(c, level, &work));
    Params P = make_params(c, level);
    LN(pt::launch_merge_random(P, forwards ? 0 : 1, forwards ? 1 : 0, weight, force_valid ? 1 : 0, work, c->stream));
    return do_sync(c, level, 0);
}

pt_status pt_merge_using_residual(pt_ctx* c, int level, int forwards) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    PatchPlanes work;
    TRY(writable_work(c, level, &work));
    Params P = make_params(c, level);
    LN(pt::launch_merge_residual(P, forwards ? 0 : 1, work, c->stream));
    return do_sync(c, level, 0);
}

pt_status pt_update_residual_cache(pt_ctx* c, int level) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    return do_residual(c, level);
}

pt_status pt_sync_buffers(pt_ctx* c, int level, int flags) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    return do_sync(c, level, flags);
}

// --- state transfer ------------------------------------------------------------

pt_status pt_load_offsets(pt_ctx* c, int level, const pt_patchxf* offs) {
    if (!c || !offs) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    size_t n = (size_t)(c->W >> level) * (c->H >> level);
    TRY(ensure_stage(c, n * sizeof(pt_patchxf)));
    TRY(h2d(c, c->stage, offs, n * sizeof(pt_patchxf)));
    PatchPlanes dst;
    TRY(base_for_partial_write(c, level, &dst));
    Params P = make_params(c, level);
    LN(pt::launch_unpack_patch(P, (const pt_patchxf*)c->stage, dst, c->stream));
    return PT_OK;
}

pt_status pt_load_residual(pt_ctx* c, int level, const float* res) {
    if (!c || !res) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    size_t n = (size_t)(c->W >> level) * (c->H >> level);
    TRY(ensure_stage(c, n * sizeof(float)));
    TRY(h2d(c, c->stage, res, n * sizeof(float)));
    Params P = make_params(c, level);
    LN(pt::launch_load_residual(P, (const float*)c->stage, c->res[c->res_i], c->stream));
    return PT_OK;
}

pt_status pt_get_offsets(pt_ctx* c, int level, pt_patchxf* out) {
    if (!c || !out) return PT_ERR_INVALID;
    TRY(check_ready(c, level, false, false));
    size_t n = (size_t)(c->W >> level) * (c->H >> level);
    TRY(ensure_stage(c, n * sizeof(pt_patchxf)));
    Params P = make_params(c, level);
    LN(pt::launch_pack_patch(P, base_planes(c), (pt_patchxf*)c->stage, c->stream));
    CU(cudaMemcpyAsync(out, c->stage, n * sizeof(pt_patchxf), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

static pt_status get_plane(pt_ctx* c, int level, const float* src, int ch, float* out) {
    TRY(check_ready(c, level, false, false));
    size_t n = (size_t)(c->W >> level) * (c->H >> level) * ch;
    TRY(ensure_stage(c, n * sizeof(float)));
    Params P = make_params(c, level);
    LN(pt::launch_gather_level(P, src, ch, (float*)c->stage, c->stream));
    CU(cudaMemcpyAsync(out, c->stage, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

pt_status pt_get_residual(pt_ctx* c, int level, float* out) {
    if (!c || !out) return PT_ERR_INVALID;
    return get_plane(c, level, c->res[c->res_i], 1, out);
}

pt_status pt_get_output(pt_ctx* c, int level, float* out) {
    if (!c || !out) return PT_ERR_INVALID;
    return get_plane(c, level, (const float*)c->canvas, 4, out);
}


pt_status pt_gaussian_kernel(int radius, int normalize, float* out) {
    if (!out || radius < 0 || radius > ptk::kMaxRadius) return PT_ERR_INVALID;
    pt::gaussian_weights(radius, normalize != 0, out);
    return PT_OK;
}

pt_status pt_convolve_separable(pt_ctx* c, const float* src, float* dst, int w, int h, int pitch, int radius) {
    if (!c || !src || !dst) return PT_ERR_INVALID;
    if (w < 1 || h < 1 || pitch < w || radius < 1 || radius > ptk::kMaxRadius)
        return fail(c, PT_ERR_INVALID, "bad convolution size %dx%d pitch %d radius %d", w, h, pitch, radius);
    CU(cudaSetDevice(c->device));
    size_t n = (size_t)pitch * h;
    if (n > c->conv_scratch_elems) {
        dfree_t(c, c->conv_scratch);
        c->conv_scratch_elems = 0;
        TRY(dalloc_t(c, &c->conv_scratch, n));
        c->conv_scratch_elems = n;
    }
    ConvKernel k;
    k.r = radius;
    pt::gaussian_weights(radius, true, k.w);
    LN(pt::launch_conv(src, c->conv_scratch, w, h, pitch, 1, k, c->stream));
    LN(pt::launch_conv(c->conv_scratch, dst, w, h, pitch, 0, k, c->stream));
    return PT_OK;
}

// --- resident pyramids ----------------------------------------------------------

// builds the float pyramid of `ch` channels from a device level-0 array;
// returns per-level device arrays (level 0 is `src` itself)
static pt_status build_avg(pt_ctx* c, float* src, int w, int h, int ch, int vel, int nlev, std::vector<float*>& out) {
    out.assign(nlev, nullptr);
    out[0] = src;
    for (int l = 1; l < nlev; l++) {
        int pw = w >> (l - 1), ph = h >> (l - 1);
        TRY(dalloc_t(c, &out[l], (size_t)(pw >> 1) * (ph >> 1) * ch));
        LN(pt::launch_down_avg(out[l - 1], pw, ph, ch, vel, out[l], c->stream));
    }
    return PT_OK;
}
static pt_status build_vote(pt_ctx* c, int* src, int w, int h, int nlev, std::vector<int*>& out) {
    out.assign(nlev, nullptr);
    out[0] = src;
    for (int l = 1; l < nlev; l++) {
        int pw = w >> (l - 1), ph = h >> (l - 1);
        TRY(dalloc_t(c, &out[l], (size_t)(pw >> 1) * (ph >> 1)));
        LN(pt::launch_down_vote(out[l - 1], pw, ph, out[l], c->stream));
    }
    return PT_OK;
}
template <class T>
static pt_status upload_or_fill(pt_ctx* c, T** dst, const void* src, size_t n, int ch, float fill) {
    TRY(dalloc_t(c, dst, n * ch));
    if (src) return h2d(c, *dst, src, n * ch * sizeof(T));
    if (fill != 0.0f) {
        std::vector<T> tmp(n * ch, (T)fill);
        TRY(h2d(c, *dst, tmp.data(), n * ch * sizeof(T)));
        CU(cudaStreamSynchronize(c->stream));
    }
    return PT_OK;
}
static pt_status orientation_pyramid(pt_ctx* c, const float* tensor, int w, int h, int nlev, std::vector<float*>& out) {
    float* t0 = nullptr;
    TRY(upload_or_fill(c, &t0, tensor, (size_t)w * h, 3, 0.0f));
    std::vector<float*> tens;
    TRY(build_avg(c, t0, w, h, 3, 0, nlev, tens));
    out.assign(nlev, nullptr);
    for (int l = 0; l < nlev; l++) {
        int n = (w >> l) * (h >> l);
        TRY(dalloc_t(c, &out[l], (size_t)n));
        LN(pt::launch_tensor_angle(tens[l], n, out[l], c->stream));
    }
    CU(cudaStreamSynchronize(c->stream));
    for (auto p : tens) dfree_t(c, p);
    return PT_OK;
}

pt_status pt_set_style(pt_ctx* c, int style, int w, int h, const float* base, const float* output,
                       const float* orient_tensor, const float* dist_trans, const int32_t* ids) {
    if (!c || !base || !output) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    if (style < 0 || style >= c->NS) return fail(c, PT_ERR_INVALID, "style %d out of range", style);
    if (w != c->SW || h != c->SH)
        return fail(c, PT_ERR_UNSUPPORTED, "style %dx%d differs from the initialized style size %dx%d", w, h, c->SW,
                    c->SH);
    int nlev = level_count(w, h);
    if ((int)c->style_levels.size() != nlev || c->style_levels[0].w != w || c->style_levels[0].h != h) {
        for (auto& L : c->style_levels) {
            dfree_t(c, L.base); dfree_t(c, L.out); dfree_t(c, L.bo); dfree_t(c, L.orient); dfree_t(c, L.dt);
            dfree_t(c, L.ids);
            free_textures(c, &L);
        }
        c->style_levels.assign(nlev, ExLevel());
        for (int l = 0; l < nlev; l++) {
            ExLevel& L = c->style_levels[l];
            L.w = w >> l;
            L.h = h >> l;
            size_t n = (size_t)L.w * L.h * c->NS;
            TRY(dalloc_t(c, &L.base, n));
            TRY(dalloc_t(c, &L.out, n));
            TRY(dalloc_t(c, &L.bo, 2 * n));
            TRY(dalloc_t(c, &L.orient, n));
            TRY(dalloc_t(c, &L.dt, n));
            TRY(dalloc_t(c, &L.ids, n));
        }
        c->style_set.assign(c->NS, 0);
    }
    size_t n0 = (size_t)w * h;
    float *b0 = nullptr, *o0 = nullptr, *d0 = nullptr;
    int* i0 = nullptr;
    TRY(upload_or_fill(c, &b0, base, n0, 4, 0.f));
    TRY(upload_or_fill(c, &o0, output, n0, 4, 0.f));
    TRY(upload_or_fill(c, &d0, dist_trans, n0, 1, 0.f));
    TRY(upload_or_fill(c, &i0, ids, n0, 1, 0.f));
    std::vector<float*> pb, po, pd, por;
    std::vector<int*> pi;
    TRY(build_avg(c, b0, w, h, 4, 0, nlev, pb));
    TRY(build_avg(c, o0, w, h, 4, 0, nlev, po));
    TRY(build_avg(c, d0, w, h, 1, 0, nlev, pd));
    TRY(build_vote(c, i0, w, h, nlev, pi));
    TRY(orientation_pyramid(c, orient_tensor, w, h, nlev, por));
    for (int l = 0; l < nlev; l++) {
        ExLevel& L = c->style_levels[l];
        size_t n = (size_t)L.w * L.h;
        CU(cudaMemcpyAsync(L.base + n * style, pb[l], n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
        CU(cudaMemcpyAsync(L.out + n * style, po[l], n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
        CU(cudaMemcpyAsync(L.orient + n * style, por[l], n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
        CU(cudaMemcpyAsync(L.dt + n * style, pd[l], n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
        CU(cudaMemcpyAsync(L.ids + n * style, pi[l], n * sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
        L.transparent = -1;
        L.bo_stale = true;
        L.tex_stale = true;
    }
    CU(cudaStreamSynchronize(c->stream));
    for (int l = 0; l < nlev; l++) {
        dfree_t(c, pb[l]); dfree_t(c, po[l]); dfree_t(c, pd[l]); dfree_t(c, pi[l]); dfree_t(c, por[l]);
    }
    c->style_set[style] = 1;
    return PT_OK;
}

pt_status pt_set_frame(pt_ctx* c, int frame, int w, int h, const float* rgba, const float* orient_tensor,
                       const float* dist_trans, const int32_t* ids, const float* vel_fwd, const float* vel_bwd,
                       const float* scale) {
    if (!c || !rgba) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    if (w != c->W || h != c->H) return fail(c, PT_ERR_INVALID, "frame %dx%d differs from image size", w, h);
    auto it = c->frames.find(frame);
    if (it != c->frames.end()) {
        for (auto& L : it->second) {
            dfree_t(c, L.rgba); dfree_t(c, L.orient); dfree_t(c, L.dt); dfree_t(c, L.ids);
            dfree_t(c, L.velf); dfree_t(c, L.velb); dfree_t(c, L.scale);
        }
        c->frames.erase(it);
    }
    int nlev = level_count(w, h);
    size_t n0 = (size_t)w * h;
    float *c0, *d0, *vf0, *vb0, *s0;
    int* i0;
    TRY(upload_or_fill(c, &c0, rgba, n0, 4, 0.f));
    TRY(upload_or_fill(c, &d0, dist_trans, n0, 1, 0.f));
    TRY(upload_or_fill(c, &i0, ids, n0, 1, 0.f));
    TRY(upload_or_fill(c, &vf0, vel_fwd, n0, 2, 0.f));
    TRY(upload_or_fill(c, &vb0, vel_bwd, n0, 2, 0.f));
    TRY(upload_or_fill(c, &s0, scale, n0, 2, 1.f));
    std::vector<float*> pc, pd, pvf, pvb, ps, por;
    std::vector<int*> pi;
    TRY(build_avg(c, c0, w, h, 4, 0, nlev, pc));
    TRY(build_avg(c, d0, w, h, 1, 0, nlev, pd));
    TRY(build_avg(c, vf0, w, h, 2, 1, nlev, pvf));
    TRY(build_avg(c, vb0, w, h, 2, 1, nlev, pvb));
    TRY(build_avg(c, s0, w, h, 2, 0, nlev, ps));
    TRY(build_vote(c, i0, w, h, nlev, pi));
    TRY(orientation_pyramid(c, orient_tensor, w, h, nlev, por));
    std::vector<FrameLevel> lv(nlev);
    for (int l = 0; l < nlev; l++) {
        FrameLevel& L = lv[l];
        L.w = w >> l;
        L.h = h >> l;
        L.rgba = (float4*)pc[l];
        L.dt = pd[l];
        L.velf = (float2*)pvf[l];
        L.velb = (float2*)pvb[l];
        L.scale = (float2*)ps[l];
        L.ids = pi[l];
        L.orient = por[l];
    }
    c->frames[frame] = std::move(lv);
    return PT_OK;
}

// Ribbon inputs of time step `step` (2, 4, 8 ...): the velocities from the
// frame to the frame `step` later (vel_fwd) and earlier (vel_bwd), pyramids
// built as the velocities' (DOWNSAMPLE_SCALE_WITH_LEVELS)
pt_status pt_set_frame_ribbons(pt_ctx* c, int frame, int step, int w, int h, const float* vel_fwd,
                               const float* vel_bwd) {
    if (!c || !vel_fwd || !vel_bwd) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "pt_initialize has not been called");
    if (w != c->W || h != c->H) return fail(c, PT_ERR_INVALID, "ribbons %dx%d differ from image size", w, h);
    if (step < 2 || (step & (step - 1))) return fail(c, PT_ERR_INVALID, "ribbon step %d is not a power of two > 1", step);
    const auto key = std::make_pair(frame, step);
    auto it = c->ribbons.find(key);
    if (it != c->ribbons.end()) {
        for (auto& L : it->second) {
            dfree_t(c, L.first); dfree_t(c, L.second);
        }
        c->ribbons.erase(it);
    }
    const int nlev = level_count(w, h);
    const size_t n0 = (size_t)w * h;
    float *vf0, *vb0;
    TRY(upload_or_fill(c, &vf0, vel_fwd, n0, 2, 0.f));
    TRY(upload_or_fill(c, &vb0, vel_bwd, n0, 2, 0.f));
    std::vector<float*> pvf, pvb;
    TRY(build_avg(c, vf0, w, h, 2, 1, nlev, pvf));
    TRY(build_avg(c, vb0, w, h, 2, 1, nlev, pvb));
    std::vector<std::pair<float2*, float2*>> lv(nlev);
    for (int l = 0; l < nlev; l++) lv[l] = std::make_pair((float2*)pvf[l], (float2*)pvb[l]);
    c->ribbons[key] = std::move(lv);
    return PT_OK;
}

pt_status pt_clear_frames(pt_ctx* c) {
    if (!c) return PT_ERR_INVALID;
    CU(cudaStreamSynchronize(c->stream));
    free_frames(c);
    return PT_OK;
}

// --- measurement ----------------------------------------------------------------

pt_status pt_timer_record(pt_ctx* c, int slot) {
    if (!c || slot < 0 || slot >= PT_TIMER_SLOTS) return PT_ERR_INVALID;
    if (!c->timers[slot]) CU(cudaEventCreate(&c->timers[slot]));
    CU(cudaEventRecord(c->timers[slot], c->stream));
    return PT_OK;
}

pt_status pt_timer_elapsed(pt_ctx* c, int a, int b, float* ms) {
    if (!c || !ms || a < 0 || b < 0 || a >= PT_TIMER_SLOTS || b >= PT_TIMER_SLOTS) return PT_ERR_INVALID;
    if (!c->timers[a] || !c->timers[b]) return fail(c, PT_ERR_STATE, "timer slot not recorded");
    CU(cudaEventSynchronize(c->timers[b]));
    CU(cudaEventElapsedTime(ms, c->timers[a], c->timers[b]));
    return PT_OK;
}

static void clear_profile(pt_ctx* c) {
    for (auto& v : c->ev_pairs) {
        for (auto& pr : v) {
            c->ev_pool.push_back(pr.first);
            c->ev_pool.push_back(pr.second);
        }
        v.clear();
    }
}

pt_status pt_set_profiling(pt_ctx* c, int flags) {
    if (!c || (flags & ~(PT_PROFILE_TIMING | PT_PROFILE_COUNTERS))) return PT_ERR_INVALID;
    CU(cudaStreamSynchronize(c->stream));
    clear_profile(c);
    if (!c->counters) TRY(dalloc_t(c, &c->counters, 3 * PT_KERNEL_COUNT));
    CU(cudaMemsetAsync(c->counters, 0, 3 * PT_KERNEL_COUNT * sizeof(unsigned long long), c->stream));
    c->profiling = flags;
    return PT_OK;
}

pt_status pt_set_tiled_kernels(pt_ctx* c, int on) {
    if (!c) return PT_ERR_INVALID;
    c->use_tiled = on != 0;
    return PT_OK;
}

pt_status pt_set_incremental(pt_ctx* c, int on) {
    if (!c) return PT_ERR_INVALID;
    c->use_incremental = on != 0;
    return PT_OK;
}

pt_status pt_get_kernel_stats(pt_ctx* c, int kernel, pt_kernel_stats* out) {
    if (!c || !out || kernel < 0 || kernel >= PT_KERNEL_COUNT) return PT_ERR_INVALID;
    CU(cudaStreamSynchronize(c->stream));
    memset(out, 0, sizeof(*out));
    for (auto& pr : c->ev_pairs[kernel]) {
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, pr.first, pr.second));
        out->total_ms += ms;
        out->launches++;
    }
    if (c->counters) {
        unsigned long long h[3] = {0, 0, 0};
        CU(cudaMemcpy(h, c->counters + 3 * kernel, sizeof(h), cudaMemcpyDeviceToHost));
        out->energy_evals = h[0];
        out->taps = h[1];
        out->temporal_taps = h[2];
    }
    return PT_OK;
}

// --- driver -------------------------------------------------------------------

// Style::load(level), style.cpp:62-140 (a pointer switch to the resident level)
static pt_status bind_style_level(pt_ctx* c, int level) {
    if (level >= (int)c->style_levels.size()) return fail(c, PT_ERR_INVALID, "style pyramid too shallow");
    for (int s = 0; s < c->NS; s++)
        if (!c->style_set[s]) return fail(c, PT_ERR_STATE, "style %d not set", s);
    c->ex = &c->style_levels[level];
    return refresh_interleaved(c, c->ex);
}

static void bind_frame_keys(pt_ctx* c, int frame, int level);

// SynthesisFrame::loadImages + loadAnimImages, synthesisFrame.cpp:562-656
static pt_status frame_level(pt_ctx* c, int frame, int level, const FrameLevel** out) {
    auto it = c->frames.find(frame);
    if (it == c->frames.end()) return fail(c, PT_ERR_STATE, "frame %d not set", frame);
    if (level >= (int)it->second.size()) return fail(c, PT_ERR_INVALID, "frame pyramid too shallow");
    *out = &it->second[level];
    return PT_OK;
}
// SynthesisFrame::loadImages, synthesisFrame.cpp:562-580: the colour into
// the current layer, orientation and ids
//
// While levels run coarse to fine (FMBM, FBMO) a layer's texels outside the
// current rectangle were never written, so the level's own array is bound
// (reads there give zero, as from the zeroed layered array).  The IND scheme
// visits a coarse level after a finer one: it copies into the full-size
// layered arrays as the reference's uploads do (`slot_copy`).
static pt_status bind_frame_images(pt_ctx* c, int frame, int level) {
    const FrameLevel* L;
    TRY(frame_level(c, frame, level, &L));
    if (c->slot_copy) {
        TRY(slot_write(c, &c->up_base[c->img.cur], &c->img.base[c->img.cur], L->rgba, L->w, L->h,
                       cudaMemcpyDeviceToDevice));
    } else {
        c->img.base[c->img.cur] = Arr<float4>{L->rgba, L->w, L->h};
    }
    c->img.orient = Arr<float>{L->orient, L->w, L->h};
    c->img.ids = Arr<int>{L->ids, L->w, L->h};
    return PT_OK;
}
// SynthesisFrame::loadAnimImages, synthesisFrame.cpp:583-656: velocities and
// distance transform into the current layer, scale
static pt_status bind_frame_anim(pt_ctx* c, int frame, int level, int time_step = 1) {
    const FrameLevel* L0;
    TRY(frame_level(c, frame, level, &L0));
    FrameLevel Ls = *L0;  // loadAnimImages with time_step > 1 takes the ribbons of that step
    if (time_step > 1) {
        auto it = c->ribbons.find(std::make_pair(frame, time_step));
        if (it == c->ribbons.end() || level >= (int)it->second.size())
            return fail(c, PT_ERR_STATE, "frame %d has no ribbons of step %d", frame, time_step);
        Ls.velf = it->second[level].first;
        Ls.velb = it->second[level].second;
    }
    const FrameLevel* L = &Ls;
    int cur = c->img.cur;
    if (c->slot_copy) {
        const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
        TRY(slot_write(c, &c->up_dt[cur], &c->img.dt[cur], L->dt, L->w, L->h, d2d));
        TRY(slot_write(c, &c->up_velf[cur], &c->img.velf[cur], L->velf, L->w, L->h, d2d));
        TRY(slot_write(c, &c->up_velb[cur], &c->img.velb[cur], L->velb, L->w, L->h, d2d));
    } else {
        c->img.dt[cur] = Arr<float>{L->dt, L->w, L->h};
        c->img.velf[cur] = Arr<float2>{L->velf, L->w, L->h};
        c->img.velb[cur] = Arr<float2>{L->velb, L->w, L->h};
    }
    c->img.scale = Arr<float2>{L->scale, L->w, L->h};
    if (c->keyed) bind_frame_keys(c, frame, level);
    return PT_OK;
}
static pt_status bind_frame_level(pt_ctx* c, int frame, int level, int time_step = 1) {
    TRY(bind_frame_images(c, frame, level));
    return bind_frame_anim(c, frame, level, time_step);
}

static pt_status store_save(pt_ctx* c, int level, int frame, int pass, bool with_canvas) {
    StoreEntry& e = c->store[std::make_tuple(level, frame, pass)];
    int lw = c->W >> level, lh = c->H >> level;
    size_t n = (size_t)lw * lh;
    if (!e.offs || e.w != lw || e.h != lh) {
        dfree_t(c, e.offs); dfree_t(c, e.res); dfree_t(c, e.canvas);
        TRY(dalloc_t(c, &e.offs, n));
        TRY(dalloc_t(c, &e.res, n));
        e.w = lw;
        e.h = lh;
    }
    Params P = make_params(c, level);
    LN(pt::launch_pack_patch(P, base_planes(c), e.offs, c->stream));
    LN(pt::launch_gather_level(P, c->res[c->res_i], 1, e.res, c->stream));
    if (with_canvas) {
        if (!e.canvas) TRY(dalloc_t(c, &e.canvas, n));
        LN(pt::launch_gather_level(P, (const float*)c->canvas, 4, (float*)e.canvas, c->stream));
    }
    return PT_OK;
}

static pt_status store_load_offsets(pt_ctx* c, int level, int frame, int pass) {
    auto it = c->store.find(std::make_tuple(level, frame, pass));
    if (it == c->store.end()) return fail(c, PT_ERR_STATE, "no saved offsets for level %d frame %d pass %d", level, frame, pass);
    PatchPlanes dst;
    TRY(base_for_partial_write(c, level, &dst));
    Params P = make_params(c, level);
    LN(pt::launch_unpack_patch(P, it->second.offs, dst, c->stream));
    return PT_OK;
}
static pt_status store_load_residual(pt_ctx* c, int level, int frame, int pass) {
    auto it = c->store.find(std::make_tuple(level, frame, pass));
    if (it == c->store.end()) return fail(c, PT_ERR_STATE, "no saved residual");
    Params P = make_params(c, level);
    LN(pt::launch_load_residual(P, it->second.res, c->res[c->res_i], c->stream));
    return PT_OK;
}
// SynthesisFrame::saveImages, synthesisFrame.cpp:758-767: saved and
// remembered as the frame's last saved pass of the level
static pt_status save_images(pt_ctx* c, int level, int frame, int pass, bool with_canvas) {
    TRY(store_save(c, level, frame, pass, with_canvas));
    c->last_saved[std::make_pair(frame, level)] = pass;
    return PT_OK;
}

// SynthesisFrame::loadLastSavedOffsets, synthesisFrame.cpp:769-772: the
// frame's last pass saved through saveImages (0 before any, the reference's
// zero-filled vector); a pass that was never saved leaves the base offsets
// as they are (WorkingBuffers::loadOffsets fails on the missing file)
static pt_status load_last_saved_offsets(pt_ctx* c, int frame, int level) {
    auto it = c->last_saved.find(std::make_pair(frame, level));
    const int pass = it == c->last_saved.end() ? 0 : it->second;
    if (!c->store.count(std::make_tuple(level, frame, pass))) return PT_OK;
    return store_load_offsets(c, level, frame, pass);
}

// SynthesisFrame::propagateAndScatter, synthesisFrame.cpp:483-508
//
// With change tracking (tiled kernels), every pass of the loop is numbered.
// Within the loop nothing but the offsets changes (the levels' images, the
// advected buffers and the parameters are fixed, and the offsets histogram
// is all zero), so a pixel's residual depends only on the offset records in
// its patch window, and a candidate's outcome only on its source record, the
// target pixel's window and the target's residual.  A pass with the same
// candidates as an earlier pass of the loop (the same propagate jump, or the
// next scatter when its candidates are drawn with the reference's
// generator) therefore skips every candidate whose inputs are unchanged
// since then: it was rejected there against the same residual and would be
// rejected again.  The sync after a pass recomputes only the canvas and
// residuals whose inputs changed.  Results are bit-identical either way.
//
// `residual_fresh`: the residual cache holds the residuals of the base
// offsets.  synthesizeInterpolated syncs without updating it, so its first
// propagate pass compares against the residuals left by earlier steps, as
// the reference's does; that pass then runs untracked and its sync computes
// every residual and tap value.
//
// With keyframe interpolation every iteration starts with a jump-0 pass and
// all passes carry the frame's key index (-1 if it is not a key).
static pt_status propagate_and_scatter(pt_ctx* c, int level, int iterations, bool residual_fresh = true,
                                       int key = -1) {
    const bool track = c->use_incremental && tiled_usable(c);
    bool fill_after_first = false;
    if (track) {
        // the per-tap values of every residual, recomputed in full once
        const int r = c->params.residualWindowSize, K = (2 * r + 1) * (2 * r + 1);
        if (c->tap_cache_k < K) {
            dfree_t(c, c->tap_cache);
            c->tap_cache_k = 0;
            TRY(dalloc_t(c, &c->tap_cache, (size_t)K * c->W * c->H));
            c->tap_cache_k = K;
        }
        if (residual_fresh) {
            c->inc_fill = 1;
            pt_status st = do_residual(c, level);
            c->inc_fill = 0;
            TRY(st);
        } else {
            fill_after_first = true;
        }
    }
    std::map<int, int> last_pass;  // jump (0 = scatter) -> index of its last pass
    auto run = [&](int jump) -> pt_status {
        if (fill_after_first) {
            fill_after_first = false;
            c->inc_fill = 1;
            pt_status st = pt_propagate(c, level, jump, key);
            c->inc_fill = 0;
            return st;
        }
        if (track) {
            c->inc_on = 1;
            c->inc_pi = ++c->inc_seq;
            auto it = last_pass.find(jump);
            bool same = it != last_pass.end() && (jump != 0 || c->params.rngMode != PT_RNG_COUNTER);
            c->inc_prev = same ? it->second : INT_MIN;
            last_pass[jump] = c->inc_pi;
        }
        pt_status st = jump ? pt_propagate(c, level, jump, key) : pt_scatter(c, level, key);
        c->inc_on = 0;
        c->inc_prev = INT_MIN;
        return st;
    };
    for (int itr = 0; itr < iterations; itr++) {
        if (c->keyed) TRY(pt_propagate(c, level, 0, key));
        for (int j = 128; j > 1; j /= 2) TRY(run(j));
        TRY(run(1));
        TRY(run(1));
        if (itr < iterations - 1) TRY(run(0));
    }
    return PT_OK;
}

// SynthesisFrame::synthesizeConsecutive, synthesisFrame.cpp:214-323
// DataAccess::keyFrameIndices().indexOf(frame): the key's full index
static int key_full_index(const pt_ctx* c, int frame) {
    for (size_t i = 0; i < c->key_frames.size(); i++)
        if (c->key_frames[i] == frame) return (int)i;
    return -1;
}
// Style::keyFrameSubrangeIndex, style.cpp:198-205
static int key_sub_index(const pt_ctx* c, int frame) {
    for (size_t i = 0; i < c->key_sub.size(); i++)
        if (c->key_sub[i] == frame) return (int)i;
    return -1;
}
// Style::keyFrameAdvectWeight, style.cpp:207-223
static float key_advect_weight(const pt_ctx* c, int frame, bool forwards) {
    const std::vector<int>& K = c->key_sub;
    int prev_key = -1;
    while (prev_key < (int)K.size() - 1 && frame > K[prev_key + 1]) prev_key++;
    const bool has_prev = prev_key >= 0, has_next = prev_key < (int)K.size() - 1;
    const int prev_frame = has_prev ? K[prev_key] : c->run_first;
    const int next_frame = has_next ? K[prev_key + 1] : c->run_last;
    if (forwards) return has_next ? float(next_frame - frame) / float(next_frame - prev_frame) : 1.0f;
    return has_prev ? float(frame - prev_frame) / float(next_frame - prev_frame) : 1.0f;
}

// SynthesisFrame::createRandomPyramid with setupWithKeys
// (synthesisFrame.cpp:66-150): the glibc stream of srand(frame*level), each
// pixel drawing its key layer first; one GPU thread walks the stream.
static pt_status random_level_keyed(pt_ctx* c, int level, int frame, Arr<float4> rgba, Arr<float> orient) {
    TRY(check_ready(c, level));
    const int lw = c->W >> level, lh = c->H >> level;
    const int mx = (c->SW >> level) - 1, my = (c->SH >> level) - 1;
    if (mx < 1 || my < 1) return fail(c, PT_ERR_INVALID, "style too small for level %d", level);
    if (!c->rnd) TRY(dalloc_t(c, &c->rnd, (size_t)c->W * c->H));
    if (c->states_cap < 31) {
        dfree_t(c, c->states);
        TRY(dalloc_t(c, &c->states, (size_t)31));
        c->states_cap = 31;
    }
    uint32_t s0[31];
    glibc_state((uint32_t)(frame * level), s0);
    CU(cudaMemcpyAsync(c->states, s0, sizeof(s0), cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    ExView ex{c->ex->base, c->ex->out, c->ex->bo, c->ex->orient, c->ex->dt, c->ex->ids, c->ex->w, c->ex->h, c->NS};
    const int nk = (int)c->key_sub.size(), first_key = key_full_index(c, c->key_sub.front());
    LN(pt::launch_random_level_keys(lw, lh, mx, my, c->params.transparencyOk, c->params.orientationEnabled, rgba,
                                    orient, ex, c->rnd, c->states, nk, first_key, c->stream));
    c->img.rnd = Arr<float4>{c->rnd, lw, lh};
    return PT_OK;
}

static pt_status synthesize_consecutive(pt_ctx* c, const pt_params& user, int frame, int level, int pass,
                                        bool is_first, bool forwards, int source_pass, bool first_pass,
                                        bool save_canvas, int time_step = 1) {
    pt_params p = user;  // SynthesisFrame::updateParameters, :522-542
    p.advectionJitter = (frame % 3 == 0) ? user.advectionJitter * 0.01f : 0.0f;
    p.direction = forwards ? PT_FORWARD : PT_BACKWARD;
    TRY(pt_set_params(c, &p));
    bool rm = user.scheme == PT_S_FMBM_RM;
    int ops = (c->keyed ? PT_ADVECT_CHECK_FRAME_TO_KEY : 0) | (rm ? 0 : PT_ADVECT_UPDATE_RESIDUAL);
    bool coarsest = level == user.levels - 1;
    // SynthesisFrame::mergeRandomly, :510-520
    const float advect_weight = c->keyed ? key_advect_weight(c, frame, forwards) : 0.5f;
    if (first_pass) {
        if (c->keyed) TRY(random_level_keyed(c, level, frame, c->img.base[c->img.cur], c->img.orient));
        else TRY(pt_create_random_level(c, level, frame));
        if (is_first) {
            if (coarsest) {
                if (c->keyed) TRY(pt_offsets_from_frame_to_key_ribbon(c, level, forwards));
                else TRY(pt_randomize_offsets(c, level));
            } else {
                TRY(store_load_offsets(c, level + 1, frame, source_pass));
                TRY(pt_upsample(c, level));
                TRY(do_sync(c, level, 0));
            }
        }
        if (!is_first && coarsest) {
            TRY(pt_advect_offsets(c, level, time_step, forwards, ops));
            c->work_i = c->base_i;  // copyBaseToWorking
        } else if (!is_first) {
            TRY(pt_advect_offsets(c, level, time_step, forwards, ops | PT_ADVECT_IGNORE_RANDOM));
            TRY(store_load_offsets(c, level + 1, frame, source_pass));
            TRY(store_load_residual(c, level + 1, frame, source_pass));
            TRY(pt_upsample(c, level));
            TRY(do_sync(c, level, 0));
            if (rm) TRY(pt_merge_randomly(c, level, forwards, advect_weight, 0));
            else TRY(pt_merge_using_residual(c, level, forwards));
        }
    } else {
        TRY(pt_advect_offsets(c, level, time_step, forwards, ops | PT_ADVECT_IGNORE_RANDOM));
        TRY(store_load_offsets(c, level, frame, pass - 1));
        TRY(store_load_residual(c, level, frame, pass - 1));
        TRY(do_sync(c, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
        if (rm) TRY(pt_merge_randomly(c, level, forwards, advect_weight, 0));
        else TRY(pt_merge_using_residual(c, level, forwards));
    }
    TRY(do_sync(c, level, 0));
    TRY(propagate_and_scatter(c, level, user.iterations, true, c->keyed ? key_full_index(c, frame) : -1));
    return save_images(c, level, frame, pass, save_canvas);
}

// SynthesisProcessor::renderAnimationFMBM + renderConsecutivePass,
// synthesisProcessor.cpp:703-753,846-878
// frees the saved states of `level`
static void drop_store_level(pt_ctx* c, int level) {
    for (auto it = c->store.begin(); it != c->store.end();) {
        if (std::get<0>(it->first) == level) {
            dfree_t(c, it->second.offs); dfree_t(c, it->second.res); dfree_t(c, it->second.canvas);
            it = c->store.erase(it);
        } else {
            ++it;
        }
    }
}

static pt_status upload_key_fields(pt_ctx* c, int level);

// SynthesisProcessor::renderAnimationIND, synthesisProcessor.cpp:807-844:
// every frame synthesised on its own, coarse to fine, each pass through
// synthesizeConsecutive as a first frame going forwards
static pt_status render_ind(pt_ctx* c, int first, int last, bool fresh) {
    const pt_params user = c->params;
    if (fresh) {
        TRY(reset_working(c));
        TRY(reset_image_slots(c));
        free_store(c);
    }
    struct SlotCopy {  // frame binds copy into the layered arrays for this run
        pt_ctx* c;
        bool was;
        explicit SlotCopy(pt_ctx* x) : c(x), was(x->slot_copy) { c->slot_copy = true; }
        ~SlotCopy() { c->slot_copy = was; }
    } slot_copy(c);
    const int total = user.fixupPasses + 1;
    const int final_pass = (user.finalLevel == 0) ? total - 1 : 0;
    c->out_level = user.finalLevel;
    c->out_pass = final_pass;
    for (int f = first; f <= last; f++) {
        for (int level = user.levels - 1; level >= user.finalLevel; level--) {
            TRY(bind_style_level(c, level));
            if (c->keyed) TRY(upload_key_fields(c, level));
            TRY(pt_reset_advected_buffers(c));
            for (int pass = 0; pass < total; pass++) {
                const bool save_canvas = (level == user.finalLevel && pass == final_pass);
                TRY(bind_frame_level(c, f, level));
                TRY(synthesize_consecutive(c, user, f, level, pass, true, true, pass, pass == 0, save_canvas));
            }
            // the coarser level is no longer needed (earlier frames are done)
            if (level + 1 < user.levels) drop_store_level(c, level + 1);
        }
    }
    c->params = user;
    return PT_OK;
}

// WorkingBuffers, as renderAnimationFBMO uses them
// (synthesisProcessor.cpp:979-980): the base offsets and residual copied
// whole into the advected buffers of `forwards`
pt_status pt_copy_offsets_to_advected(pt_ctx* c, int forwards) {
    if (!c) return PT_ERR_INVALID;
    if (!c->initialized) return fail(c, PT_ERR_STATE, "context not initialized");
    const int d = forwards ? 0 : 1;
    TRY(copy_planes_full(c, c->adv[d].off, base_planes(c)));
    CU(cudaMemcpyAsync(c->adv[d].res, c->res[c->res_i], (size_t)c->W * c->H * sizeof(float),
                       cudaMemcpyDeviceToDevice, c->stream));
    c->adv_written[d] = true;
    return PT_OK;
}

// SynthesisFrame::advectNeighbors, synthesisFrame.cpp:325-382: the
// neighbours' last saved offsets advected into this frame (the neighbour's
// images in the current layer, then this frame's velocities in the other).
// Neighbours are the frames of the synthesised range.
// With keys, a side without a neighbour advects this frame's frame-to-key
// ribbons instead (ADVECT_DO_NOT_CHECK_PREVIOUS).  `neighbours` false: the
// refine of TCTF's initialisation pass, which is given none.
static pt_status advect_neighbors(pt_ctx* c, int frame, int level, int source_pass, int first, int last,
                                  bool neighbours = true, int ts = 1) {
    TRY(pt_reset_advected_buffers(c));
    const pt_params& p = c->params;
    const int ops = c->keyed ? PT_ADVECT_CHECK_FRAME_TO_KEY : 0;
    const bool has_prior = neighbours && frame - ts >= first, has_next = neighbours && frame + ts <= last;
    const bool temporal = p.timeDerivativeInputWeight > 0.f || p.timeDerivativeOutputWeight > 0.f ||
                          p.temporalCoherenceWeight > 0.f;
    if (last == first || !temporal || !(has_prior || has_next || c->keyed))
        return bind_frame_anim(c, frame, level, ts);
    for (int side = 0; side < 2; side++) {
        const bool fwd = side == 0;
        const int nb = fwd ? frame - ts : frame + ts;
        if ((fwd ? has_prior : has_next) && source_pass >= 0) {
            TRY(bind_frame_level(c, nb, level, ts));
            TRY(pt_flip_anim_buffers(c));
            TRY(bind_frame_anim(c, frame, level, ts));
            TRY(load_last_saved_offsets(c, nb, level));
            TRY(pt_advect_offsets(c, level, ts, fwd ? 1 : 0, ops));
        } else if (c->keyed) {
            TRY(bind_frame_anim(c, frame, level, ts));
            TRY(ensure_random(c));
            TRY(pt_advect_offsets(c, level, ts, fwd ? 1 : 0, ops | PT_ADVECT_DO_NOT_CHECK_PREVIOUS));
        }
    }
    return PT_OK;
}

// SynthesisFrame::synthesizeInterpolated, synthesisFrame.cpp:384-418: one
// frame between its advected neighbours, both temporal terms on
static pt_status synthesize_interpolated(pt_ctx* c, const pt_params& user, int frame, int level, int this_pass,
                                         int source_pass, int first, int last, bool save_canvas) {
    pt_params p = user;  // updateParameters(BIDIRECTIONAL), :522-542
    p.advectionJitter = (frame % 3 == 0) ? user.advectionJitter * 0.01f : 0.0f;
    p.direction = PT_BIDIRECTIONAL;
    TRY(pt_set_params(c, &p));
    TRY(advect_neighbors(c, frame, level, source_pass, first, last));
    TRY(bind_frame_images(c, frame, level));
    TRY(store_load_offsets(c, level, frame, source_pass));
    TRY(do_sync(c, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
    TRY(propagate_and_scatter(c, level, user.iterations, false, c->keyed ? key_full_index(c, frame) : -1));
    return save_images(c, level, frame, this_pass, save_canvas);
}

// SynthesisProcessor::renderAnimationFBMO, synthesisProcessor.cpp:926-1022:
// per level a forward and a backward consecutive pass, their results merged
// at random (pass 2), then fix-up passes that synthesise every frame between
// its neighbours
static pt_status render_fbmo(pt_ctx* c, int first, int last, bool fresh) {
    const pt_params user = c->params;
    if (fresh) {
        TRY(reset_working(c));
        TRY(reset_image_slots(c));
        free_store(c);
    }
    const int final_pass = user.fixupPasses + 2;
    c->out_level = user.finalLevel;
    c->out_pass = final_pass;
    for (int level = user.levels - 1; level >= user.finalLevel; level--) {
        TRY(bind_style_level(c, level));
        if (c->keyed) TRY(upload_key_fields(c, level));
        const bool final_level = level == user.finalLevel;
        for (int pass = 0; pass < 2; pass++) {  // passes 0 and 1
            TRY(pt_reset_advected_buffers(c));
            const bool forwards = pass == 0;
            for (int i = 0; i <= last - first; i++) {
                const int f = forwards ? first + i : last - i;
                const bool is_first = i == 0;
                if (!is_first || pass > 0) TRY(pt_flip_anim_buffers(c));
                TRY(bind_frame_level(c, f, level));
                TRY(synthesize_consecutive(c, user, f, level, pass, is_first, forwards, final_pass, true, false));
            }
        }
        for (int f = first; f <= last; f++) {  // pass 2
            TRY(store_load_offsets(c, level, f, 0));
            TRY(store_load_residual(c, level, f, 0));
            TRY(pt_copy_offsets_to_advected(c, 1));
            TRY(do_sync(c, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
            TRY(store_load_offsets(c, level, f, 1));
            TRY(store_load_residual(c, level, f, 1));
            TRY(do_sync(c, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
            // SynthesisFrame::mergeRandomly, :510-520
            TRY(pt_merge_randomly(c, level, 1, c->keyed ? key_advect_weight(c, f, true) : 0.5f, 1));
            TRY(store_save(c, level, f, 2, final_level && final_pass == 2));
        }
        for (int pass = 3; pass < user.fixupPasses + 3; pass++) {  // renderInterpolatedFixupPass, :880-924
            for (int f = first; f <= last; f++) {
                const FrameLevel* L;
                TRY(frame_level(c, f, level, &L));
                const Arr<float4> rgba{L->rgba, L->w, L->h};
                const Arr<float> orient{L->orient, L->w, L->h};
                if (c->keyed) TRY(random_level_keyed(c, level, f, rgba, orient));
                else TRY(random_level(c, level, f, rgba, orient));
                TRY(synthesize_interpolated(c, user, f, level, pass, pass - 1, first, last,
                                            final_level && pass == final_pass));
            }
        }
        if (level + 1 < user.levels) drop_store_level(c, level + 1);
    }
    c->params = user;
    return PT_OK;
}

// --- keyframe interpolation driver ----------------------------------------------

static void free_key_ribbons(pt_ctx* c) {
    for (int d = 0; d < 2; d++) {
        for (auto& kv : c->f2k_pyr[d])
            for (float4* p : kv.second) dfree_t(c, p);
        for (auto& kv : c->k2k_pyr[d])
            for (float4* p : kv.second) dfree_t(c, p);
        c->f2k_pyr[d].clear();
        c->k2k_pyr[d].clear();
    }
    c->img.f2k[0] = c->img.f2k[1] = Arr<float4>{};
}

// SynthesisFrame::loadAnimImages with keys (synthesisFrame.cpp:613-627):
// the frame's frame-to-key ribbons of the level
static void bind_frame_keys(pt_ctx* c, int frame, int level) {
    for (int d = 0; d < 2; d++) {
        auto it = c->f2k_pyr[d].find(frame);
        if (it == c->f2k_pyr[d].end() || level >= (int)it->second.size()) continue;
        c->img.f2k[d] = Arr<float4>{it->second[level], c->W >> level, c->H >> level};
    }
}

// Style::load with keys (style.cpp:122-134): the key-to-key ribbons of the
// subrange's keys as the cumulative fields of the level, layer = subrange
// index (uploaded only once the first key's backward ribbon exists)
static pt_status upload_key_fields(pt_ctx* c, int level) {
    if (!c->k2k_pyr[0].count(0) || c->key_sub.empty()) return PT_OK;
    const int lw = c->W >> level, lh = c->H >> level;
    const size_t n = (size_t)lw * lh;
    TRY(pt_initialize_cumulative_fields(c, lw, lh, (int)c->key_sub.size()));
    for (size_t i = 0; i < c->key_sub.size(); i++) {
        const int full = key_full_index(c, c->key_sub[i]);
        for (int d = 0; d < 2; d++) {
            auto it = c->k2k_pyr[d].find(full);
            if (it == c->k2k_pyr[d].end() || level >= (int)it->second.size()) continue;
            CU(cudaMemcpyAsync(c->cumul[d] + i * n, it->second[level], n * sizeof(float4), cudaMemcpyDeviceToDevice,
                               c->stream));
        }
    }
    return PT_OK;
}

// initializeRibbonPyramid (imagePyramid.cpp:211-235) of a level-0 ribbon field
static pt_status ribbon_pyramid(pt_ctx* c, const ptk::Ribbon* src, int levels, std::vector<float4*>* out) {
    for (float4* p : *out) dfree_t(c, p);
    out->assign(levels, nullptr);
    for (int l = 0; l < levels; l++) {
        const int w = c->W >> l, h = c->H >> l;
        TRY(dalloc_t(c, &(*out)[l], (size_t)std::max(w, 1) * std::max(h, 1)));
        if (l == 0) LN(pt::launch_ribbon_pack(src, w, h, (*out)[0], c->stream));
        else LN(pt::launch_ribbon_down((*out)[l - 1], c->W >> (l - 1), (*out)[l], w, h, c->stream));
    }
    return PT_OK;
}

// SynthesisProcessor::accumulateRibbon, synthesisProcessor.cpp:528-627, at
// level 0: every frame's ribbon to the nearest key behind it in time,
// carried by accumulateRibbonField from the frames 1, 2, 4 ... behind it
// (steps above 1 through the ribbon inputs, as far as they exist).  Guides
// are not built (no kernel reads them).
static pt_status accumulate_ribbons(pt_ctx* c, bool forwards, int sfirst, int slast) {
    const int d = forwards ? 0 : 1;
    const int first_key = c->key_sub.front(), last_key = c->key_sub.back();
    const size_t n = (size_t)c->W * c->H, rb = n * sizeof(ptk::Ribbon);
    std::vector<int> blank, frames;
    if (forwards) {
        for (int f = c->run_first; f < first_key; f++) blank.push_back(f);
        for (int f = first_key; f <= slast; f++) frames.push_back(f);
    } else {
        for (int f = last_key + 1; f <= c->run_last; f++) blank.push_back(f);
        for (int f = last_key; f >= sfirst; f--) frames.push_back(f);
    }
    std::map<int, ptk::Ribbon*> acc;
    struct Free {
        pt_ctx* c;
        std::map<int, ptk::Ribbon*>* m;
        ~Free() {
            for (auto& kv : *m) dfree_t(c, kv.second);
        }
    } free_acc{c, &acc};
    auto levels_of = [&](int f) { return (int)c->frames[f].size(); };
    TRY(ensure_ribbons(c));
    const int k0 = frames.front();
    TRY(dalloc_t(c, &acc[k0], n));
    LN(pt::launch_fill_ribbons(acc[k0], n, -1, c->stream));
    CU(cudaMemcpyAsync(c->rib[0], acc[k0], rb, cudaMemcpyDeviceToDevice, c->stream));
    for (int f : blank) TRY(ribbon_pyramid(c, acc[k0], levels_of(f), &c->f2k_pyr[d][f]));
    const int cur = c->img.cur, prev_slot = 1 - c->img.cur;
    // level-0 velocities of `f` over `step` frames: its own, or its ribbons
    auto vel = [&](int f, int step, bool fwd) -> const float2* {
        if (step == 1) return fwd ? c->frames[f][0].velf : c->frames[f][0].velb;
        auto it = c->ribbons.find(std::make_pair(f, step));
        if (it == c->ribbons.end()) return nullptr;
        return fwd ? it->second[0].first : it->second[0].second;
    };
    for (int f : frames) {
        TRY(bind_frame_images(c, f, 0));  // loadImages(0)
        for (int ts = forwards ? -1 : 1; (forwards && f + ts >= first_key) || (!forwards && f + ts <= last_key);
             ts *= 2) {
            // loadRibbonPair(0, f + ts), synthesisFrame.cpp:658-706: steps
            // above 1 read the ribbon inputs and stop where there are none
            const int pf = f + ts, step = ts < 0 ? -ts : ts;
            const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
            const bool ahead = pf < f;
            const float2* vc = vel(f, step, !ahead);
            const float2* vp = vel(pf, step, ahead);
            if (!vc || !vp) break;
            if (ahead) {
                TRY(slot_write(c, &c->up_velb[cur], &c->img.velb[cur], vc, c->W, c->H, d2d));
                TRY(slot_write(c, &c->up_velf[prev_slot], &c->img.velf[prev_slot], vp, c->W, c->H, d2d));
            } else {
                TRY(slot_write(c, &c->up_velf[cur], &c->img.velf[cur], vc, c->W, c->H, d2d));
                TRY(slot_write(c, &c->up_velb[prev_slot], &c->img.velb[prev_slot], vp, c->W, c->H, d2d));
            }
            CU(cudaMemcpyAsync(c->rib[0], acc[pf], rb, cudaMemcpyDeviceToDevice, c->stream));
            TRY(pt_accumulate_ribbon_field(c, 0, forwards ? 1 : 0, ts, step == 1 ? 1 : 0));
        }
        if (!acc.count(f)) TRY(dalloc_t(c, &acc[f], n));
        CU(cudaMemcpyAsync(acc[f], c->rib[0], rb, cudaMemcpyDeviceToDevice, c->stream));
        const int k = key_sub_index(c, f);
        if (k >= 0) {
            const int full = key_full_index(c, f);
            TRY(ribbon_pyramid(c, acc[f], levels_of(f), &c->k2k_pyr[d][full]));
            const ExLevel& S = c->style_levels[0];
            const float4* key_out = S.out + (size_t)full * S.w * S.h;
            const size_t px = sizeof(float4);
            CU(cudaMemcpy2DAsync(c->canvas, c->W * px, key_out, S.w * px, S.w * px, S.h, cudaMemcpyDeviceToDevice,
                                 c->stream));
            CU(cudaMemcpy2DAsync(c->adv[0].out, c->W * px, key_out, S.w * px, S.w * px, S.h,
                                 cudaMemcpyDeviceToDevice, c->stream));
            LN(pt::launch_fill_ribbons(acc[f], n, k, c->stream));
            CU(cudaMemcpyAsync(c->rib[0], acc[f], rb, cudaMemcpyDeviceToDevice, c->stream));
        }
        TRY(ribbon_pyramid(c, acc[f], levels_of(f), &c->f2k_pyr[d][f]));
    }
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

// Style::updateKeyFrameSubrange, style.cpp:175-196 (a key just outside the
// range joins it through each neighbour inside, once per neighbour)
static void update_key_subrange(pt_ctx* c, int first, int last) {
    const std::vector<int>& K = c->key_frames;
    c->key_sub.clear();
    for (size_t i = 0; i < K.size(); i++) {
        const int idx = K[i];
        if (idx >= first && idx <= last) {
            c->key_sub.push_back(idx);
        } else {
            if (i + 1 < K.size() && K[i + 1] > first && K[i + 1] <= last) c->key_sub.push_back(idx);
            if (i > 0 && K[i - 1] >= first && K[i - 1] < last) c->key_sub.push_back(idx);
        }
    }
}

// renderAnimation with keyframe interpolation: keyFramesPreprocess
// (synthesisProcessor.cpp:629-674) then renderAnimationFMBM with
// SynthesisFrame's keyframe paths
static pt_status render_fmbm(pt_ctx* c, int first, int last, bool fresh);
static pt_status render_fbmo(pt_ctx* c, int first, int last, bool fresh);
static pt_status render_tctf(pt_ctx* c, int first, int last, bool fresh);
static pt_status render_ind(pt_ctx* c, int first, int last, bool fresh);
static pt_status render_keyed(pt_ctx* c, int first, int last) {
    const pt_params user = c->params;
    if (c->key_frames.empty()) return fail(c, PT_ERR_STATE, "no keyframes set (pt_set_keyframes)");
    update_key_subrange(c, first, last);
    if (c->key_sub.empty()) return fail(c, PT_ERR_INVALID, "no keyframe in or next to frames %d..%d", first, last);
    const int sfirst = std::min(first, c->key_sub.front()), slast = std::max(last, c->key_sub.back());
    for (int f = sfirst; f <= slast; f++)
        if (!c->frames.count(f)) return fail(c, PT_ERR_STATE, "frame %d not set", f);
    const ExLevel& S0 = c->style_levels.empty() ? ExLevel() : c->style_levels[0];
    if (S0.w != c->W || S0.h != c->H) return fail(c, PT_ERR_INVALID, "keyframe styles must have the image's size");
    TRY(reset_working(c));
    TRY(reset_image_slots(c));
    free_store(c);
    free_key_ribbons(c);
    struct Keyed {  // this run interpolates keys; layered uploads copy
        pt_ctx* c;
        explicit Keyed(pt_ctx* x) : c(x) { c->keyed = c->slot_copy = true; }
        ~Keyed() { c->keyed = c->slot_copy = false; }
    } keyed(c);
    c->run_first = first;
    c->run_last = last;
    pt_params p = user;
    p.interpolateKeyFrame = 0;  // the preprocess runs the plain kernels
    TRY(pt_set_params(c, &p));
    TRY(bind_style_level(c, 0));
    TRY(accumulate_ribbons(c, true, sfirst, slast));
    TRY(accumulate_ribbons(c, false, sfirst, slast));
    p = user;  // keyFramesPreprocess, :664-671
    p.interpolateKeyFrame = 1;
    p.numFrames = slast - sfirst;
    p.firstKeyIndex = key_full_index(c, c->key_sub.front());
    p.lastKeyIndex = key_full_index(c, c->key_sub.back());
    TRY(pt_set_params(c, &p));
    pt_status st;
    switch (user.scheme) {
        case PT_S_FBMO: st = render_fbmo(c, first, last, false); break;
        case PT_S_TCTF: st = render_tctf(c, first, last, false); break;
        case PT_S_IND: st = render_ind(c, first, last, false); break;
        default: st = render_fmbm(c, first, last, false); break;
    }
    c->params = user;
    return st;
}

pt_status pt_set_keyframes(pt_ctx* c, const int32_t* frames, int count) {
    if (!c || count < 0 || (count > 0 && !frames)) return PT_ERR_INVALID;
    if (count > c->NS) return fail(c, PT_ERR_INVALID, "%d keyframes but %d style layers", count, c->NS);
    for (int i = 1; i < count; i++)
        if (frames[i] <= frames[i - 1]) return fail(c, PT_ERR_INVALID, "keyframes must increase");
    c->key_frames.assign(frames, frames + count);
    return PT_OK;
}

// SynthesisProcessor::renderConsecutivePass, synthesisProcessor.cpp:703-753
static pt_status consecutive_pass(pt_ctx* c, const pt_params& user, int level, int pass, int source_pass, int first,
                                  int last, bool save_canvas, int time_step = 1) {
    const bool forwards = (pass % 2) == 0;
    std::vector<int> fr;
    if (forwards) for (int f = first; f <= last; f += time_step) fr.push_back(f);
    else for (int f = last; f >= first; f -= time_step) fr.push_back(f);
    if (pass > 0) {  // the frame still in memory starts the fix-up pass
        TRY(store_save(c, level, fr[0], pass, save_canvas));
        fr.erase(fr.begin());
    }
    for (size_t i = 0; i < fr.size(); i++) {
        const bool is_first = (i == 0) && (pass == 0);
        if (!is_first) TRY(pt_flip_anim_buffers(c));
        TRY(bind_frame_level(c, fr[i], level, time_step));
        TRY(synthesize_consecutive(c, user, fr[i], level, pass, is_first, forwards, source_pass, pass == 0,
                                   save_canvas, time_step));
    }
    return PT_OK;
}

// SynthesisFrame::spatialUpsample, synthesisFrame.cpp:465-481: the frame's
// last saved offsets of the coarse level upsampled (no images are loaded)
static pt_status spatial_upsample(pt_ctx* c, int frame, int coarse, int fine, bool save, bool save_canvas) {
    TRY(load_last_saved_offsets(c, frame, coarse));
    TRY(pt_upsample(c, fine));
    TRY(do_sync(c, fine, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
    if (save) TRY(save_images(c, fine, frame, 0, save_canvas));
    return PT_OK;
}

// SynthesisProcessor::renderAnimationFMBM, synthesisProcessor.cpp:846-878
// (`fresh`: a new run; a keyed run starts from the state its
// keyFramesPreprocess left)
static pt_status render_fmbm(pt_ctx* c, int first, int last, bool fresh) {
    const pt_params user = c->params;
    if (fresh) {
        TRY(reset_working(c));
        TRY(reset_image_slots(c));
        free_store(c);
    }
    const int total = user.fixupPasses + 1;
    const int final_pass = (user.finalLevel == 0) ? total - 1 : 0;
    c->out_level = 0;
    c->out_pass = final_pass;
    for (int level = user.levels - 1; level >= user.finalLevel; level--) {
        TRY(bind_style_level(c, level));
        if (c->keyed) TRY(upload_key_fields(c, level));
        TRY(pt_reset_advected_buffers(c));
        for (int pass = 0; pass < total; pass++)
            TRY(consecutive_pass(c, user, level, pass, total - 1, first, last,
                                 level == 0 && pass == final_pass));
        // the coarser level's saved state is no longer needed
        if (level + 1 < user.levels) drop_store_level(c, level + 1);
    }
    // renderSpatialUpsample (:1025-1045) down to level 0 from a final level
    for (int level = user.finalLevel; level > 0; level--) {
        TRY(bind_style_level(c, level - 1));
        if (c->keyed) TRY(upload_key_fields(c, level - 1));
        for (int f = first; f <= last; f++) TRY(spatial_upsample(c, f, level, level - 1, true, level == 1));
        if (level + 1 < user.levels) drop_store_level(c, level + 1);
    }
    c->params = user;
    return PT_OK;
}

// WorkingBuffers::linkTempImagesToNextPass (workingBuffers.cpp:329-365)
// through SynthesisFrame::linkImagesToPass: pass `this_pass` of the frame
// becomes a copy of its last saved pass (the frame's last saved pass stays)
static pt_status link_to_pass(pt_ctx* c, int frame, int level, int this_pass) {
    auto ls = c->last_saved.find(std::make_pair(frame, level));
    const int src = ls == c->last_saved.end() ? 0 : ls->second;
    auto it = c->store.find(std::make_tuple(level, frame, src));
    if (it == c->store.end() || src == this_pass) return PT_OK;  // no file to link
    const StoreEntry S = it->second;
    StoreEntry& D = c->store[std::make_tuple(level, frame, this_pass)];
    const size_t n = (size_t)S.w * S.h;
    if (!D.offs || D.w != S.w || D.h != S.h) {
        dfree_t(c, D.offs); dfree_t(c, D.res); dfree_t(c, D.canvas);
        D.canvas = nullptr;
        TRY(dalloc_t(c, &D.offs, n));
        TRY(dalloc_t(c, &D.res, n));
        D.w = S.w;
        D.h = S.h;
    }
    CU(cudaMemcpyAsync(D.offs, S.offs, n * sizeof(pt_patchxf), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(D.res, S.res, n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    if (S.canvas) {
        if (!D.canvas) TRY(dalloc_t(c, &D.canvas, n));
        CU(cudaMemcpyAsync(D.canvas, S.canvas, n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
    }
    return PT_OK;
}

enum RefineOp { REFINE_ODD, REFINE_EVEN, REFINE_EVEN_AND_ODD, INITIALIZE_EVEN_AND_ODD };

// SynthesisProcessor::renderRefinePass (synthesisProcessor.cpp:1078-1150)
// and renderInitializationPass (:1047-1076) with SynthesisFrame::refine
// (synthesisFrame.cpp:420-463): the frames of the op (odd multiples of the
// time step, even ones, or all) each synthesised between its neighbours one
// time step away, started by temporal upsampling (mergeAdvectedBuffers,
// random fallback: the odd frames of the coarsest level, and every frame of
// the keyframe initialisation there), spatial upsampling (the level's
// first refine, odd frames below the coarsest level) or from its own last
// saved pass; ODD and EVEN passes link the frames they skip to the new pass
static pt_status refine_pass(pt_ctx* c, const pt_params& user, int level, int last_coarse_pass, int this_pass,
                             int first, int last, bool save_canvas, int op = REFINE_EVEN_AND_ODD, int ts = 1) {
    const bool coarsest = level == user.levels - 1;
    const int coarse_step = ts * 2;
    std::vector<int> frames;
    const int start = op == REFINE_ODD ? first + ts : first;
    const int step = (op == REFINE_ODD || op == REFINE_EVEN) ? coarse_step : ts;
    for (int f = start; f <= last; f += step) frames.push_back(f);
    enum { PREVIOUS, SPATIAL, TEMPORAL } init = PREVIOUS;
    if (op == INITIALIZE_EVEN_AND_ODD || op == REFINE_ODD) init = coarsest ? TEMPORAL : SPATIAL;
    else if (op == REFINE_EVEN_AND_ODD && last_coarse_pass == this_pass - 1) init = SPATIAL;
    const bool neighbours = op != INITIALIZE_EVEN_AND_ODD;
    for (int f : frames) {
        pt_params p = user;  // updateParameters(BIDIRECTIONAL), :522-542
        p.advectionJitter = (f % 3 == 0) ? user.advectionJitter * 0.01f : 0.0f;
        p.direction = PT_BIDIRECTIONAL;
        TRY(pt_set_params(c, &p));
        TRY(advect_neighbors(c, f, level, this_pass - 1, first, last, neighbours, ts));
        if (init == TEMPORAL) {
            TRY(ensure_random(c));
            TRY(pt_merge_advected_buffers(c, level, PT_MERGE_FALLBACK_RANDOM));
        } else if (init == SPATIAL) {
            TRY(spatial_upsample(c, f, level + 1, level, false, false));
        } else {
            TRY(load_last_saved_offsets(c, f, level));
            TRY(do_sync(c, level, PT_DONT_COPY_OFFSETS | PT_DONT_UPDATE_RESIDUAL));
        }
        TRY(bind_frame_images(c, f, level));
        TRY(propagate_and_scatter(c, level, user.iterations, false, c->keyed ? key_full_index(c, f) : -1));
        TRY(save_images(c, level, f, this_pass, save_canvas));
    }
    if (op == REFINE_ODD)
        for (int f = first; f <= last; f += coarse_step) TRY(link_to_pass(c, f, level, this_pass));
    else if (op == REFINE_EVEN)
        for (int f = first + ts; f <= last; f += coarse_step) TRY(link_to_pass(c, f, level, this_pass));
    return PT_OK;
}

// the longest ribbon step every frame of the range has, with all shorter
// ones (NLShot::setup stops at the first step a frame lacks; 1 without
// ribbons, the max(1, ...) of renderAnimationTCTF)
static int max_ribbon_step(const pt_ctx* c, int first, int last) {
    int step = 1;
    for (;;) {
        const int next = step * 2;
        for (int f = first; f <= last; f++)
            if (!c->ribbons.count(std::make_pair(f, next))) return step;
        step = next;
    }
}

// SynthesisProcessor::renderAnimationTCTF, synthesisProcessor.cpp:1152-1312,
// run locally: the longest ribbon step T every frame has (1 without ribbon
// inputs); a consecutive pass at the coarsest level over every T-th frame
// (with keys: the initialisation pass), refine passes at every level for
// step T (fixupPasses + 1 more while T < last - first), then for each
// halved step the odd frames refined at every level with fix-up passes, then
// spatial upsampling down to level 0.  Level-0 passes keep their output.
static pt_status render_tctf(pt_ctx* c, int first, int last, bool fresh) {
    const pt_params user = c->params;
    if (fresh) {
        TRY(reset_working(c));
        TRY(reset_image_slots(c));
        free_store(c);
    }
    enum { CONSECUTIVE = 100, UPSAMPLE = 101 };
    struct Op {
        int kind, level, ts;
    };
    const int max_ts = max_ribbon_step(c, first, last);
    const int L = user.levels - 1;
    // with several time steps the levels are revisited coarse after fine:
    // frame binds copy into the full-size layered arrays (as for IND)
    struct SlotCopy {
        pt_ctx* c;
        bool was;
        SlotCopy(pt_ctx* x, bool on) : c(x), was(x->slot_copy) { c->slot_copy = was || on; }
        ~SlotCopy() { c->slot_copy = was; }
    } slot_copy(c, max_ts > 1);
    std::vector<Op> ops;
    ops.push_back({c->keyed ? (int)INITIALIZE_EVEN_AND_ODD : (int)CONSECUTIVE, L, max_ts});
    for (int level = L; level >= user.finalLevel; level--) {
        ops.push_back({REFINE_EVEN_AND_ODD, level, max_ts});
        if (max_ts < last - first)
            for (int i = 0; i < user.fixupPasses + 1; i++) ops.push_back({REFINE_EVEN_AND_ODD, level, max_ts});
    }
    for (int ts = max_ts / 2; ts > 0; ts /= 2)
        for (int level = L; level >= user.finalLevel; level--) {
            ops.push_back({REFINE_ODD, level, ts});
            if (ts < last - first)
                for (int i = 0; i < user.fixupPasses; i++) ops.push_back({REFINE_EVEN_AND_ODD, level, ts});
        }
    for (int level = user.finalLevel - 1; level >= 0; level--) ops.push_back({UPSAMPLE, level, 1});
    // the pass counters of the schedule (:1257-1285)
    int passes_this = 0, passes_last = 0, last_level = -1;
    TRY(pt_reset_advected_buffers(c));
    for (const Op& op : ops) {
        const int level = op.level;
        if (last_level != level) {
            TRY(bind_style_level(c, level));
            if (c->keyed) TRY(upload_key_fields(c, level));
            passes_last = passes_this;  // (levels are revisited per time step: every level's passes stay)
            last_level = level;
        }
        const bool keep = level == 0;
        if (op.kind == INITIALIZE_EVEN_AND_ODD) {
            TRY(refine_pass(c, user, level, passes_this - 1, 0, first, last, keep, INITIALIZE_EVEN_AND_ODD, op.ts));
            passes_this = 1;
        } else if (op.kind == CONSECUTIVE) {
            TRY(consecutive_pass(c, user, level, passes_this, passes_this - 1, first, last, keep, op.ts));
            passes_this++;
        } else if (op.kind == UPSAMPLE) {
            for (int f = first; f <= last; f++) TRY(spatial_upsample(c, f, level + 1, level, true, keep));
            passes_this = 1;
        } else {
            TRY(refine_pass(c, user, level, passes_last - 1, passes_this, first, last, keep, op.kind, op.ts));
            passes_this++;
        }
    }
    c->out_level = 0;
    c->out_pass = passes_this - 1;
    c->params = user;
    return PT_OK;
}

static pt_status render(pt_ctx* c, int first, int last) {
    const pt_params& user = c->params;
    if (user.interpolateKeyFrame) return render_keyed(c, first, last);
    if (user.levels < 1 || user.finalLevel < 0 || user.finalLevel >= user.levels)
        return fail(c, PT_ERR_INVALID, "bad levels/finalLevel");
    for (int f = first; f <= last; f++)
        if (!c->frames.count(f)) return fail(c, PT_ERR_STATE, "frame %d not set", f);
    switch (user.scheme) {
        case PT_S_FMBM:
        case PT_S_FMBM_RM: return render_fmbm(c, first, last, true);
        case PT_S_FBMO: return render_fbmo(c, first, last, true);
        case PT_S_TCTF: return render_tctf(c, first, last, true);
        case PT_S_IND: return render_ind(c, first, last, true);
        default: return fail(c, PT_ERR_INVALID, "unknown scheme %d", user.scheme);
    }
}

static pt_status fetch_final(pt_ctx* c, int frame, float* out_rgba, pt_patchxf* out_offsets) {
    auto it = c->store.find(std::make_tuple(c->out_level, frame, c->out_pass));
    if (it == c->store.end()) return fail(c, PT_ERR_STATE, "no final output for frame %d", frame);
    size_t n = (size_t)it->second.w * it->second.h;
    if (out_rgba)
        CU(cudaMemcpyAsync(out_rgba, it->second.canvas, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    if (out_offsets)
        CU(cudaMemcpyAsync(out_offsets, it->second.offs, n * sizeof(pt_patchxf), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

pt_status pt_synthesize_frame(pt_ctx* c, int frame, float* out_rgba, pt_patchxf* out_offsets) {
    if (!c) return PT_ERR_INVALID;
    if (!c->initialized || !c->have_params) return fail(c, PT_ERR_STATE, "context not initialized");
    CU(cudaSetDevice(c->device));
    TRY(render(c, frame, frame));
    return fetch_final(c, frame, out_rgba, out_offsets);
}

pt_status pt_synthesize_animation(pt_ctx* c, int first, int last, pt_frame_callback cb, void* user) {
    if (!c || last < first) return PT_ERR_INVALID;
    if (!c->initialized || !c->have_params) return fail(c, PT_ERR_STATE, "context not initialized");
    CU(cudaSetDevice(c->device));
    TRY(render(c, first, last));
    if (cb) {
        // each frame is handed to the callback from page-locked staging
        int lw = c->W >> c->out_level, lh = c->H >> c->out_level;
        size_t n = (size_t)lw * lh;
        size_t need = n * (sizeof(float4) + sizeof(pt_patchxf));
        if (c->cb_stage_bytes < need) {
            if (c->cb_stage) cudaFreeHost(c->cb_stage);
            c->cb_stage = nullptr;
            c->cb_stage_bytes = 0;
            CU(cudaMallocHost(&c->cb_stage, need));
            c->cb_stage_bytes = need;
        }
        float* rgba = (float*)c->cb_stage;
        pt_patchxf* offs = (pt_patchxf*)((char*)c->cb_stage + n * sizeof(float4));
        for (int f = first; f <= last; f++) {
            TRY(fetch_final(c, f, rgba, offs));
            cb(f, rgba, offs, lw, lh, user);
        }
    }
    return PT_OK;
}

pt_status pt_get_frame_result(pt_ctx* c, int frame, float* out_rgba, pt_patchxf* out_offsets) {
    if (!c) return PT_ERR_INVALID;
    if (!c->initialized || !c->have_params) return fail(c, PT_ERR_STATE, "context not initialized");
    CU(cudaSetDevice(c->device));
    return fetch_final(c, frame, out_rgba, out_offsets);
}

pt_status pt_get_frame_residual(pt_ctx* c, int frame, float* out_residual) {
    if (!c || !out_residual) return PT_ERR_INVALID;
    if (!c->initialized || !c->have_params) return fail(c, PT_ERR_STATE, "context not initialized");
    CU(cudaSetDevice(c->device));
    auto it = c->store.find(std::make_tuple(c->out_level, frame, c->out_pass));
    if (it == c->store.end()) return fail(c, PT_ERR_STATE, "no final output for frame %d", frame);
    size_t n = (size_t)it->second.w * it->second.h;
    CU(cudaMemcpyAsync(out_residual, it->second.res, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

pt_status pt_host_alloc(size_t bytes, void** out) {
    if (!out) return PT_ERR_INVALID;
    *out = nullptr;
    if (bytes == 0) return PT_OK;
    if (cudaMallocHost(out, bytes) != cudaSuccess) {
        *out = nullptr;
        return PT_ERR_CUDA;
    }
    return PT_OK;
}

pt_status pt_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) return PT_ERR_CUDA;
    return PT_OK;
}
