// pt_context.cpp -- the context of libpainttween_gb300: errors, device memory
// (the per-context block cache and texture arrays), kernel parameters,
// creation, parameters, initialisation and the step-wise image uploads.
#include "pt_ctx.h"

#include <mutex>

// ---------------------------------------------------------------------------
// errors and allocation
// ---------------------------------------------------------------------------

pt_status fail(pt_ctx* c, pt_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
    return s;
}

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
pt_status dalloc(pt_ctx* c, void** p, size_t bytes) {
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
void dfree(pt_ctx* c, void* p) {
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

pt_status ensure_stage(pt_ctx* c, size_t bytes) {
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


Params make_params(pt_ctx* c, int level) {
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
void free_textures(pt_ctx* c, ExLevel* L) {
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
pt_status refresh_interleaved(pt_ctx* c, ExLevel* L) {
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

pt_status check_ready(pt_ctx* c, int level, bool need_ex, bool need_img) {
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
pt_status copy_planes_full(pt_ctx* c, PatchPlanes dst, PatchPlanes src) {
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
pt_status writable_work(pt_ctx* c, int level, PatchPlanes* out, bool* was_aliased) {
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
pt_status base_for_partial_write(pt_ctx* c, int level, PatchPlanes* out) {
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

cudaEvent_t pool_event(pt_ctx* c) {
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
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
bool tiled_usable(pt_ctx* c) {
    int r = c->params.residualWindowSize;
    return c->use_tiled && !c->params.interpolateKeyFrame && c->params.colorspace == 0 &&
           c->params.coherenceWeight <= 0.f &&
           temporal_mode(c) >= 0 && r >= 2 && r <= 4;
}

// launches the tiled kernel of `kind` if one is instantiated for this
// configuration; *done = false otherwise (the generic kernel is used)
// cuTensorMapEncodeTiled, from the driver through the runtime (the library
// links the runtime statically and not the driver)
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return (EncodeTiledFn)p;
    }();
    return fn;
}

// The tensor map of a float4 plane (`pitch` texels per row) over a w x h
// level: a FLOAT32 tensor of 4w x h elements whose boxes are tw x th texels
// (4 tw elements: 16 tw bytes, a multiple of 16).  False when the plane
// cannot be mapped (no encoder, an address not on 16 bytes, a level smaller
// than a box); its tiles are then staged by plain loads.
static bool plane_map(pt_ctx* c, const void* p, int pitch, int w, int h, int tw, int th, CUtensorMap* out) {
    if (!p || ((uintptr_t)p & 15) || pitch < w || w < tw || h < th) return false;
    const auto key = std::make_tuple(p, pitch, w, h, tw * 1024 + th);
    auto it = c->tmaps.find(key);
    if (it != c->tmaps.end()) {
        *out = it->second;
        return true;
    }
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {4ull * (cuuint64_t)w, (cuuint64_t)h};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float4)};
    const cuuint32_t box[2] = {4u * (cuuint32_t)tw, (cuuint32_t)th};
    const cuuint32_t es[2] = {1, 1};
    CUtensorMap m;
    if (fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(p), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    if (c->tmaps.size() >= 512) c->tmaps.clear();
    c->tmaps.emplace(key, m);
    *out = m;
    return true;
}

// the tensor maps of the planes a tiled kernel of mode tm stages
static void tile_maps(pt_ctx* c, const Params& P, int tm, TileMaps* M) {
    memset(M, 0, sizeof(*M));
    M->err = c->tma_err;
    if (!c->use_tma || !c->tma_err) return;
    const int tw = ptk::kTileW + 2 * P.r, th = ptk::kTileH + 2 * P.r;
    const Arr<float4>& ib = P.img.base[P.img.cur];
    bool ok = plane_map(c, ib.p, ib.w, P.lw, P.lh, tw, th, &M->base) &&
              plane_map(c, P.canvas, P.W, P.lw, P.lh, tw, th, &M->canvas);
    if (ok && tm) {
        const AdvView& A = P.adv[tm == 1 ? 0 : 1];
        ok = plane_map(c, A.base, P.W, P.lw, P.lh, tw, th, &M->pbase) &&
             plane_map(c, A.out, P.W, P.lw, P.lh, tw, th, &M->pout) &&
             plane_map(c, A.off.B, P.W, P.lw, P.lh, tw, th, &M->prec);
    }
    M->on = ok ? 1 : 0;
}

// Propagate's warps per tile row for this launch (0: one, 1: two) and the
// variant being timed (-1: none).  Launch shapes are keyed by radius,
// temporal mode, filter mode and the tile count relative to the SM count,
// in powers of two (up to a quarter, half, one, 2, 4, 8 SMs' worth, more):
// the choice depends on how much of the GPU the tiles fill.  Decisions are shared by the contexts of a
// device; until a shape's two variants have been timed, shapes with no
// more tiles than SMs take two warps.
static std::mutex g_tune_mutex;
static std::map<std::tuple<int, int, int, int, int>, int> g_tune;  // (device, shape) -> choice

static std::tuple<int, int, int, int> tune_key(pt_ctx* c, const Params& P, int tm, int* blocks) {
    if (!c->sm_count) {
        if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) {
            cudaGetLastError();
            c->sm_count = 152;
        }
    }
    *blocks = ((P.lw + ptk::kTileW - 1) / ptk::kTileW) * ((P.lh + ptk::kTileH - 1) / ptk::kTileH);
    int cls = 0;
    while (cls < 6 && 4 * (long long)*blocks > ((long long)c->sm_count << cls)) cls++;
    return std::make_tuple(P.r, tm, P.ex.hw, cls);
}

static int propagate_variant(pt_ctx* c, const Params& P, int tm, int* probe) {
    *probe = -1;
    if (c->prop_lanes) return c->prop_lanes - 1;
    int blocks = 0;
    const auto key = tune_key(c, P, tm, &blocks);
    const auto gkey = std::tuple_cat(std::make_tuple(c->device), key);
    const int fallback = blocks <= c->sm_count ? 1 : 0;
    {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        auto it = g_tune.find(gkey);
        if (it != g_tune.end()) return it->second;
    }
    pt_ctx::Tune& t = c->tune[key];
    if (t.choice >= 0) return t.choice;
    if (t.probes < 2) {
        for (int k = 0; k < 2; k++)
            if (!t.ev[2 * t.probes + k] && cudaEventCreate(&t.ev[2 * t.probes + k]) != cudaSuccess) {
                cudaGetLastError();
                t.choice = fallback;  // no events: no timing
                return fallback;
            }
        *probe = t.probes;
        return t.probes++;
    }
    if (cudaEventQuery(t.ev[3]) == cudaSuccess && cudaEventQuery(t.ev[1]) == cudaSuccess) {
        float a = 0.f, b = 0.f;
        if (cudaEventElapsedTime(&a, t.ev[0], t.ev[1]) == cudaSuccess &&
            cudaEventElapsedTime(&b, t.ev[2], t.ev[3]) == cudaSuccess) {
            t.choice = b < a ? 1 : 0;
            std::lock_guard<std::mutex> lk(g_tune_mutex);
            g_tune.emplace(gkey, t.choice);
        } else {
            t.choice = fallback;
        }
        cudaGetLastError();
        for (auto& e : t.ev) {
            if (e) cudaEventDestroy(e);
            e = nullptr;
        }
        return t.choice;
    }
    cudaGetLastError();  // (cudaErrorNotReady)
    return fallback;
}

cudaError_t launch_tiled(pt_ctx* c, int kind, const Params& P, PatchPlanes work, int arg, uint32_t pass_id,
                         float* out, bool* done) {
    *done = false;
    if (!tiled_usable(c)) return cudaSuccess;
    int tm = temporal_mode(c);
    if (P.r < 2 || P.r > 4) return cudaSuccess;
    TileMaps M;
    tile_maps(c, P, tm, &M);
    int probe = -1;
    const int wide = kind == 0 ? propagate_variant(c, P, tm, &probe) : 0;
    int blocks = 0;
    pt_ctx::Tune* t = probe >= 0 ? &c->tune[tune_key(c, P, tm, &blocks)] : nullptr;
    if (t) cudaEventRecord(t->ev[2 * probe], c->stream);
    *done = true;
    cudaError_t e;
    switch (P.r) {
        case 2: e = pt::launch_tiled_2(kind, tm, P, M, work, arg, pass_id, out, wide, c->stream); break;
        case 3: e = pt::launch_tiled_3(kind, tm, P, M, work, arg, pass_id, out, wide, c->stream); break;
        default: e = pt::launch_tiled_4(kind, tm, P, M, work, arg, pass_id, out, wide, c->stream); break;
    }
    if (t) cudaEventRecord(t->ev[2 * probe + 1], c->stream);
    return e;
}

// the tensor-copy error flag: PT_ERR_CUDA (and the flag cleared) when a
// tiled kernel's block gave up waiting for its staging copies
pt_status check_tma(pt_ctx* c) {
    if (!c->tma_err) return PT_OK;
    int v = 0;
    CU(cudaMemcpyAsync(&v, c->tma_err, sizeof v, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (!v) return PT_OK;
    CU(cudaMemsetAsync(c->tma_err, 0, sizeof(int), c->stream));
    return fail(c, PT_ERR_CUDA, "a tiled kernel's wait for its tensor copies ran out");
}

pt_status do_residual(pt_ctx* c, int level) {
    Params P = make_params(c, level);
    float* out = c->res[c->res_i];
    return profiled(c, PT_KERNEL_RESIDUAL, P, [&](const Params& Q) {
        bool done = false;
        cudaError_t e = launch_tiled(c, 2, Q, PatchPlanes{}, 0, 0, out, &done);
        return done ? e : pt::launch_residual(Q, out, c->stream);
    });
}

// TexSynth::syncBuffers, texSynth_kernel.cu:1240-1303
pt_status do_sync(pt_ctx* c, int level, int flags) {
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
void glibc_state(uint32_t seed, uint32_t out[31]) {
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
std::vector<uint32_t> step_power(uint64_t n) {
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
    if (dalloc_t(c, &c->flag, 4) != PT_OK || dalloc_t(c, &c->tma_err, 1) != PT_OK) {
        cudaStreamDestroy(c->stream);
        delete c;
        return PT_ERR_OOM;
    }
    *out = c;
    return PT_OK;
}

void free_frames(pt_ctx* c) {
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
void free_store(pt_ctx* c) {
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
    for (auto& kv : c->tune)
        for (auto& e : kv.second.ev)
            if (e) cudaEventDestroy(e);
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
    return check_tma(c);
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
pt_status reset_working(pt_ctx* c) {
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
pt_status rect_copy(pt_ctx* c, void* dst, size_t dpitch, const void* src, size_t spitch, size_t row_bytes,
                    int rows, cudaMemcpyKind kind) {
    CU(cudaMemcpy2DAsync(dst, dpitch, src, spitch, row_bytes, rows, kind, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

pt_status h2d(pt_ctx* c, void* dst, const void* src, size_t bytes) {
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

// A layered input image (colour, distance transform, velocities) as the
// reference keeps it (cudaImageBuffer.h layered copyFromHost): one
// full-size array per layer, which an upload of a level overwrites on that
// level's rectangle only, so texels outside the rectangle keep what a finer
// level left there.  Allocated zeroed; bound with the full width as pitch.

// A fresh run: no input image or random level bound, the layered arrays all
// zero.
pt_status reset_image_slots(pt_ctx* c) {
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
