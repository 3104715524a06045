// pt_ctx.h -- the context of libpainttween_gb300 (struct pt_ctx) and the
// helpers its host translation units share: pt_context.cpp (errors, device
// memory, kernel parameters, set-up and uploads), pt_steps.cpp (the step-wise
// compute calls of the TexSynth interface), pt_frames.cpp (the resident working
// set and the measurement calls) and pt_driver.cpp (the per-frame driver and
// its animation schemes).
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
#pragma once
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
using ptk::TileMaps;


namespace ptc {

inline int level_count(int w, int h) {
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

}  // namespace ptc

using ptc::ExLevel;
using ptc::FrameLevel;
using ptc::StoreEntry;
using ptc::TexArray;
using ptc::level_count;

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
    bool use_tma = true;                   // interior tiles staged by tensor copies
    // propagate's warps per tile row: 0 = picked by the autotuner below, 1 or 2
    int prop_lanes = 0;
    int sm_count = 0;
    // autotuner of propagate's warps per tile row, per launch shape (radius,
    // temporal mode, filter mode, tile-count class): one launch of each
    // variant is timed with events (the results are identical), and the
    // faster one is kept, for every context of the device
    struct Tune {
        int choice = -1;   // 0: one warp per row, 1: two; -1: not decided
        int probes = 0;    // variants launched with events
        cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    };
    std::map<std::tuple<int, int, int, int>, Tune> tune;
    int* tma_err = nullptr;                // set by a block whose tensor-copy wait ran out
    // tensor maps of staged planes: (plane, pitch, level w, level h, box) -> map
    std::map<std::tuple<const void*, int, int, int, int>, CUtensorMap> tmaps;

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

// helpers defined in one translation unit and used in others (not exported)
#define PT_HIDDEN __attribute__((visibility("hidden")))

inline PatchPlanes base_planes(pt_ctx* c) { return c->off[c->base_i]; }
PT_HIDDEN pt_status base_for_partial_write(pt_ctx* c, int level, PatchPlanes* out);
PT_HIDDEN pt_status check_tma(pt_ctx* c);
PT_HIDDEN pt_status check_ready(pt_ctx* c, int level, bool need_ex = true, bool need_img = true);
PT_HIDDEN pt_status copy_planes_full(pt_ctx* c, PatchPlanes dst, PatchPlanes src);
PT_HIDDEN pt_status dalloc(pt_ctx* c, void** p, size_t bytes);
PT_HIDDEN void dfree(pt_ctx* c, void* p);
PT_HIDDEN pt_status do_residual(pt_ctx* c, int level);
PT_HIDDEN pt_status do_sync(pt_ctx* c, int level, int flags);
PT_HIDDEN pt_status ensure_random(pt_ctx* c);
PT_HIDDEN pt_status ensure_ribbons(pt_ctx* c);
PT_HIDDEN pt_status ensure_stage(pt_ctx* c, size_t bytes);
PT_HIDDEN pt_status fail(pt_ctx* c, pt_status s, const char* fmt, ...);
PT_HIDDEN void free_frames(pt_ctx* c);
PT_HIDDEN void free_store(pt_ctx* c);
PT_HIDDEN void free_textures(pt_ctx* c, ExLevel* L);
PT_HIDDEN void glibc_state(uint32_t seed, uint32_t out[31]);
PT_HIDDEN pt_status h2d(pt_ctx* c, void* dst, const void* src, size_t bytes);
PT_HIDDEN cudaError_t launch_tiled(pt_ctx* c, int kind, const Params& P, PatchPlanes work, int arg, uint32_t pass_id,
                                   float* out, bool* done);
PT_HIDDEN Params make_params(pt_ctx* c, int level);
PT_HIDDEN cudaEvent_t pool_event(pt_ctx* c);
PT_HIDDEN pt_status random_level(pt_ctx* c, int level, int frame, Arr<float4> rgba, Arr<float> orient);
PT_HIDDEN pt_status rect_copy(pt_ctx* c, void* dst, size_t dpitch, const void* src, size_t spitch, size_t row_bytes,
                              int rows, cudaMemcpyKind kind);
PT_HIDDEN pt_status refresh_interleaved(pt_ctx* c, ExLevel* L);
PT_HIDDEN pt_status reset_image_slots(pt_ctx* c);
PT_HIDDEN pt_status reset_working(pt_ctx* c);
PT_HIDDEN std::vector<uint32_t> step_power(uint64_t n);
PT_HIDDEN bool tiled_usable(pt_ctx* c);
PT_HIDDEN pt_status writable_work(pt_ctx* c, int level, PatchPlanes* out, bool* was_aliased = nullptr);

template <class T>
static pt_status dalloc_t(pt_ctx* c, T** p, size_t count) {
    void* v = nullptr;
    pt_status s = dalloc(c, &v, count * sizeof(T));
    *p = (T*)v;
    return s;
}
template <class T>
static void dfree_t(pt_ctx* c, T*& p) {
    dfree(c, (void*)p);
    p = nullptr;
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
