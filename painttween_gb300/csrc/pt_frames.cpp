// pt_frames.cpp -- the resident working set (exemplar and frame pyramids built
// on the device by pt_set_style / pt_set_frame, ribbon inputs) and the
// measurement calls (timers, profiling, kernel statistics).
#include "pt_ctx.h"

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

pt_status pt_set_propagate_lanes(pt_ctx* c, int warps_per_row) {
    if (!c || warps_per_row < 0 || warps_per_row > 2) return PT_ERR_INVALID;
    c->prop_lanes = warps_per_row;
    return PT_OK;
}

pt_status pt_set_tma_staging(pt_ctx* c, int on) {
    if (!c) return PT_ERR_INVALID;
    c->use_tma = on != 0;
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
