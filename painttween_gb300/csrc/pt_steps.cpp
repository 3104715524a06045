// pt_steps.cpp -- the step-wise compute calls of the C ABI, one per TexSynth
// operation (texSynth_kernel.h:38-91): random levels, propagate, scatter,
// upsample, advection, merges, residual and buffer syncs, keyframe fields,
// state transfers and the separable Gaussian.
#include "pt_ctx.h"

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

pt_status pt_create_random_level(pt_ctx* c, int level, int frame) {
    if (!c) return PT_ERR_INVALID;
    TRY(check_ready(c, level));
    return random_level(c, level, frame, c->img.base[c->img.cur], c->img.orient);
}

pt_status random_level(pt_ctx* c, int level, int frame, Arr<float4> rgba, Arr<float> orient) {
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

pt_status ensure_ribbons(pt_ctx* c) {
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
pt_status ensure_random(pt_ctx* c) {
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
