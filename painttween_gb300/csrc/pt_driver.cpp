// pt_driver.cpp -- the per-frame driver over the resident working set:
// propagateAndScatter, the FMBM / FBMO / TCTF / IND schemes, keyframe
// interpolation, and pt_synthesize_frame / pt_synthesize_animation.
#include "pt_ctx.h"

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
    TRY(check_tma(c));
    return fetch_final(c, frame, out_rgba, out_offsets);
}

pt_status pt_synthesize_animation(pt_ctx* c, int first, int last, pt_frame_callback cb, void* user) {
    if (!c || last < first) return PT_ERR_INVALID;
    if (!c->initialized || !c->have_params) return fail(c, PT_ERR_STATE, "context not initialized");
    CU(cudaSetDevice(c->device));
    TRY(render(c, first, last));
    TRY(check_tma(c));
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
