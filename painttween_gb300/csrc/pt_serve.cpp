// pt_serve.cpp -- many synthesis requests on one GPU (pt_server_*, pt_serve).
//
// Worker threads each use a context of the server (its own device buffers,
// memory cache and CUDA stream, kept between runs) and take requests in
// arrival order.  A request is admitted once its arrival time has passed and
// its device memory fits the budget beside the requests in flight: with a
// budget, admission waits until the running requests' contexts are set up
// and counts the memory those contexts actually hold, plus an estimate from
// the new request's sizes.  Several requests' kernels so run on
// the GPU at once: a small still alone fills only a few of the GPU's 152
// SMs.  Everything here goes through the public C ABI; the contexts share
// nothing, so each result is the one a request gets on a context of its own.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

#include "painttween.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// Device memory a request needs, estimated from its sizes: per image pixel
// the offset, residual, canvas and advected planes, the change-tracking
// planes and the per-tap residual values, per frame pixel its pyramid, per
// style texel its pyramid with the interleaved copy and the histogram.
size_t estimate_bytes(const pt_request& r) {
    const size_t px = (size_t)r.image_w * r.image_h;
    const size_t taps = (size_t)(2 * r.params.residualWindowSize + 1) * (2 * r.params.residualWindowSize + 1);
    const size_t per_px = 720 + 4 * taps;
    const size_t per_frame_px = 96;
    const size_t per_texel = 150;
    return px * per_px + px * per_frame_px * (size_t)std::max(r.frames, 1) +
           (size_t)r.style_w * r.style_h * per_texel;
}

#define PT_TRY(expr)                   \
    do {                               \
        pt_status s_ = (expr);         \
        if (s_ != PT_OK) return s_;    \
    } while (0)

// the request's buffers, exemplar pyramid and frame pyramids on the context
pt_status setup_request(pt_ctx* c, pt_request& r) {
    if (r.frames < 1 || !r.inputs || r.image_w < 2 || r.image_h < 2) return PT_ERR_INVALID;
    PT_TRY(pt_initialize(c, r.image_w, r.image_h, r.style_w, r.style_h, 1));
    PT_TRY(pt_set_params(c, &r.params));
    PT_TRY(pt_set_style(c, 0, r.style_w, r.style_h, r.style_base, r.style_output, r.style_orient_tensor,
                        r.style_dist_trans, r.style_ids));
    PT_TRY(pt_clear_frames(c));
    for (int f = 0; f < r.frames; f++) {
        const pt_frame_inputs& in = r.inputs[f];
        PT_TRY(pt_set_frame(c, f, r.image_w, r.image_h, in.rgba, in.orient_tensor, in.dist_trans, in.ids, in.vel_fwd,
                            in.vel_bwd, in.scale));
    }
    return PT_OK;
}

// its synthesis, results into the request's output arrays
pt_status synthesize_request(pt_ctx* c, pt_request& r) {
    const int fl = PT_OUTPUT_LEVEL(&r.params);
    const size_t n = (size_t)(r.image_w >> fl) * (size_t)(r.image_h >> fl);
    if (r.frames == 1) {
        PT_TRY(pt_synthesize_frame(c, 0, r.out_rgba, r.out_offsets));
    } else {
        PT_TRY(pt_synthesize_animation(c, 0, r.frames - 1, nullptr, nullptr));
        for (int f = 0; f < r.frames; f++)
            PT_TRY(pt_get_frame_result(c, f, r.out_rgba ? r.out_rgba + (size_t)f * n * 4 : nullptr,
                                       r.out_offsets ? r.out_offsets + (size_t)f * n : nullptr));
    }
    PT_TRY(pt_clear_frames(c));
    return PT_OK;
}
#undef PT_TRY

struct Queue {
    std::mutex m;
    std::condition_variable cv;
    std::vector<int> order;  // request indices by arrival time
    size_t next = 0;         // next request of `order` to admit
    size_t in_flight = 0;    // bytes of the admitted, unfinished requests
    int running = 0;
    int setting_up = 0;      // admitted requests whose memory is still an estimate
};

}  // namespace

struct pt_server {
    int device = 0;
    int max_in_flight = 1;
    size_t budget = 0;
    std::vector<pt_ctx*> ctxs;  // one per worker, created on first use and kept
};

pt_status pt_server_create(int device, int max_in_flight, size_t hbm_budget, pt_server** out) {
    if (!out || max_in_flight < 1) return PT_ERR_INVALID;
    pt_server* s = new pt_server;
    s->device = device;
    s->max_in_flight = max_in_flight;
    s->budget = hbm_budget;
    s->ctxs.assign(max_in_flight, nullptr);
    *out = s;
    return PT_OK;
}

pt_status pt_server_destroy(pt_server* s) {
    if (!s) return PT_ERR_INVALID;
    for (pt_ctx* c : s->ctxs)
        if (c) pt_destroy(c);
    delete s;
    return PT_OK;
}

pt_status pt_server_run(pt_server* srv, pt_request* reqs, int count) {
    if (!srv || count < 0 || (count > 0 && !reqs)) return PT_ERR_INVALID;
    const int device = srv->device, max_in_flight = srv->max_in_flight;
    const size_t hbm_budget = srv->budget;
    for (int i = 0; i < count; i++) {
        reqs[i].status = PT_ERR_STATE;  // not run
        reqs[i].start_ms = reqs[i].done_ms = 0.0;
        reqs[i].device_bytes = 0;
    }
    Queue q;
    q.order.resize(count);
    for (int i = 0; i < count; i++) q.order[i] = i;
    std::stable_sort(q.order.begin(), q.order.end(),
                     [&](int a, int b) { return reqs[a].arrival_ms < reqs[b].arrival_ms; });
    const Clock::time_point t0 = Clock::now();
    const int workers = std::min(max_in_flight, std::max(count, 1));
    std::vector<std::thread> pool;
    for (int w = 0; w < workers; w++) {
        pool.emplace_back([&, w]() {
            pt_ctx*& c = srv->ctxs[w];
            const pt_status created = c ? PT_OK : pt_create(device, 0, &c);
            for (;;) {
                int idx = -1;
                size_t est = 0;
                {
                    std::unique_lock<std::mutex> lk(q.m);
                    for (;;) {
                        if (q.next >= q.order.size()) break;
                        idx = q.order[q.next];
                        est = estimate_bytes(reqs[idx]);
                        const double now = ms_since(t0);
                        if (now < reqs[idx].arrival_ms) {  // not arrived yet
                            q.cv.wait_for(lk, std::chrono::duration<double, std::milli>(reqs[idx].arrival_ms - now));
                            idx = -1;
                            continue;
                        }
                        // with a budget, the next admission waits until every running request's
                        // memory is known, then needs room for its own estimate beside them
                        if (hbm_budget && q.running > 0 && (q.setting_up > 0 || q.in_flight + est > hbm_budget)) {
                            q.cv.wait(lk);
                            idx = -1;
                            continue;
                        }
                        q.next++;
                        q.in_flight += est;
                        q.running++;
                        q.setting_up++;
                        break;
                    }
                }
                if (idx < 0) break;
                pt_request& r = reqs[idx];
                r.start_ms = ms_since(t0);
                r.status = (created == PT_OK) ? setup_request(c, r) : created;
                r.device_bytes = c ? pt_device_bytes(c) : 0;
                {
                    // the budget from now on counts what the context actually holds
                    std::lock_guard<std::mutex> lk(q.m);
                    if (r.status == PT_OK) {
                        q.in_flight = q.in_flight - est + r.device_bytes;
                        est = r.device_bytes;
                    }
                    q.setting_up--;
                }
                q.cv.notify_all();
                if (r.status == PT_OK) r.status = synthesize_request(c, r);
                r.done_ms = ms_since(t0);
                {
                    std::lock_guard<std::mutex> lk(q.m);
                    q.in_flight -= est;
                    q.running--;
                }
                q.cv.notify_all();
            }
        });
    }
    for (auto& t : pool) t.join();
    for (int i = 0; i < count; i++)
        if (reqs[i].status != PT_OK) return reqs[i].status;
    return PT_OK;
}

pt_status pt_serve(int device, pt_request* reqs, int count, int max_in_flight, size_t hbm_budget) {
    pt_server* s = nullptr;
    pt_status st = pt_server_create(device, max_in_flight, hbm_budget, &s);
    if (st != PT_OK) return st;
    st = pt_server_run(s, reqs, count);
    pt_server_destroy(s);
    return st;
}
