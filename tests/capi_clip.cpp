// capi_clip.cpp -- a native C++ caller of the C ABI (include/painttween.h),
// the way a host application links the library: no Python, no torch.
//
// Usage: capi_clip <input.bin> <output.bin>
//
// input.bin (little-endian, written by tests/test_capi_native.py):
//   int32 magic 'PTCL', w, h, ew, eh, frames, sizeof(pt_params)
//   pt_params
//   exemplar: base rgba [eh][ew][4] f32, output rgba [eh][ew][4] f32,
//             orientation tensor [eh][ew][3] f32, distance transform [eh][ew] f32,
//             object ids [eh][ew] i32
//   per frame: rgba [h][w][4] f32, orientation tensor [h][w][3] f32,
//              distance transform [h][w] f32, object ids [h][w] i32,
//              forward and backward velocities [h][w][2] f32 each,
//              scale [h][w][2] f32
// output.bin: per frame, in frame order, the final rgba [oh][ow][4] f32 and
//   offsets [oh][ow] pt_patchxf from pt_synthesize_animation's callback, then
//   the last frame's rgba and offsets again as read back by
//   pt_get_frame_result into page-locked memory, then the results of the same
//   clip submitted twice at once to pt_serve (two requests in flight): for
//   each request, all frames' rgba, then all frames' offsets.
//
// Exits 0 on success; on any failure prints the status and the context's last
// error and exits 1.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "painttween.h"

namespace {

pt_ctx* g_ctx = nullptr;

void check(pt_status s, const char* what) {
    if (s != PT_OK) {
        std::fprintf(stderr, "%s: %s (%s)\n", what, pt_status_string(s), g_ctx ? pt_last_error(g_ctx) : "");
        std::exit(1);
    }
}

template <class T>
std::vector<T> read_array(std::FILE* f, size_t n) {
    std::vector<T> v(n);
    if (std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "short input\n");
        std::exit(1);
    }
    return v;
}

struct Output {
    std::FILE* f;
    int frames_seen;
    int next_frame;
    bool in_order;
};

void on_frame(int frame, const float* rgba, const pt_patchxf* offsets, int w, int h, void* user) {
    Output* o = static_cast<Output*>(user);
    if (frame != o->next_frame) o->in_order = false;
    o->next_frame = frame + 1;
    o->frames_seen++;
    std::fwrite(rgba, sizeof(float), (size_t)w * h * 4, o->f);
    std::fwrite(offsets, sizeof(pt_patchxf), (size_t)w * h, o->f);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    std::FILE* in = std::fopen(argv[1], "rb");
    if (!in) {
        std::perror(argv[1]);
        return 1;
    }
    std::vector<int32_t> hdr = read_array<int32_t>(in, 7);
    if (hdr[0] != 0x4C435450 || hdr[6] != (int32_t)sizeof(pt_params)) {
        std::fprintf(stderr, "bad header (params size %d, compiled %d)\n", hdr[6], (int)sizeof(pt_params));
        return 1;
    }
    const int w = hdr[1], h = hdr[2], ew = hdr[3], eh = hdr[4], frames = hdr[5];
    pt_params params = read_array<pt_params>(in, 1)[0];
    const size_t ne = (size_t)ew * eh, ni = (size_t)w * h;
    std::vector<float> ex_base = read_array<float>(in, ne * 4), ex_out = read_array<float>(in, ne * 4);
    std::vector<float> ex_tensor = read_array<float>(in, ne * 3), ex_dt = read_array<float>(in, ne);
    std::vector<int32_t> ex_ids = read_array<int32_t>(in, ne);

    if (pt_abi_version() != PT_ABI_VERSION) {
        std::fprintf(stderr, "library ABI %d, header %d\n", pt_abi_version(), PT_ABI_VERSION);
        return 1;
    }
    check(pt_create(0, 0, &g_ctx), "pt_create");
    check(pt_initialize(g_ctx, w, h, ew, eh, 1), "pt_initialize");
    check(pt_set_params(g_ctx, &params), "pt_set_params");
    check(pt_set_style(g_ctx, 0, ew, eh, ex_base.data(), ex_out.data(), ex_tensor.data(), ex_dt.data(),
                       ex_ids.data()),
          "pt_set_style");
    struct Frame {
        std::vector<float> rgba, tensor, dt, vf, vb, scale;
        std::vector<int32_t> ids;
    };
    std::vector<Frame> clip(frames);
    for (int f = 0; f < frames; f++) {
        Frame& fr = clip[f];
        fr.rgba = read_array<float>(in, ni * 4);
        fr.tensor = read_array<float>(in, ni * 3);
        fr.dt = read_array<float>(in, ni);
        fr.ids = read_array<int32_t>(in, ni);
        fr.vf = read_array<float>(in, ni * 2);
        fr.vb = read_array<float>(in, ni * 2);
        fr.scale = read_array<float>(in, ni * 2);
        check(pt_set_frame(g_ctx, f, w, h, fr.rgba.data(), fr.tensor.data(), fr.dt.data(), fr.ids.data(),
                           fr.vf.data(), fr.vb.data(), fr.scale.data()),
              "pt_set_frame");
    }
    std::fclose(in);

    std::FILE* out = std::fopen(argv[2], "wb");
    if (!out) {
        std::perror(argv[2]);
        return 1;
    }
    Output o = {out, 0, 0, true};
    check(pt_synthesize_animation(g_ctx, 0, frames - 1, on_frame, &o), "pt_synthesize_animation");
    if (o.frames_seen != frames || !o.in_order) {
        std::fprintf(stderr, "callback saw %d frames (in order: %d), expected %d\n", o.frames_seen, (int)o.in_order,
                     frames);
        return 1;
    }
    const int fl = PT_OUTPUT_LEVEL(&params);
    const size_t no = (size_t)(w >> fl) * (h >> fl);
    float* rgba = nullptr;
    pt_patchxf* offs = nullptr;
    check(pt_host_alloc(no * 4 * sizeof(float), (void**)&rgba), "pt_host_alloc");
    check(pt_host_alloc(no * sizeof(pt_patchxf), (void**)&offs), "pt_host_alloc");
    check(pt_get_frame_result(g_ctx, frames - 1, rgba, offs), "pt_get_frame_result");
    std::fwrite(rgba, sizeof(float), no * 4, out);
    std::fwrite(offs, sizeof(pt_patchxf), no, out);
    check(pt_host_free(rgba), "pt_host_free");
    check(pt_host_free(offs), "pt_host_free");
    std::printf("capi_clip: %d frames %dx%d, %llu kernel launches\n", frames, w >> fl, h >> fl,
                (unsigned long long)pt_kernel_launches(g_ctx));
    check(pt_destroy(g_ctx), "pt_destroy");
    g_ctx = nullptr;

    // the same clip as two requests served at once
    std::vector<pt_frame_inputs> inputs(frames);
    for (int f = 0; f < frames; f++) {
        const Frame& fr = clip[f];
        inputs[f] = {fr.rgba.data(), fr.tensor.data(), fr.dt.data(), fr.ids.data(),
                     fr.vf.data(), fr.vb.data(), fr.scale.data()};
    }
    const int nreq = 2;
    std::vector<std::vector<float> > req_rgba(nreq, std::vector<float>(no * 4 * frames));
    std::vector<std::vector<pt_patchxf> > req_offs(nreq, std::vector<pt_patchxf>(no * frames));
    std::vector<pt_request> reqs(nreq);
    for (int r = 0; r < nreq; r++) {
        pt_request& q = reqs[r];
        std::memset(&q, 0, sizeof(q));
        q.params = params;
        q.style_w = ew;
        q.style_h = eh;
        q.style_base = ex_base.data();
        q.style_output = ex_out.data();
        q.style_orient_tensor = ex_tensor.data();
        q.style_dist_trans = ex_dt.data();
        q.style_ids = ex_ids.data();
        q.image_w = w;
        q.image_h = h;
        q.frames = frames;
        q.inputs = inputs.data();
        q.out_rgba = req_rgba[r].data();
        q.out_offsets = req_offs[r].data();
        q.arrival_ms = 0.0;
    }
    check(pt_serve(0, reqs.data(), nreq, nreq, 0), "pt_serve");
    for (int r = 0; r < nreq; r++) {
        check(reqs[r].status, "request");
        std::fwrite(req_rgba[r].data(), sizeof(float), req_rgba[r].size(), out);
        std::fwrite(req_offs[r].data(), sizeof(pt_patchxf), req_offs[r].size(), out);
    }
    std::fclose(out);
    return 0;
}
