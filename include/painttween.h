/*
 * painttween.h -- C ABI of the GB300-native offset-field synthesis library
 * (libpainttween_gb300.so).
 *
 * This is the drop-in boundary for PaintTween's per-frame offset-field
 * synthesis: the PatchMatch-style nearest-neighbour-field optimisation run at
 * each pyramid level, with offset advection along velocity fields for
 * animations.  Every entry point below replaces one call of the reference's
 * C++ namespace `TexSynth` (src/PaintTweenCUDA/texSynth_kernel.h:38-91) or of
 * the per-frame driver that sequences those calls
 * (src/PaintTweenCUDA/synthesisFrame.cpp, synthesisProcessor.cpp).  The
 * reference keeps its state in file-scope globals (texture references,
 * `__constant__ TsParameters gParams`, `gCurrentBuffer`) and exits the process
 * on any CUDA error; here all state lives in an opaque context and every call
 * returns a status code.
 *
 * Conventions
 *  - Host arrays are owned by the caller; device memory is owned by the
 *    context.  Host pointers are plain row-major arrays of the level size.
 *  - One context per host thread; a context is bound to one CUDA device and
 *    one stream (created by pt_create).
 *  - Image-size buffers are allocated at full (level-0) resolution; level L
 *    uses the top-left (W>>L) x (H>>L) rectangle, as in the reference
 *    (src/PaintTweenCUDA/cudaImageBuffer.h:124-129).
 *  - No call falls back to the CPU: if the CUDA kernels cannot run the call
 *    returns PT_ERR_CUDA.
 */
#ifndef PAINTTWEEN_GB300_H
#define PAINTTWEEN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_ABI_VERSION 1
#define PT_MAX_STYLES 5 /* NUM_MAX_STYLES, texSynth_interface.h:37 */

typedef enum {
    PT_OK = 0,
    PT_ERR_INVALID = 1,     /* bad argument, size or layer */
    PT_ERR_CUDA = 2,        /* CUDA runtime error (message in pt_last_error) */
    PT_ERR_OOM = 3,         /* device allocation failed */
    PT_ERR_STATE = 4,       /* call made before the state it needs exists */
    PT_ERR_UNSUPPORTED = 5, /* feature outside the implemented path */
    PT_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
    PT_ERR_BUDGET = 7       /* request does not fit the context's HBM budget */
} pt_status;

/* One offset-field sample; same field order, types and 36-byte size as the
 * reference's PatchXF (src/PaintTweenCUDA/types.h:94-109). */
typedef struct {
    float x, y, theta, hysteresis;
    int32_t layer;
    float scaleU, scaleV;
    float lumShiftY, lumShiftA; /* Luminance luminanceShift {y, a} */
} pt_patchxf;

/* RibbonP (types.h:111-126): accumulated motion from a pixel to a keyframe
 * (x, y), the frames it spans and the keyframe's index; layer < 0 marks an
 * invalid ribbon.  As an RGBA image (toColor4) it is (time_step, y, x,
 * layer). */
typedef struct {
    float x, y;
    int32_t time_step, layer;
} pt_ribbon;

/* Pass direction (types.h:122-126). */
enum { PT_FORWARD = 0, PT_BACKWARD = 1, PT_BIDIRECTIONAL = 2 };

/* Synthesis schemes (types.h:128-134); all five are implemented. */
enum { PT_S_FMBM = 0, PT_S_FMBM_RM = 1, PT_S_FBMO = 2, PT_S_TCTF = 3, PT_S_IND = 4 };

/* Random-number mode.
 *  PT_RNG_REFERENCE: the reference's behaviour -- the random-offset pyramid
 *    is the glibc srand(frame*level)/rand() sequence of
 *    SynthesisFrame::createRandomPyramid (synthesisFrame.cpp:66-150), and the
 *    scatter search uses r = theta = 0 because the reference's randFloat()
 *    returns an unsigned int (texSynth_util.h:155-163).
 *  PT_RNG_COUNTER: counter-based hash candidates (seeded, order-independent)
 *    for both the random pyramid and a real random search. */
enum { PT_RNG_REFERENCE = 0, PT_RNG_COUNTER = 1 };

/* Filtering of the linearly filtered inputs (exemplar colours and distance
 * transform, image colours, distance transform, velocities and scale,
 * keyframe ribbon fields), which the reference fetches through the texture
 * unit with bilinear filtering (texSynth_kernel.cu:2120-2253).
 *  PT_FILTER_TEXTURE: the texture unit's own arithmetic, as measured on
 *    GB300: weights quantised to 1/256 (round half up of the fractions,
 *    w11 = round(a*b), the others by difference), texels aligned to the
 *    largest exponent and truncated to 28 bits, the weighted sum rounded
 *    half away from zero, subnormal texels read as zero.  The exemplar
 *    colour samples of the tiled kernels go through the texture unit itself.
 *  PT_FILTER_EXACT: bilinear weights and sums in exact FP32 arithmetic. */
enum { PT_FILTER_EXACT = 0, PT_FILTER_TEXTURE = 1 };

/* Field-for-field copy of TsParameters (texSynth_interface.h:79-152); C bools
 * are int32 here.  The trailing fields are this library's additions. */
typedef struct {
    int32_t residualWindowSize; /* patch radius r: taps in [-r, r]^2 */
    float coherenceWeight;
    float distTransWeight;
    float lumShiftWeight;
    int32_t lumShiftEnable;
    float inputAnalogyWeight;
    float canvasOutputWeight;
    int32_t numStyles;
    float offsetsHistogramSlope[PT_MAX_STYLES];
    float offsetsHistogramThreshold[PT_MAX_STYLES];
    float maxDistortion;
    float alphaWeight;
    int32_t transparencyOk;
    float styleObjIdWeight;
    int32_t orientationEnabled;
    int32_t colorspace; /* 0 = RGB, 1 = Lab (RGBtoLAB before every comparison) */
    float coherenceRatioRange;
    float coherenceAngleRange;
    int32_t levels;
    int32_t scatterSamplesCount;
    float advectionJitter;
    float timeDerivativeInputWeight;
    float timeDerivativeOutputWeight;
    float temporalCoherenceWeight;
    float hysteresisWeight;
    int32_t interpolateKeyFrame; /* keyframe interpolation (pt_set_keyframes) */
    int32_t useGuide;
    int32_t currentInterpolationIndex;
    int32_t numFrames;
    int32_t numKeyFrames;
    int32_t firstKeyIndex;
    int32_t lastKeyIndex;
    int32_t distTransCull;
    float residualWindowScaleU, residualWindowScaleV;
    int32_t direction; /* PT_FORWARD / PT_BACKWARD / PT_BIDIRECTIONAL */
    /* --- driver parameters (NLParameters "iterations", "fixupPasses",
     *     "synthesisScheme", "maxLevel"; GUI/nlParameters.cpp:106-144) --- */
    int32_t iterations;
    int32_t fixupPasses;
    int32_t scheme;
    int32_t finalLevel;
    int32_t rngMode;     /* PT_RNG_* */
    uint32_t rngSeed;    /* seed of PT_RNG_COUNTER */
    int32_t filterMode;  /* PT_FILTER_* */
    int32_t reserved[5];
} pt_params;

/* Image layers (TsImageLayer, texSynth_interface.h:53-77, in-scope subset;
 * the numeric values are the reference's). */
enum {
    PT_LAYER_EXEMPLAR_BASE = 0,
    PT_LAYER_EXEMPLAR_OUTPUT = 1,
    PT_LAYER_EXEMPLAR_ORIENTATION = 2,
    PT_LAYER_EXEMPLAR_DIST_TRANS = 3,
    PT_LAYER_EXEMPLAR_OBJECT_IDS = 4,
    PT_LAYER_INPUT_COLOR = 5,
    PT_LAYER_INPUT_ORIENTATION = 6,
    PT_LAYER_INPUT_DIST_TRANS = 7,
    PT_LAYER_INPUT_SCALE = 8,
    PT_LAYER_INPUT_ID = 9,
    PT_LAYER_INPUT_SURF_ID = 10,          /* accepted, read by no kernel */
    PT_LAYER_INPUT_VEL_B = 11,
    PT_LAYER_INPUT_VEL_F = 12,
    PT_LAYER_INPUT_VEL_B_PREVIOUS = 13,
    PT_LAYER_INPUT_VEL_F_PREVIOUS = 14,
    PT_LAYER_GUIDE_B = 15,                /* accepted, read by no kernel */
    PT_LAYER_GUIDE_F = 16,
    PT_LAYER_CUMUL_FIELD_B = 17,          /* key-to-key ribbons, layer = key index */
    PT_LAYER_CUMUL_FIELD_F = 18,
    PT_LAYER_FRAME_TO_KEY_RIBBON_B = 19,  /* frame-to-key ribbons of the level */
    PT_LAYER_FRAME_TO_KEY_RIBBON_F = 20,
    PT_LAYER_RANDOM = 21
};

/* syncBuffers / advect / merge flags (texSynth_kernel.h:79-91). */
enum {
    PT_DONT_COPY_OFFSETS = 0x01,
    PT_DONT_UPDATE_RESIDUAL = 0x10,
    PT_MERGE_FALLBACK_RANDOM = 0x20,
    PT_MERGE_FALLBACK_LAST_PASS = 0x40
};
enum {
    PT_ADVECT_IGNORE_RANDOM = 0x1,
    PT_ADVECT_DO_NOT_CHECK_PREVIOUS = 0x10,
    PT_ADVECT_CHECK_FRAME_TO_KEY = 0x20,
    PT_ADVECT_UPDATE_RESIDUAL = 0x80
};

typedef struct pt_ctx pt_ctx;

/* ---- context ------------------------------------------------------------ */

/* Creates a context on `device` with its own stream.  `hbm_budget_bytes`
 * caps the device memory the context may allocate (0 = no cap).
 * Replaces SynthesisProcessor's ownership of WorkingBuffers
 * (synthesisProcessor.cpp:109,119). */
pt_status pt_create(int device, size_t hbm_budget_bytes, pt_ctx** out);
pt_status pt_destroy(pt_ctx* ctx);
const char* pt_status_string(pt_status s);
/* Last error message of this context (never NULL). */
const char* pt_last_error(const pt_ctx* ctx);
/* ABI version number (PT_ABI_VERSION). */
int pt_abi_version(void);
/* Default parameters: NLParameters::getTsDefaultParams
 * (GUI/nlParameters.cpp:63-104) plus iterations 3, fixupPasses 1,
 * scheme FMBM_RM (nlParameters.cpp:133-137) and distTransCull 50
 * (synthesisProcessor.cpp:220). */
void pt_default_params(pt_params* out);
/* Device memory currently held by the context, in bytes. */
size_t pt_device_bytes(const pt_ctx* ctx);

/* ---- configuration (TexSynth::setup / uploadParameters,
 *      texSynth_kernel.cu:109-123) ---------------------------------------- */
pt_status pt_set_params(pt_ctx* ctx, const pt_params* params);
pt_status pt_get_params(const pt_ctx* ctx, pt_params* out);

/* Allocates the image-size working buffers (offsets, residual, canvas,
 * advected F/B) at image_w x image_h and the style-size histogram at
 * style_w x (style_h * num_styles); everything is zeroed.
 * Replaces WorkingBuffers::initialize (workingBuffers.cpp:48-94) and
 * TexSynth::initialize_images (texSynth_kernel.cu:2120-2126). */
pt_status pt_initialize(pt_ctx* ctx, int image_w, int image_h,
                        int style_w, int style_h, int num_styles);
/* Sizes the exemplar arrays for one pyramid level (w, h = level size).
 * Replaces TexSynth::initialize_exemplars (texSynth_kernel.cu:2128-2135). */
pt_status pt_initialize_exemplars(pt_ctx* ctx, int w, int h, int num_styles);

/* Uploads one pyramid level of one layer from host memory; w, h must be the
 * level size.  `style` selects the exemplar layer (style index).
 * Replaces TexSynth::uploadImage_{Color4,float,float2,int}
 * (texSynth_kernel.cu:2143-2253). */
pt_status pt_upload_image_color4(pt_ctx* ctx, int level, int layer,
                                 const float* rgba, int w, int h, int style);
pt_status pt_upload_image_float(pt_ctx* ctx, int level, int layer,
                                const float* data, int w, int h, int style);
pt_status pt_upload_image_float2(pt_ctx* ctx, int level, int layer,
                                 const float* xy, int w, int h);
pt_status pt_upload_image_int(pt_ctx* ctx, int level, int layer,
                              const int32_t* data, int w, int h, int style);
/* Swaps the current/previous frame layers (TexSynth::flipAnimBuffers,
 * texSynth_kernel.cu:1534-1538). */
pt_status pt_flip_anim_buffers(pt_ctx* ctx);

/* ---- per-step compute (TexSynth::*, texSynth_kernel.h:58-76) ------------ */

/* Builds the random-offset level from the uploaded input colour/orientation
 * and exemplar output/orientation, on the device; replaces
 * SynthesisFrame::createRandomPyramid (synthesisFrame.cpp:66-150). */
pt_status pt_create_random_level(pt_ctx* ctx, int level, int frame);
pt_status pt_randomize_offsets(pt_ctx* ctx, int level);          /* :2100 */
pt_status pt_propagate(pt_ctx* ctx, int level, int jump, int key_index); /* :1306 */
pt_status pt_scatter(pt_ctx* ctx, int level, int key_index);      /* :1360 */
pt_status pt_upsample(pt_ctx* ctx, int fine_level);               /* :1513 */
pt_status pt_advect_offsets(pt_ctx* ctx, int level, int time_step,
                            int forwards, int op_flags);           /* :1695 */
pt_status pt_merge_randomly(pt_ctx* ctx, int level, int forwards,
                            float weight_advected, int force_valid); /* :2003 */
pt_status pt_merge_using_residual(pt_ctx* ctx, int level, int forwards); /* :1978 */
pt_status pt_update_residual_cache(pt_ctx* ctx, int level);       /* :1221 */
pt_status pt_sync_buffers(pt_ctx* ctx, int level, int op_flags);  /* :1240 */
pt_status pt_reset_advected_buffers(pt_ctx* ctx); /* workingBuffers.cpp:119-123 */
/* offsets.base().copyTo(advectedF/B.offsets()) and
 * residualCache.base().copyTo(advectedF/B.residual()), the merge set-up of
 * renderAnimationFBMO (synthesisProcessor.cpp:979-980). */
pt_status pt_copy_offsets_to_advected(pt_ctx* ctx, int forwards);

/* Keyframes for pt_synthesize_* with params.interpolateKeyFrame: style
 * layer i (pt_set_style, the image's size) is the painted key of frame
 * frames[i], increasing (DataAccess::keyFrameIndices).  The run then does
 * keyFramesPreprocess (synthesisProcessor.cpp:528-674: ribbons from every
 * frame to its nearest keys, accumulated frame by frame) and
 * renderAnimationFMBM with SynthesisFrame's keyframe paths (FMBM and
 * FMBM_RM schemes); frames from the nearest keys outside first..last must
 * be set too. */
pt_status pt_set_keyframes(pt_ctx* ctx, const int32_t* frames, int count);

/* ---- keyframe interpolation (texSynth_kernel.cu:290-304,723-1110,
 *      1728-1853,2061-2118,2138-2142).  With params.interpolateKeyFrame set,
 *      pt_propagate / pt_scatter run propagate_kernel_keys /
 *      scatter_kernel_keys, which also test the candidates that the
 *      key-to-key cumulative fields carry to the keys firstKeyIndex ..
 *      lastKeyIndex; with key_index >= 0 a pixel under that key's mask (the
 *      alpha of exemplar output layer key_index at the pixel) takes the key
 *      (propagate) or keeps its offset (scatter).  The cumulative fields and
 *      frame-to-key ribbons are uploaded as RGBA images
 *      (pt_upload_image_color4 with PT_LAYER_CUMUL_FIELD_B/F, style = key
 *      layer, and PT_LAYER_FRAME_TO_KEY_RIBBON_B/F). */
pt_status pt_initialize_cumulative_fields(pt_ctx* ctx, int w, int h, int layers); /* :2138 */
/* The ribbon field (working <- base carried along the velocities from the
 * previous frame, then copied to base) and advectedF.output <- the canvas at
 * each ribbon's end (accumulateRibbonField, :1830-1853). */
pt_status pt_accumulate_ribbon_field(pt_ctx* ctx, int level, int forwards, int time_step, int overwrite);
/* Offsets from the frame-to-key ribbons, random where a ribbon is invalid
 * (offsetsFromFrameToKeyRibbon, :2111-2118; ends with a sync). */
pt_status pt_offsets_from_frame_to_key_ribbon(pt_ctx* ctx, int level, int look_forwards);
/* mergeAdvectedKernel (:1938-1976, host :2025-2042): the forward and
 * backward advected offsets merged, at random where both are valid, else
 * PT_MERGE_FALLBACK_RANDOM (the random level's fractional parts) or
 * PT_MERGE_FALLBACK_LAST_PASS (the base offsets); ends with a sync. */
pt_status pt_merge_advected_buffers(pt_ctx* ctx, int level, int merge_fallback);
/* ribbonField.base() and canvasOutputCache to and from the host (level
 * rectangle, row-major), advectedF/B.output() to the host. */
pt_status pt_load_ribbon_field(pt_ctx* ctx, int level, const pt_ribbon* ribbons);
pt_status pt_get_ribbon_field(pt_ctx* ctx, int level, pt_ribbon* out);
pt_status pt_load_canvas(pt_ctx* ctx, int level, const float* rgba);
pt_status pt_get_advected_output(pt_ctx* ctx, int forwards, int level, float* out_rgba);

/* ---- state transfer (WorkingBuffers load/getOutput,
 *      workingBuffers.cpp:118-207) ---------------------------------------- */
/* Writes the level rectangle of the offsets base buffer (loadOffsets). */
pt_status pt_load_offsets(pt_ctx* ctx, int level, const pt_patchxf* offsets);
/* Writes the level rectangle of the residual buffer, rounding each value
 * through IEEE half precision as the reference's EXR round trip does
 * (loadResidual reads the half-precision .b channel). */
pt_status pt_load_residual(pt_ctx* ctx, int level, const float* residual);
pt_status pt_get_offsets(pt_ctx* ctx, int level, pt_patchxf* out);
pt_status pt_get_residual(pt_ctx* ctx, int level, float* out);
/* Stylised output (canvasOutputCache), RGBA float32. */
pt_status pt_get_output(pt_ctx* ctx, int level, float* out_rgba);

/* Separable normalised Gaussian blur (sigma = radius / 3, zero outside the
 * image) of one float image: convolutionRowsGPU followed by
 * convolutionColumnsGPU (convolution.h:36-44, convolution.cu:63-210), the
 * smoothing the reference applies to its offsets histogram.  src and dst are
 * device pointers with a row pitch of `pitch` floats; the row-pass result is
 * kept in the context's scratch buffer.  Runs on the context's stream. */
pt_status pt_convolve_separable(pt_ctx* ctx, const float* src_dev, float* dst_dev, int w, int h, int pitch,
                                int radius);

/* The Gaussian weights allocateGaussianKernel (convolution.cu:37-60)
 * uploads: 2*radius+1 floats into `out` (host memory), sigma = radius / 3,
 * unnormalised (the patch-distance window) or, with `normalize`, divided by
 * sqrt(2*pi)*sigma (the histogram smoothing of pt_convolve_separable).
 * Host-only: no device is used. */
pt_status pt_gaussian_kernel(int radius, int normalize, float* out);

/* Allocation-free variant of pt_convolve_separable, for callers that cannot
 * allocate device memory when they call it (a plugin host that owns all
 * device memory through its own pool and forbids cudaMalloc in its frame
 * callbacks, or a process whose memory a framework's caching allocator
 * holds).  It has no counterpart in the reference.
 *  - No context: the caller passes device pointers to its input and output
 *    (row pitch `pitch` floats) and the CUDA stream to run on (NULL = the
 *    default stream); the current device is used.
 *  - The row-pass intermediate lives in a fixed array of
 *    PT_NOALLOC_MAX_PIXELS floats (4 MiB) in the library's device memory,
 *    which every GPU that loads the library holds until the process exits.
 *    pitch * h above that limit returns PT_ERR_INVALID.  Nothing is
 *    allocated or freed by the call.
 *  - Every call looks up the array's device address in the current
 *    device's context (cudaGetSymbolAddress), so the address stays right
 *    after a cudaDeviceReset.  The first call on a device also loads the
 *    library's device code there; make that first call outside any stream
 *    capture.
 *  - A CUDA error already pending on the calling thread is left in place
 *    and the call returns PT_ERR_CUDA without launching anything.
 *  - All calls share the one array and it keeps the last call's contents:
 *    calls that overlap on the GPU (different streams, or different host
 *    threads on one device) race on it and must be serialised by the caller.
 *    No element needs clearing: the column pass reads only what the row
 *    pass of the same call wrote. */
#define PT_NOALLOC_MAX_PIXELS (1 << 20)
pt_status pt_convolve_separable_noalloc(const float* src_dev, float* dst_dev, int w, int h, int pitch, int radius,
                                        void* stream);

/* ---- working-set level API (pyramids built and kept on the device) ----- */

/* Uploads one style exemplar at level-0 size and builds its pyramid on the
 * device (2x2 average for colours/DT, structure-tensor average then angle for
 * orientation, 2x2 majority vote for IDs; downsample.cpp:41-209,
 * GUI/nlDataAccess.cpp:82-93).  orient_tensor is (xx, xy, yy) per pixel; NULL
 * orient_tensor/dt/ids mean zero images, as the reference substitutes blank
 * images for missing elements (GUI/nlDataAccess.cpp:331-341). */
pt_status pt_set_style(pt_ctx* ctx, int style, int w, int h,
                       const float* base_rgba, const float* output_rgba,
                       const float* orient_tensor, const float* dist_trans,
                       const int32_t* object_ids);
/* Uploads the inputs of one frame at level-0 size and builds its pyramids on
 * the device; velocities are averaged and halved per level
 * (DOWNSAMPLE_SCALE_WITH_LEVELS, downsample.cpp:69-72).  NULL vel/scale mean
 * zero velocities / unit scale. Frames stay resident until pt_clear_frames. */
pt_status pt_set_frame(pt_ctx* ctx, int frame, int w, int h,
                       const float* rgba, const float* orient_tensor,
                       const float* dist_trans, const int32_t* object_ids,
                       const float* vel_fwd, const float* vel_bwd,
                       const float* scale);
/* Ribbon inputs of one frame (the shot's IN_RIBBON_F/B elements,
 * GUI/nlShot.cpp:160-190, nlDataAccess.cpp:160-210): velocities to the frame
 * `step` frames later (vel_fwd) and earlier (vel_bwd), step = 2, 4, 8 ...
 * TCTF runs over time steps up to the longest step every frame of the range
 * has; keyframe preprocessing accumulates ribbons over them. */
pt_status pt_set_frame_ribbons(pt_ctx* ctx, int frame, int step, int w, int h, const float* vel_fwd,
                               const float* vel_bwd);
pt_status pt_clear_frames(pt_ctx* ctx);

/* Level of the final output (copyOutputToFinal, synthesisProcessor.cpp:
 * 122-139, hands out level 0): FMBM, FMBM_RM and TCTF upsample their final
 * level down to level 0; IND and FBMO write no level-0 output in the
 * reference when finalLevel > 0, and here hand out their final level. */
#define PT_OUTPUT_LEVEL(params) \
    (((params)->scheme == PT_S_IND || (params)->scheme == PT_S_FBMO) ? (params)->finalLevel : 0)

/* Synthesises one still (renderAnimation with one frame,
 * synthesisProcessor.cpp:769-1312 for the scheme of pt_params.scheme).
 * Outputs at PT_OUTPUT_LEVEL; either output pointer may be NULL. */
pt_status pt_synthesize_frame(pt_ctx* ctx, int frame, float* out_rgba,
                              pt_patchxf* out_offsets);

/* Called once per frame with the final stylised output of the animation. */
typedef void (*pt_frame_callback)(int frame, const float* rgba,
                                  const pt_patchxf* offsets, int w, int h,
                                  void* user);
/* Synthesises frames first..last (all uploaded with pt_set_frame) with the
 * scheme of pt_params.scheme: FMBM(_RM) forward/backward consecutive passes
 * (synthesisProcessor.cpp:703-753,846-878), FBMO (:880-1022), TCTF
 * (:1047-1312, time steps from pt_set_frame_ribbons) or IND (:807-844). */
pt_status pt_synthesize_animation(pt_ctx* ctx, int first, int last,
                                  pt_frame_callback cb, void* user);

/* The final output (level PT_OUTPUT_LEVEL) of one frame of the last
 * pt_synthesize_frame / pt_synthesize_animation, copied into the caller's
 * buffers; either pointer may be NULL.  No counterpart in the reference
 * (its frames end up in EXR files): a caller that passes NULL as the
 * animation callback fetches frames with this call, straight into its own
 * (ideally page-locked) memory. */
pt_status pt_get_frame_result(pt_ctx* ctx, int frame, float* out_rgba, pt_patchxf* out_offsets);
/* The residual (patch energy per pixel) stored with a synthesised frame's
 * final offsets -- the reference saves it as the `residual` temporary image
 * of that pass (WorkingBuffers::saveTempImages, workingBuffers.cpp:242-296);
 * level-size float32, into caller memory. */
pt_status pt_get_frame_residual(pt_ctx* ctx, int frame, float* out_residual);

/* Measurement: the rate (GB/s) of 32-byte record gathers from an L2-resident
 * 32 MiB buffer on `device` -- the ceiling of the patch-distance kernels'
 * exemplar gathers -- with every lane at a random record (coherent = 0) or
 * each warp at a random run of consecutive records (coherent = 1).  CUDA
 * events around 10 launches after 3 warm-up launches.  No counterpart in the
 * reference. */
pt_status pt_measure_gather(int device, int coherent, double* out_gbs);

/* Page-locked host memory (cudaMallocHost / cudaFreeHost) for frame inputs
 * and results: copies from and to it run at the full host link speed.  No
 * counterpart in the reference. */
pt_status pt_host_alloc(size_t bytes, void** out);
pt_status pt_host_free(void* p);

/* ---- Serving: many requests on one GPU --------------------------------------
 * No counterpart in the reference, which runs one synthesis per process.
 * A request is a style plus one frame (a still) or several (a clip).
 * pt_serve runs up to max_in_flight requests at once, each on its own
 * context and CUDA stream, so the kernels of requests in flight overlap on
 * the GPU (a small request alone leaves most of it idle).  Requests are
 * admitted in arrival order once their arrival time has passed and their
 * device memory fits hbm_budget beside the requests in flight (0: no
 * budget): the running requests count with the memory their contexts
 * actually hold once set up (pt_device_bytes; admission waits for that),
 * the new one with an estimate from its sizes; a request larger than the
 * budget still runs, alone.  Each
 * result equals pt_synthesize_frame / pt_synthesize_animation of that request
 * on a context of its own.  Returns the first failing request's status, after
 * all requests have run. */
typedef struct {
    const float* rgba;           /* image_w x image_h RGBA (required) */
    const float* orient_tensor;  /* x3 structure tensor, or NULL */
    const float* dist_trans;     /* or NULL */
    const int32_t* ids;          /* or NULL */
    const float* vel_fwd;        /* x2, or NULL */
    const float* vel_bwd;        /* x2, or NULL */
    const float* scale;          /* x2, or NULL (1, 1) */
} pt_frame_inputs;

typedef struct {
    pt_params params;
    int style_w, style_h;
    const float* style_base;           /* RGBA */
    const float* style_output;         /* RGBA */
    const float* style_orient_tensor;  /* or NULL */
    const float* style_dist_trans;     /* or NULL */
    const int32_t* style_ids;          /* or NULL */
    int image_w, image_h, frames;
    const pt_frame_inputs* inputs;     /* `frames` entries */
    float* out_rgba;          /* frames x (image_h >> L) x (image_w >> L) x 4, or NULL; L = PT_OUTPUT_LEVEL */
    pt_patchxf* out_offsets;  /* frames x (image_h >> L) x (image_w >> L), or NULL */
    double arrival_ms;        /* arrival, in ms after pt_serve starts */
    double start_ms;          /* out: when its synthesis started */
    double done_ms;           /* out: when its results were written */
    pt_status status;         /* out */
    size_t device_bytes;      /* out: device memory its worker context held once the request was set up */
} pt_request;

pt_status pt_serve(int device, pt_request* requests, int count, int max_in_flight, size_t hbm_budget);

/* The same as a server that keeps its worker contexts (device buffers,
 * memory cache, CUDA streams) between runs, so that later runs skip their
 * set-up: create once, run any number of request lists, destroy. */
typedef struct pt_server pt_server;
pt_status pt_server_create(int device, int max_in_flight, size_t hbm_budget, pt_server** out);
pt_status pt_server_run(pt_server* server, pt_request* requests, int count);
pt_status pt_server_destroy(pt_server* server);

/* Number of this library's kernel launches issued so far by the context. */
uint64_t pt_kernel_launches(const pt_ctx* ctx);

/* ---- measurement (no counterpart in the reference, which has no GPU
 *      timers; its Stats/ScopeTimer are host wall clocks, stats.h:41-182) -- */
#define PT_TIMER_SLOTS 16
/* Records CUDA event `slot` (0..15) on the context's stream. */
pt_status pt_timer_record(pt_ctx* ctx, int slot);
/* Waits for both events and returns the time between them in ms. */
pt_status pt_timer_elapsed(pt_ctx* ctx, int slot_a, int slot_b, float* ms);

/* Kernels whose launches are timed when profiling is on. */
enum { PT_KERNEL_PROPAGATE = 0, PT_KERNEL_SCATTER = 1, PT_KERNEL_RESIDUAL = 2,
       PT_KERNEL_CANVAS = 3, PT_KERNEL_COUNT = 4 };
typedef struct {
    uint64_t launches;        /* launches since profiling was switched on */
    double total_ms;          /* sum of per-launch CUDA-event durations */
    uint64_t energy_evals;    /* patch-distance evaluations performed */
    uint64_t taps;            /* taps summed over those evaluations */
    uint64_t temporal_taps;   /* taps of evaluations with temporal terms */
} pt_kernel_stats;
/* Profiling of the patch-distance and canvas launches (clears the
 * statistics): flags = 0 (off) or a combination of PT_PROFILE_TIMING (a
 * CUDA event pair around every launch, read back as total_ms / launches)
 * and PT_PROFILE_COUNTERS (device-side counts of evaluations and taps, which
 * cost atomics inside the kernels). */
#define PT_PROFILE_TIMING 1
#define PT_PROFILE_COUNTERS 2
pt_status pt_set_profiling(pt_ctx* ctx, int flags);
/* Selects the kernels of the patch-distance passes: 1 (default) = the tiled
 * shared-memory kernels where an instantiation exists (patch radius 2-4, no
 * coherence term, one temporal direction), 0 = the generic kernels
 * everywhere.  Both compute identical results. */
pt_status pt_set_tiled_kernels(pt_ctx* ctx, int on);
/* Selects how the tiled kernels stage the pixel-side planes of a tile and
 * its halo in shared memory: 1 (default) = tensor copies
 * (cp.async.bulk.tensor, completed on an mbarrier) for every tile whose halo
 * lies inside the level rectangle, plain loads with the clamp rules for the
 * others; 0 = plain loads everywhere.  Both compute identical results.  A
 * block that gives up waiting for its copies (a bounded wait) makes the next
 * pt_synchronize / pt_synthesize_* return PT_ERR_CUDA. */
pt_status pt_set_tma_staging(pt_ctx* ctx, int on);
/* Warps per tile row of the tiled propagate kernel: 1 = one (a lane per
 * pixel), 2 = two (the second warp only evaluates candidates from the row's
 * queue: twice the lanes for the same candidates), 0 (default) = picked per
 * launch shape (radius, temporal mode, filter mode, tile count) by an
 * autotuner that times one launch of each.  All compute identical results. */
pt_status pt_set_propagate_lanes(pt_ctx* ctx, int warps_per_row);
/* Selects whether the propagate/scatter loops of pt_synthesize_frame and
 * pt_synthesize_animation track which offsets each pass changed and skip the
 * evaluations whose inputs are unchanged since an earlier pass with the same
 * candidates (1, default; tiled kernels only), or evaluate everything (0).
 * Both compute identical results.  No counterpart in the reference: its
 * loop (synthesisFrame.cpp:483-508) always evaluates everything. */
pt_status pt_set_incremental(pt_ctx* ctx, int on);
/* Statistics of one kernel (waits for the stream). */
pt_status pt_get_kernel_stats(pt_ctx* ctx, int kernel, pt_kernel_stats* out);
/* Blocks until the context's stream is idle. */
pt_status pt_synchronize(pt_ctx* ctx);

/* ---- file formats (host only) ---------------------------------------------
 * Decodes the Huffman block of an OpenEXR PIZ chunk (the stage that
 * OpenEXR's reader runs on the reference's PIZ-compressed RGBA temporaries,
 * imageIO.h:131-133): `block` holds the u32 header (first and last symbol,
 * table bytes, bit count, 0), the packed code-length table and the bits;
 * writes exactly n_words 16-bit words.  PT_ERR_INVALID for a malformed or
 * truncated block, or one that decodes to another count of words. */
pt_status pt_piz_huffman_decode(const uint8_t* block, size_t block_bytes, uint16_t* out, size_t n_words);

#ifdef __cplusplus
}
#endif

#endif /* PAINTTWEEN_GB300_H */
