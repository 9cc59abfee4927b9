/*
 * isti — GB300-native per-frame image-based spatio-temporal interpolation.
 *
 * C ABI of the interpolation path of the reference renderer
 * (DerThomy/ImageBasedSpatioTemporalInterpolation, src/renderer.cu).  The
 * entry points below replace, one for one:
 *
 *   isti_renderer_create / _destroy  <- Renderer::Renderer() (include/renderer.h:54)
 *                                        and its lazily allocated members
 *                                        (src/renderer.cu:549-605); the reference
 *                                        never frees them, this library does on destroy.
 *   isti_render                      <- Renderer::render(ImageBuffer<uchar4,4>&,
 *                                        const RenderInfo, const FrameData&)
 *                                        (include/renderer.h:56, src/renderer.cu:607-694)
 *   isti_frame_data / isti_view      <- FrameData / MotionZBufferImage / AuxCamData
 *                                        (include/data.h:12-116)
 *   isti_render_info                 <- RenderInfo / AdditionalRenderInfo
 *                                        (include/renderer.h:18-35)
 *   isti_renderer_view_buffers       <- read access to the private splat buffers and
 *                                        flow fields (include/renderer.h:64-92), for
 *                                        bit-exact checks
 *
 * Conventions
 *  - Pixel data lives in device memory, dense row-major, (x, y) at y*width + x;
 *    the structs themselves are host memory.  Reads outside an image return
 *    zero, as the reference's border-mode textures do.
 *  - Matrices are float[16], column-major (element row r, column c at [c*4+r]),
 *    the glm layout.
 *  - Work is enqueued on `stream` (a cudaStream_t, NULL = legacy default
 *    stream); no call blocks the host.  A renderer owns per-frame
 *    intermediates, so use one renderer per concurrently rendering stream.
 *  - Errors are returned, never thrown; isti_last_error() describes the last
 *    failure on the calling thread.
 *  - Arithmetic (isti_renderer_set_arithmetic): by default IEEE binary32 with
 *    every multiply and add rounded separately (no contraction), reproducible
 *    bit for bit on any host; or the reference GPU build's own arithmetic
 *    (-use_fast_math), which reproduces that build's results.
 */
#ifndef ISTI_H
#define ISTI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ISTI_ABI_VERSION 1
#define ISTI_MAX_AUX_CAMS 7

typedef enum isti_status
{
    ISTI_OK = 0,
    ISTI_ERR_INVALID_ARG = 1,
    ISTI_ERR_OOM = 2,
    ISTI_ERR_CUDA = 3,
    ISTI_ERR_TIMEOUT = 4,
    ISTI_ERR_UNSUPPORTED = 5
} isti_status;

/* RenderMode, include/renderer.h:9-16 */
typedef enum isti_render_mode
{
    ISTI_MODE_OURS = 0,
    ISTI_MODE_BACKWARD_BIDIRECTIONAL = 1,
    ISTI_MODE_BACKWARD_UNIDIRECTIONAL = 2,
    ISTI_MODE_SPLATTING = 3,
    ISTI_MODE_TIMEWARP = 4
} isti_render_mode;

/* Object-motion layout.  F32X4 is the reference's float4 image
 * (include/data.h:56); F16X3 is the compact half-precision xyz form, widened
 * exactly to float on load. */
typedef enum isti_motion_format
{
    ISTI_MOTION_NONE = 0,
    ISTI_MOTION_F32X4 = 1,
    ISTI_MOTION_F16X3 = 2
} isti_motion_format;

/* One camera at one keyframe (MotionZBufferImage, include/data.h:12-62). */
typedef struct isti_view
{
    uint32_t width, height;        /* 1..65535 */
    const void *color;             /* RGBA8, 4-byte aligned */
    const float *z;                /* NDC z in [-1, 1] */
    const void *motion;            /* NDC delta to the other keyframe, this view's
                                      viewproj; NULL = no object motion */
    int32_t motion_format;         /* isti_motion_format */
    const void *shadow_color_a;    /* RGBA8 or NULL (NULL disables soft shadows) */
    const void *shadow_color_b;    /* RGBA8 or NULL */
    const void *shadow_info;       /* RGBA8, RGB = 24-bit field of 2-bit levels;
                                      required when shadow_color_a is given */
    float viewproj[16];
    float inv_viewproj[16];
} isti_view;

/* FrameData (include/data.h:79-116): fwd = earlier keyframe, bwd = later one;
 * aux_curr[i] / aux_next[i] = aux camera i at those keyframes. */
typedef struct isti_frame_data
{
    isti_view fwd, bwd;
    int32_t num_aux;               /* 0..ISTI_MAX_AUX_CAMS */
    const isti_view *aux_curr;
    const isti_view *aux_next;
    const int32_t *aux_priority;   /* NULL = all 0 */
} isti_frame_data;

/* RenderInfo + AdditionalRenderInfo (include/renderer.h:18-35). */
typedef struct isti_render_info
{
    uint32_t width, height;        /* must equal the main keyframes' size */
    float alpha;                   /* interpolation factor t */
    float viewproj[16];            /* client camera */
    float inv_viewproj[16];
    int32_t frames_per_anchor;
    int32_t shadow_frames_per_anchor; /* 0..16 */
    int32_t no_shadows;
    int32_t mode;                  /* isti_render_mode */
} isti_render_info;

typedef struct isti_renderer isti_renderer;

int32_t isti_abi_version(void);
const char *isti_last_error(void);
const char *isti_status_string(isti_status s);

isti_status isti_renderer_create(isti_renderer **out);
isti_status isti_renderer_destroy(isti_renderer *r);

/* Renders one interpolated client frame into out_rgba (device, width*height
 * RGBA8).  Pixels without a valid result keep their previous content
 * (temporal hole filling, src/renderer.cu:416-419,462-463), so the caller
 * keeps the buffer alive across frames. */
isti_status isti_render(isti_renderer *r, void *out_rgba, const isti_render_info *info, const isti_frame_data *frame,
                        void *stream);

/* Renders n_frames client frames of one keyframe pair (several t values or
 * eyes) with one splat launch and one reprojection launch (no counterpart in
 * the reference, which renders frame by frame, src/main.cu:152-190).  Frame k
 * uses infos[k] (same width, height and mode for all k) and writes
 * out_rgba[k].  The result equals n_frames isti_render calls in order:
 *  - chain_outputs == 0: each out_rgba[k] is updated in place like a
 *    separate isti_render call on that buffer;
 *  - chain_outputs != 0: as if all frames went into one persistent buffer
 *    that starts as out_rgba[0]'s content and is copied to out_rgba[k] after
 *    frame k (out_rgba[k], k >= 1, is fully overwritten).
 * The work that does not depend on the client camera (world positions,
 * keyframe-to-keyframe flow) is done once for all frames.
 * 1 <= n_frames <= ISTI_MAX_BATCH_FRAMES. */
#define ISTI_MAX_BATCH_FRAMES 8
isti_status isti_render_batch(isti_renderer *r, int32_t n_frames, void *const *out_rgba, const isti_render_info *infos,
                              const isti_frame_data *frame, int32_t chain_outputs, void *stream);

/* The frames of several keyframe pairs in ONE persistent launch (no counterpart in the
 * reference, which renders frame by frame, src/main.cu:152-190).  pairs[i] renders
 * n_frames client frames of pairs[i].frame exactly as isti_render_batch would (same
 * chain_outputs meaning, same bits): key initialisation, splatting and reprojection of every
 * pair are units of one cooperative kernel that takes them from a device work queue, the
 * next pair's initialisation and splatting ahead of the previous pair's reprojection.  All
 * pairs share the render mode (not timewarp) and the number of source views.
 * 1 <= n_pairs <= ISTI_MAX_PAIRS.  The kernel parameters travel through pinned staging
 * buffers of the renderer, one for uncaptured and one for captured calls: a call captured
 * into a CUDA graph reads its buffer when the graph runs, so capture no other
 * isti_render_pairs call on that renderer while the graph is in use, and make one call of
 * the same size outside any capture first (a capture allocates nothing; a larger one is
 * refused with ISTI_ERR_INVALID_ARG).  isti_renderer_device_status reports the call's
 * status word. */
#define ISTI_MAX_PAIRS 64
typedef struct isti_pair_frames
{
    const isti_frame_data *frame;
    int32_t n_frames;               /* 1..ISTI_MAX_BATCH_FRAMES */
    void *const *out_rgba;          /* n_frames device RGBA8 buffers */
    const isti_render_info *infos;  /* n_frames */
    int32_t chain_outputs;
} isti_pair_frames;
isti_status isti_render_pairs(isti_renderer *r, int32_t n_pairs, const isti_pair_frames *pairs, void *stream);

/* Work-unit sizes of isti_render_pairs on this renderer: source rows per splat unit
 * (32 columns of one view, every frame; 1..256) and KiB of splat keys per init unit
 * (16..4096); 0 keeps a default (32 rows, 256 KiB).  The output does not depend on them. */
isti_status isti_renderer_set_pair_units(isti_renderer *r, int32_t splat_rows, int32_t init_unit_kib);

/* Device pointers to the intermediates of the last render call for view
 * `view` (0 fwd, 1 bwd, 2+2i aux i curr, 3+2i aux i next; after a batch,
 * frame k's views follow at k * (2 + 2 * num_aux)): 64-bit splat keys
 * (depth bits << 32 | x << 16 | y), the f32x2 (x, y) of the source->client
 * flow and the f32x4 source->other-keyframe flow (shared by the frames of a
 * batch), each width*height elements.  The reference keeps the client flow
 * as f32x4 (x, y, dz, visible); its other two parts are read by
 * isti_renderer_view_depth.  A field that is not materialised is returned as
 * NULL.  Valid until the next render or destroy. */
isti_status isti_renderer_view_buffers(const isti_renderer *r, int32_t view, const uint64_t **splat, const float **cam_xy,
                                       const float **full_ff, uint32_t *width, uint32_t *height);

/* The rest of the client flow of the same view: per source pixel the depth the
 * reprojection derives from it, z_to_depth(z + dz) (src/renderer.cu:339, the
 * reference's rounding: dz first, then the sum), f32, and visible_in_main as
 * one byte (0 / 1, the reference flow's w; shared by the frames of a batch),
 * each width*height elements.  NULL when not materialised. */
isti_status isti_renderer_view_depth(const isti_renderer *r, int32_t view, const float **cam_depth, const uint8_t **visible);

/* Per-stage device time (no counterpart in the reference, which has no
 * timers): when enabled, each render records CUDA events around the key
 * initialisation, the splat launch and the reprojection launch on its stream. */
typedef struct isti_timing
{
    int32_t frames;          /* renders timed since the previous query */
    int32_t kernel_launches; /* launches of this library's kernels in those renders */
    float init_ms;           /* summed device time of the splat-key initialisation */
    float splat_ms;          /* summed device time of the splat kernel */
    float reproj_ms;         /* summed device time of the reprojection kernel */
} isti_timing;

/* Device-side status of the last render call (no counterpart in the reference):
 * waits for the device, then stores ISTI_OK, or ISTI_ERR_TIMEOUT when a bounded
 * wait inside a kernel gave up (its frame is then not trustworthy). */
isti_status isti_renderer_device_status(isti_renderer *r, int32_t *device_status);

/* Arithmetic of a renderer's kernels (no counterpart in the reference, which has one
 * build).  ISTI_ARITH_IEEE (the default): every float operation correctly rounded
 * and none contracted, in the reference source's operation order -- the results
 * equal the reference's code executed under IEEE rules (on a CPU) bit for bit.
 * ISTI_ARITH_REFERENCE_GPU: the kernels compiled as the reference compiles its
 * renderer (-use_fast_math, CMakeLists.txt:36: approximate division and square
 * root, flushed denormals, contracted multiply-adds) with the reference's
 * expression trees -- the results follow the reference's own GPU build.  Takes
 * effect from the next render; autotuning results are dropped on a change. */
typedef enum isti_arithmetic
{
    ISTI_ARITH_IEEE = 0,
    ISTI_ARITH_REFERENCE_GPU = 1
} isti_arithmetic;
isti_status isti_renderer_set_arithmetic(isti_renderer *r, int32_t arith);

/* Failure-detection test hook (no counterpart in the reference).  From the next
 * render on, the reprojection block that covers output pixel (x, y) announces its
 * splat-key tiles but issues no copy, so its bounded wait runs out after
 * `wait_limit` polls (0: the default limit, seconds at most): the block sets
 * ISTI_ERR_TIMEOUT in the device status word and leaves without reading a tile or
 * writing a pixel; every other block renders normally.  Only renders that fetch
 * their tiles by TMA have such a wait.  x < 0 switches the hook off. */
isti_status isti_renderer_test_withhold_tile(isti_renderer *r, int32_t x, int32_t y, uint32_t wait_limit);

/* Failure-detection test hook for isti_render_pairs (no counterpart in the reference).
 * From the next isti_render_pairs call on, the reprojection units of pair `pair` wait for
 * one splat unit more than the pair has, so that dependency wait runs out after
 * `spin_limit` polls (0: the default limit, about two seconds): the unit sets
 * ISTI_ERR_TIMEOUT in the device status word and is skipped, and every unit that starts
 * after that only counts itself done.  pair < 0 switches the hook off. */
isti_status isti_renderer_test_stall_pair(isti_renderer *r, int32_t pair, uint32_t spin_limit);

isti_status isti_renderer_enable_timing(isti_renderer *r, int32_t on);
/* Waits for the recorded events, returns the sums and resets them. */
isti_status isti_renderer_timing(isti_renderer *r, isti_timing *out);

/* Autotuning of the reprojection launch (no counterpart in the reference, which has one
 * launch shape).  With autotuning on, the first uncaptured render of each shape class
 * (mode, source views, frames per call, render size, shadows present) also times every
 * candidate launch of its reprojection -- register cap x output row pairs per block x
 * key tiles staged by TMA copies or by plain loads -- on the call's stream, waits for them (one host synchronisation per class), and the
 * class's later renders, captured ones included, use the fastest.  Every candidate
 * computes the same result and the reprojection rewrites its outputs identically when
 * repeated, so the output does not depend on the choice.  Off (the default): a fixed
 * rule measured on GB300 (register cap by window size, view count and the resident blocks
 * the call's shared memory allows; output row pairs by views and frames per call).
 * Chained calls of several frames use at most one output row per source view in a block
 * (row pairs <= views / 2), whatever is asked for. */
isti_status isti_renderer_set_autotune(isti_renderer *r, int32_t on);

/* Pins the reprojection launch of every later render (no counterpart in the reference):
 * register cap (40 or 48 for the 3x3 window, 56 for the 7x7 window; 0: the rule's), output
 * row pairs per block (1..3; 0: the rule's) and key tiles by plain loads (1) or TMA copies
 * where the views allow them (0).  A cap the render mode is not built with takes the mode's
 * own (48 for the 3x3 window, 56 for the 7x7).  A pinned launch takes precedence over a
 * tuned one.  The output does not depend on it.  ISTI_ERR_INVALID_ARG for other values. */
isti_status isti_renderer_set_reproj_launch(isti_renderer *r, int32_t regs, int32_t row_pairs, int32_t plain_tiles);

typedef struct isti_tuning
{
    int32_t mode, n_views, n_frames, shadows; /* the shape class */
    uint32_t width, height;
    int32_t regs, row_pairs;                  /* the chosen launch: register cap, output row pairs per block */
    float best_ms, rule_ms;                   /* reprojection time of the choice and of the fixed rule */
    int32_t plain_tiles;                      /* 1: key tiles by plain loads instead of TMA copies */
} isti_tuning;

/* Number of tuned shape classes, and the index-th of them (0-based, in tuning order). */
isti_status isti_renderer_tuning_count(const isti_renderer *r, int32_t *count);
isti_status isti_renderer_tuning(const isti_renderer *r, int32_t index, isti_tuning *out);

/* Render without allocating (no counterpart in the reference, whose Renderer
 * always allocates its own buffers).
 *
 * For callers that must not allocate device memory while they run: hosts
 * whose device-memory budget is fully reserved up front by their own pool,
 * and real-time loops (a compositor or serving thread with a per-frame
 * deadline) where cudaMalloc/cudaFree may synchronise the device and take
 * unbounded time.  Same inputs, output and semantics as isti_render, but no
 * renderer handle: the splat keys and flow fields live in one fixed device
 * array inside this library (ISTI_NOALLOC_SCRATCH_BYTES, held by every GPU
 * that loads the library until the process exits).
 *
 *  - Limit: the sum over source views of width*height*37 bytes and
 *    (width+height)*4 bytes (each buffer rounded up to 256 bytes) must fit in
 *    ISTI_NOALLOC_SCRATCH_BYTES minus the 256 bytes of its status word, e.g.
 *    640x360 with up to two aux cameras; larger frames are rejected with
 *    ISTI_ERR_INVALID_ARG.
 *  - A call made outside a stream capture looks up the array's device address
 *    (with the device current) and remembers it; a captured call uses the
 *    remembered one.  So make the first call on a device, and the first call
 *    after a device reset, before any stream capture.
 *  - Every call uses the same array and re-initialises the keys itself; calls
 *    whose work overlaps on the GPU (other streams, other threads) race on it,
 *    so serialise them. */
#define ISTI_NOALLOC_SCRATCH_BYTES (64u << 20)
isti_status isti_render_noalloc(void *out_rgba, const isti_render_info *info, const isti_frame_data *frame, void *stream);

/* Device-side status of the last isti_render_noalloc call on the current device
 * (the counterpart of isti_renderer_device_status for the call without a
 * renderer): waits for the device, then stores ISTI_OK, or ISTI_ERR_TIMEOUT when
 * a bounded wait inside a kernel gave up (that frame is then not trustworthy).
 * The word sits at a fixed place in the scratch array; the next call resets it. */
isti_status isti_noalloc_device_status(int32_t *device_status);

#ifdef __cplusplus
}
#endif
#endif
