/*
 * CPU oracle for the per-frame interpolation path of the reference renderer
 * (src/renderer.cu:65-465 and the math of include/util/helper_common.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline / reference legs of bench.py may load this library, and only
 * as the checker or as the timed CPU baseline.  The product path never calls
 * it: the CUDA extension fails loudly when it is missing.
 *
 * Arithmetic: IEEE-754 binary32, round-to-nearest, no fused multiply-add
 * (built with -ffp-contract=off), in the operation order of the reference's
 * source and of the glm subset in ref_host/glm/glm.hpp.  Float->int
 * conversions follow the PTX rules the GPU applies (truncation toward zero,
 * saturation, NaN -> 0).
 *
 * Images are dense row-major arrays, (x, y) at y * width + x.  A read outside
 * an image returns zero, which is what the reference's border-mode textures
 * return (src/util/image_buffer.cu:227-249).
 */
#ifndef ISTI_ORACLE_H
#define ISTI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One source view: one camera at one keyframe (reference MotionZBufferImage,
 * include/data.h:12-62).  Matrices are column-major, element (row r, col c)
 * at [c * 4 + r]. */
typedef struct oracle_view
{
    uint32_t width, height;
    const uint8_t *color;          /* RGBA8 */
    const float *z;                /* NDC z in [-1, 1] */
    const float *motion;           /* f32x4 NDC delta to the other keyframe (w unused); NULL = none */
    const uint8_t *shadow_color_a; /* RGBA8 or NULL */
    const uint8_t *shadow_color_b; /* RGBA8 or NULL */
    const uint8_t *shadow_info;    /* RGBA8, RGB = 24-bit field of 2-bit levels; NULL when A is NULL */
    float viewproj[16];
    float inv_viewproj[16];
} oracle_view;

/* Reference FrameData (include/data.h:79-116): the two bracketing keyframes
 * of the main camera plus aux cameras (curr = earlier, next = later). */
typedef struct oracle_frame
{
    oracle_view fwd, bwd;
    int32_t num_aux;
    const oracle_view *aux_curr;
    const oracle_view *aux_next;
    const int32_t *aux_priority;
} oracle_frame;

/* Reference RenderInfo + AdditionalRenderInfo (include/renderer.h:18-35). */
typedef struct oracle_render_info
{
    uint32_t width, height;
    float alpha;
    float viewproj[16];
    float inv_viewproj[16];
    int32_t frames_per_anchor;
    int32_t shadow_frames_per_anchor;
    int32_t no_shadows;
    int32_t mode; /* 0 OURS, 1 BACKWARD_BIDIRECTIONAL, 2 BACKWARD_UNIDIRECTIONAL, 3 SPLATTING, 4 TIMEWARP */
} oracle_render_info;

/* Per-view intermediates, each NULL or width*height elements of the view:
 * splat = 64-bit keys, cam_ff / full_ff = f32x4 flow fields (source -> client
 * camera, source -> other keyframe).  View order: fwd, bwd, then aux i
 * curr, aux i next. */
typedef struct oracle_view_out
{
    uint64_t *splat;
    float *cam_ff;
    float *full_ff;
} oracle_view_out;

/* Renders one interpolated frame into out_rgba (width*height RGBA8, updated
 * in place: pixels without a valid result keep their previous value).
 * outs may be NULL; when given it has 2 + 2 * num_aux entries, and entries
 * that are NULL are computed in scratch memory.  nthreads <= 0 uses all
 * OpenMP threads.  Returns 0, or -1 on invalid arguments / allocation
 * failure. */
int oracle_render(const oracle_frame *frame, const oracle_render_info *info, uint8_t *out_rgba, oracle_view_out *outs, int nthreads);

/* Individual device functions, exposed for unit tests. */
uint64_t oracle_encode_key(float depth, uint32_t x, uint32_t y);
void oracle_decode_key(uint64_t key, float *depth, uint32_t *x, uint32_t *y);

#ifdef __cplusplus
}
#endif
#endif
