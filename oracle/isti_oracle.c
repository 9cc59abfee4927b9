/*
 * CPU oracle: a plain C restatement of the reference's per-frame
 * interpolation path (src/renderer.cu, include/util/helper_common.h,
 * include/util/helper_math.h).  TEST INFRASTRUCTURE ONLY: it is the checker
 * of the CUDA kernels and the timed CPU baseline, never part of the product.
 *
 * Build: gcc -std=c11 -O2 -ffp-contract=off -fopenmp -fPIC -shared.
 * -ffp-contract=off keeps every multiply and add separately rounded, which is
 * the arithmetic the CUDA kernels use (nvcc -fmad=false), so both sides give
 * bit-identical floats.  See isti_oracle.h for conventions.
 */
#include "isti_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/renderer.cu:16-28 */
static const float EPS_1_FULL_RES = 0.002f;
#define EPS_1_LOW_RES (0.002f * 4.0f) /* EPS_1_FULL_RES * 4.0f, evaluated in float */
static const float EPS_2_FULL_RES = 0.001f;
static const float EPS_2_LOW_RES = 0.004f;
static const float EPS_3 = 0.01f;
#define SPLAT_INIT_BYTE 0xfe
#define SOFTSHADOW_BITS 2u
#define SOFTSHADOW_VAL_MASK 3u

typedef struct { float x, y; } f2;
typedef struct { float x, y, z; } f3;
typedef struct { float x, y, z, w; } f4;
typedef struct { int32_t x, y; } i2;
typedef struct { uint32_t x, y; } u2;
typedef struct { uint8_t x, y, z, w; } c4;

/* ---- PTX float->int conversion rules (truncate, saturate, NaN -> 0) ---- */

static int32_t cvt_s32(float f)
{
    if (f != f)
        return 0;
    if (f >= 2147483648.0f)
        return INT32_MAX;
    if (f <= -2147483648.0f)
        return INT32_MIN;
    return (int32_t)f;
}

static uint8_t cvt_u8(float f)
{
    if (f != f || f <= 0.0f)
        return 0;
    if (f >= 255.0f)
        return 255;
    return (uint8_t)f;
}

static uint32_t sat_u32(double r)
{
    if (r != r || r <= 0.0)
        return 0u;
    if (r >= 4294967295.0)
        return 4294967295u;
    return (uint32_t)r;
}
static uint32_t f2u_rn(float x) { return sat_u32(nearbyint((double)x)); }
static uint32_t f2u_rd(float x) { return sat_u32(floor((double)x)); }
static uint32_t f2u_ru(float x) { return sat_u32(ceil((double)x)); }

/* PTX shr.b32: shift amounts >= 32 give 0 */
static uint32_t shr32(uint32_t v, uint32_t s) { return s >= 32u ? 0u : (v >> s); }

/* ---- include/util/helper_common.h ---- */

static int in_range(i2 p, u2 dims) /* :8-11 */
{
    return p.x >= 0 && (uint32_t)p.x < dims.x && p.y >= 0 && (uint32_t)p.y < dims.y;
}

static f2 pixel2CS(u2 p, u2 res) /* :66-69  2 * (p + 0.5) / res - 1 */
{
    f2 a = {(float)p.x + 0.5f, (float)p.y + 0.5f};
    a.x = 2.0f * a.x;
    a.y = 2.0f * a.y;
    a.x = a.x / (float)res.x;
    a.y = a.y / (float)res.y;
    a.x = a.x - 1.0f;
    a.y = a.y - 1.0f;
    return a;
}

static i2 CS2pixel(f2 cs, u2 res) /* :71-75  floor((cs + 1) * res * 0.5) */
{
    f2 a = {cs.x + 1.0f, cs.y + 1.0f};
    a.x = a.x * (float)res.x;
    a.y = a.y * (float)res.y;
    a.x = a.x * 0.5f;
    a.y = a.y * 0.5f;
    i2 r = {cvt_s32(floorf(a.x)), cvt_s32(floorf(a.y))};
    return r;
}

/* mat4 * vec4 in the glm-subset order: (m0*x + m1*y) + (m2*z + m3*w) */
static f4 matvec(const float *m, f4 v)
{
    f4 r;
    float a, b;
    a = m[0] * v.x + m[4] * v.y;
    b = m[8] * v.z + m[12] * v.w;
    r.x = a + b;
    a = m[1] * v.x + m[5] * v.y;
    b = m[9] * v.z + m[13] * v.w;
    r.y = a + b;
    a = m[2] * v.x + m[6] * v.y;
    b = m[10] * v.z + m[14] * v.w;
    r.z = a + b;
    a = m[3] * v.x + m[7] * v.y;
    b = m[11] * v.z + m[15] * v.w;
    r.w = a + b;
    return r;
}

static f4 project(const float *m, f4 v) /* CS2WS / WS2CS :77-87 : (M v) / (M v).w */
{
    f4 p = matvec(m, v);
    f4 r = {p.x / p.w, p.y / p.w, p.z / p.w, p.w / p.w};
    return r;
}

static float z_to_depth(float z) { return (z + 1.0f) * 0.5f; } /* :89-91 */
static float depth_to_z(float d) { return d * 2.0f - 1.0f; }   /* :93-95 */

/* lerp_color :22-25 : (a + t * (b - a)) / 255 */
static f4 lerp_color(c4 a, c4 b, float t)
{
    f4 r;
    r.x = ((float)a.x + t * ((float)b.x - (float)a.x)) / 255.f;
    r.y = ((float)a.y + t * ((float)b.y - (float)a.y)) / 255.f;
    r.z = ((float)a.z + t * ((float)b.z - (float)a.z)) / 255.f;
    r.w = ((float)a.w + t * ((float)b.w - (float)a.w)) / 255.f;
    return r;
}

static uint8_t to_8bit(float f) /* :27-30  min(255, max(0, int(f * 255))) */
{
    int32_t v = cvt_s32(f * 255.f);
    v = v < 0 ? 0 : v;
    return (uint8_t)(v > 255 ? 255 : v);
}

static c4 color_to_uchar4(f4 c)
{
    c4 r = {to_8bit(c.x), to_8bit(c.y), to_8bit(c.z), to_8bit(c.w)};
    return r;
}

/* ---- border-addressed image reads (zero outside) ---- */

static float ld_f(const float *img, u2 dims, u2 p)
{
    return (p.x < dims.x && p.y < dims.y) ? img[(size_t)p.y * dims.x + p.x] : 0.0f;
}
static f4 ld_f4(const float *img, u2 dims, u2 p)
{
    f4 r = {0.f, 0.f, 0.f, 0.f};
    if (p.x < dims.x && p.y < dims.y)
        memcpy(&r, img + 4 * ((size_t)p.y * dims.x + p.x), sizeof r);
    return r;
}
static c4 ld_c4(const uint8_t *img, u2 dims, u2 p)
{
    c4 r = {0, 0, 0, 0};
    if (img && p.x < dims.x && p.y < dims.y)
        memcpy(&r, img + 4 * ((size_t)p.y * dims.x + p.x), sizeof r);
    return r;
}

/* ---- keys, src/renderer.cu:65-74 ---- */

typedef struct
{
    float depth;
    u2 source_pixel;
} key_info;

static uint32_t f_bits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static float bits_f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

uint64_t oracle_encode_key(float depth, uint32_t x, uint32_t y)
{
    return ((uint64_t)f_bits(depth) << 32) | (uint64_t)((x << 16) | y);
}

static key_info decode_key(uint64_t key)
{
    key_info k;
    k.depth = bits_f((uint32_t)(key >> 32));
    k.source_pixel.x = ((uint32_t)key) >> 16;
    k.source_pixel.y = (uint32_t)(key & 0xFFFFull);
    return k;
}

void oracle_decode_key(uint64_t key, float *depth, uint32_t *x, uint32_t *y)
{
    key_info k = decode_key(key);
    *depth = k.depth;
    *x = k.source_pixel.x;
    *y = k.source_pixel.y;
}

static void atomic_min_u64(uint64_t *p, uint64_t v)
{
    uint64_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < old && !__atomic_compare_exchange_n(p, &old, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
    {
    }
}

/* ---- per-view state (reference CamReprojInfo, include/renderer.h:37-50) ---- */

typedef struct
{
    const oracle_view *v;
    u2 dims;
    int forward;
    int priority;
    uint64_t *splat;
    float *cam_ff;
    float *full_ff;
    /* splat-time parameters (src/renderer.cu:643-649) */
    float weight;
    const float *vp_to;
    const float *vp_from_main;
} view_ctx;

/* computeFlowFields_sortedSplatting_kernel, src/renderer.cu:76-146 */
static void splat_pixel(const view_ctx *c, const float *vp_cam, int linear, uint32_t x, uint32_t y)
{
    const oracle_view *v = c->v;
    const u2 dims = c->dims;
    const size_t idx = (size_t)y * dims.x + x;
    const u2 px = {x, y};

    const float z_from = v->z[idx];
    f4 om = {0.f, 0.f, 0.f, 0.f};
    if (v->motion)
        memcpy(&om, v->motion + 4 * idx, sizeof om);

    const f2 pcs = pixel2CS(px, dims);
    const f4 posCS_from = {pcs.x, pcs.y, z_from, 1.0f};
    const f4 posWS_from = project(v->inv_viewproj, posCS_from);
    const f4 moved = {posCS_from.x + om.x, posCS_from.y + om.y, posCS_from.z + om.z, posCS_from.w + 0.0f};
    const f4 posWS_to = project(v->inv_viewproj, moved);

    const f4 cm = project(c->vp_from_main, posWS_from);
    const float lim = 1.0f - 1e-3f;
    const int visible = cm.x > -lim && cm.x < lim && cm.y > -lim && cm.y < lim && cm.z > -lim && cm.z < lim;

    const float wgt = c->weight;
    const f4 scaled = {posWS_from.x + wgt * (posWS_to.x - posWS_from.x), posWS_from.y + wgt * (posWS_to.y - posWS_from.y),
                       posWS_from.z + wgt * (posWS_to.z - posWS_from.z), posWS_from.w + wgt * (posWS_to.w - posWS_from.w)};
    const f4 posCS_to = project(c->vp_to, posWS_to);
    const f4 fm = {posCS_to.x - posCS_from.x, posCS_to.y - posCS_from.y, posCS_to.z - posCS_from.z, posCS_to.w - posCS_from.w};
    float *ff = c->full_ff + 4 * idx;
    ff[0] = fm.x;
    ff[1] = fm.y;
    ff[2] = fm.z;
    ff[3] = visible ? 1.0f : 0.0f;

    float depth = z_to_depth(posCS_from.z);
    u2 pix = px;
    float *cf = c->cam_ff + 4 * idx;
    if (!linear)
    {
        const f4 pc = project(vp_cam, scaled);
        cf[0] = pc.x - posCS_from.x;
        cf[1] = pc.y - posCS_from.y;
        cf[2] = pc.z - posCS_from.z;
        cf[3] = visible ? 1.0f : 0.0f;
        const float depth_cam = z_to_depth(pc.z);
        const f2 pcxy = {pc.x, pc.y};
        const i2 pixel_cam = CS2pixel(pcxy, dims);
        if (!in_range(pixel_cam, dims) || depth_cam < 0.0f)
            return;
        depth = depth_cam;
        pix.x = (uint32_t)pixel_cam.x;
        pix.y = (uint32_t)pixel_cam.y;
    }
    else
    {
        cf[0] = fm.x * wgt;
        cf[1] = fm.y * wgt;
        cf[2] = fm.z * wgt;
        cf[3] = visible ? 1.0f : 0.0f;
    }
    atomic_min_u64(&c->splat[(size_t)pix.y * dims.x + pix.x], oracle_encode_key(depth, x, y));
}

/* initializeSearchFromSplatting<W>, src/renderer.cu:148-175 */
static key_info init_search(u2 idx, u2 res, const uint64_t *splat, int W)
{
    key_info lowest = decode_key(splat[(size_t)idx.y * res.x + idx.x]);
    for (int yo = -W; yo <= W; yo++)
        for (int xo = -W; xo <= W; xo++)
        {
            const i2 n = {(int32_t)idx.x + xo, (int32_t)idx.y + yo};
            if (!in_range(n, res))
                continue;
            const key_info cur = decode_key(splat[(size_t)n.y * res.x + n.x]);
            if (cur.depth > 0.0f && (!isfinite(lowest.depth) || lowest.depth < 0.0f || cur.depth < lowest.depth))
                lowest = cur;
        }
    return lowest;
}

/* iterativeSearch<N>, src/renderer.cu:177-202 */
static u2 iterative_search(u2 start, u2 idx, u2 res, u2 low_res, const float *ff, int N)
{
    u2 result = start;
    for (int i = 0; i < N; i++)
    {
        const f4 m = ld_f4(ff, low_res, result);
        const f2 p = pixel2CS(idx, res);
        const f2 q = {p.x - m.x, p.y - m.y};
        const i2 t = CS2pixel(q, low_res);
        if (!in_range(t, low_res))
            continue;
        result.x = (uint32_t)t.x;
        result.y = (uint32_t)t.y;
    }
    return result;
}

/* computeReprojError, src/renderer.cu:204-215 */
static float reproj_error(u2 pixel_from, u2 res_from, f2 pcs_cam, f4 m)
{
    const f2 pf = pixel2CS(pixel_from, res_from);
    f2 e = {(pf.x + m.x) - pcs_cam.x, (pf.y + m.y) - pcs_cam.y};
    const uint32_t mn = res_from.x < res_from.y ? res_from.x : res_from.y;
    const f2 s = {(float)res_from.x / (float)mn, (float)res_from.y / (float)mn};
    e.x = e.x * s.x;
    e.y = e.y * s.y;
    return sqrtf(e.x * e.x + e.y * e.y);
}

/* colorFromShadow (level index form), src/renderer.cu:217-268 */
static c4 color_from_shadow_idx(uint32_t sidx, int32_t sfpa, const view_ctx *c, u2 p)
{
    const oracle_view *v = c->v;
    const c4 main_color = ld_c4(v->color, c->dims, p);
    if (sidx < (uint32_t)sfpa && sidx > 0)
    {
        const c4 si = ld_c4(v->shadow_info, c->dims, p);
        const uint32_t bf = ((uint32_t)si.x << 16) | ((uint32_t)si.y << 8) | (uint32_t)si.z;
        if (v->shadow_color_b)
        {
            if (bf != 0)
            {
                const int32_t init_val = (int32_t)(bf & SOFTSHADOW_VAL_MASK);
                const int32_t my_val = (int32_t)(shr32(bf, SOFTSHADOW_BITS * sidx) & SOFTSHADOW_VAL_MASK);
                int32_t mn = (int32_t)SOFTSHADOW_VAL_MASK, mx = 0;
                for (int32_t i = 0; i < sfpa; i++)
                {
                    const int32_t lv = (int32_t)(shr32(bf, SOFTSHADOW_BITS * (uint32_t)i) & SOFTSHADOW_VAL_MASK);
                    mn = lv < mn ? lv : mn;
                    mx = lv > mx ? lv : mx;
                }
                const float t = (float)(my_val - mn) / (float)(mx - mn);
                const c4 cmin = mn == init_val ? main_color : ld_c4(v->shadow_color_a, c->dims, p);
                const c4 cmax = mx == init_val ? main_color : ld_c4(v->shadow_color_b, c->dims, p);
                const float omt = (float)(1.0 - (double)t);
                c4 r;
                r.x = cvt_u8((float)cmin.x * omt + (float)cmax.x * t);
                r.y = cvt_u8((float)cmin.y * omt + (float)cmax.y * t);
                r.z = cvt_u8((float)cmin.z * omt + (float)cmax.z * t);
                r.w = 255;
                return r;
            }
        }
    }
    return main_color;
}

static uint32_t frame_idx_to_idx(int forward, int32_t frame_idx, int32_t fpa) /* :227-230 */
{
    return (uint32_t)(forward ? frame_idx : (fpa - frame_idx));
}

/* colorFromShadow (two sub-frame form), src/renderer.cu:270-295 */
static c4 color_from_shadow(u2 sf, float sf_t, const oracle_render_info *s, const view_ctx *c, u2 p)
{
    if (s->no_shadows || sf.x >= (uint32_t)s->shadow_frames_per_anchor || sf.y == 0 || !c->v->shadow_color_a)
        return ld_c4(c->v->color, c->dims, p);
    const int32_t sfpa = s->shadow_frames_per_anchor;
    const u2 vi = {frame_idx_to_idx(c->forward, (int32_t)sf.x, sfpa), frame_idx_to_idx(c->forward, (int32_t)sf.y, sfpa)};
    if (vi.x == vi.y || vi.y >= (uint32_t)sfpa)
        return color_from_shadow_idx(vi.x, sfpa, c, p);
    if (vi.x >= (uint32_t)sfpa)
        return color_from_shadow_idx(vi.y, sfpa, c, p);
    const c4 a = color_from_shadow_idx(vi.x, sfpa, c, p);
    const c4 b = color_from_shadow_idx(vi.y, sfpa, c, p);
    return color_to_uchar4(lerp_color(a, b, sf_t));
}

/* secondChanceAndBlend_kernel<EPS_2>, src/renderer.cu:297-327 */
static c4 second_chance(float weight, uint32_t frame_idx, u2 sf, float sf_t, key_info info, const oracle_render_info *s,
                        const view_ctx *from, const view_ctx *to, float eps2)
{
    const f4 m_ft = ld_f4(from->full_ff, from->dims, info.source_pixel);
    const f2 spcs = pixel2CS(info.source_pixel, from->dims);
    const f3 sourceCS = {spcs.x, spcs.y, ld_f(from->v->z, from->dims, info.source_pixel)};
    const f3 projCS = {sourceCS.x + m_ft.x, sourceCS.y + m_ft.y, sourceCS.z + m_ft.z};
    const f2 pxy = {projCS.x, projCS.y};
    const i2 proj_pixel = CS2pixel(pxy, to->dims);

    c4 out = color_from_shadow(sf, sf_t, s, from, info.source_pixel);
    if (frame_idx >= (uint32_t)s->frames_per_anchor)
        return out;
    if (in_range(proj_pixel, to->dims))
    {
        const u2 pp = {(uint32_t)proj_pixel.x, (uint32_t)proj_pixel.y};
        const float actual_z = ld_f(to->v->z, to->dims, pp);
        const f4 m_tf = ld_f4(to->full_ff, to->dims, pp);
        const f3 d = {m_ft.x - (-m_tf.x), m_ft.y - (-m_tf.y), m_ft.z - (-m_tf.z)};
        const float dist = sqrtf((d.x * d.x + d.y * d.y) + d.z * d.z);
        if (dist < EPS_3 && fabsf(actual_z - projCS.z) < eps2)
            out = color_to_uchar4(lerp_color(color_from_shadow(sf, sf_t, s, to, pp), out, weight));
    }
    return out;
}

/* ReprojResult, src/renderer.cu:49-57.  Fields the reference leaves
 * indeterminate (error/depth of the always-valid blend) are 0 here. */
typedef struct
{
    int valid;
    int visible_in_main;
    int priority;
    float error;
    float depth;
    c4 color;
} reproj_result;

/* bidirectionalReprojection<SW, SI, ALWAYS_VALID, EPS_1, EPS_2>, src/renderer.cu:329-398 */
static reproj_result bidir(int SW, int SI, int always_valid, float eps1, float eps2, u2 idx, u2 full_res_idx, u2 full_res,
                           float alpha, f2 pcs, const oracle_render_info *s, const view_ctx *fwd, const view_ctx *bwd)
{
    float fwd_e = FLT_MAX;
    int fwd_vis = 0;
    key_info fi = init_search(idx, fwd->dims, fwd->splat, SW);
    if (fi.depth > 0.0f && alpha < 1.0f)
    {
        fi.source_pixel = iterative_search(fi.source_pixel, full_res_idx, full_res, fwd->dims, fwd->cam_ff, SI);
        const f4 m = ld_f4(fwd->cam_ff, fwd->dims, fi.source_pixel);
        fi.depth = z_to_depth(ld_f(fwd->v->z, fwd->dims, fi.source_pixel) + m.z);
        fwd_e = reproj_error(fi.source_pixel, fwd->dims, pcs, m);
        fwd_vis = m.w > 0.0f;
    }

    float bwd_e = FLT_MAX;
    int bwd_vis = 0;
    key_info bi = init_search(idx, bwd->dims, bwd->splat, SW);
    if (bi.depth > 0.0f)
    {
        bi.source_pixel = iterative_search(bi.source_pixel, full_res_idx, full_res, bwd->dims, bwd->cam_ff, SI);
        const f4 m = ld_f4(bwd->cam_ff, bwd->dims, bi.source_pixel);
        bi.depth = z_to_depth(ld_f(bwd->v->z, bwd->dims, bi.source_pixel) + m.z);
        bwd_e = reproj_error(bi.source_pixel, bwd->dims, pcs, m);
        bwd_vis = m.w > 0.0f;
    }

    const uint32_t frame_idx = f2u_rn((float)s->frames_per_anchor * alpha);
    const u2 sf = {f2u_rd((float)s->shadow_frames_per_anchor * alpha + 1e-9f), f2u_ru((float)s->shadow_frames_per_anchor * alpha - 1e-9f)};
    const float sf_t = (float)s->shadow_frames_per_anchor * alpha - (float)sf.x;

    reproj_result r = {0, 0, 0, 0.0f, 0.0f, {0, 0, 0, 0}};
    if (fwd_e < eps1 || bwd_e < eps1)
    {
        const int both = fwd_e < eps1 && bwd_e < eps1;
        const int similar = fabsf(depth_to_z(fi.depth) - depth_to_z(bi.depth)) < eps2;
        const int choose_fwd = (both && !similar && fi.depth < bi.depth) || ((!both || similar) && fwd_e < bwd_e);
        if (choose_fwd)
        {
            r.valid = 1;
            r.visible_in_main = fwd_vis || (both && similar && bwd_vis);
            r.priority = fwd->priority;
            r.error = fwd_e;
            r.depth = fi.depth;
            r.color = second_chance(1.0f - alpha, frame_idx, sf, sf_t, fi, s, fwd, bwd, eps2);
        }
        else
        {
            r.valid = 1;
            r.visible_in_main = bwd_vis || (both && similar && fwd_vis);
            r.priority = bwd->priority;
            r.error = bwd_e;
            r.depth = bi.depth;
            r.color = second_chance(alpha, frame_idx, sf, sf_t, bi, s, bwd, fwd, eps2);
        }
    }
    else if (always_valid)
    {
        r.valid = 1;
        const c4 cf = second_chance(1.0f - alpha, frame_idx, sf, sf_t, fi, s, fwd, bwd, eps2);
        const c4 cb = second_chance(alpha, frame_idx, sf, sf_t, bi, s, bwd, fwd, eps2);
        r.color = color_to_uchar4(lerp_color(cf, cb, 0.5f));
    }
    return r;
}

/* bidirectionalReprojection_kernel<SW, SI, MAIN_ALWAYS_VALID>, src/renderer.cu:400-465 */
static void reproj_pixel(const oracle_render_info *s, const view_ctx *views, int n_aux, int SW, int SI, int main_always_valid,
                         uint32_t x, uint32_t y, uint8_t *out)
{
    const u2 res = {s->width, s->height};
    const u2 idx = {x, y};
    const f2 pcs = pixel2CS(idx, res);
    uint8_t *o = out + 4 * ((size_t)y * res.x + x);

    const reproj_result m = bidir(SW, SI, main_always_valid, EPS_1_FULL_RES, EPS_2_FULL_RES, idx, idx, res, s->alpha, pcs, s, &views[0], &views[1]);
    if (m.valid)
        memcpy(o, &m.color, 4);
    if (n_aux <= 0)
        return;

    reproj_result best = {0, 0, 0, 0.0f, 0.0f, {0, 0, 0, 0}};
    for (int i = 0; i < n_aux; i++)
    {
        const view_ctx *vf = &views[2 + 2 * i];
        const view_ctx *vb = &views[3 + 2 * i];
        const u2 ar = vf->dims;
        const u2 aidx = {x / (res.x / ar.x), y / (res.y / ar.y)};
        const f2 apcs = pixel2CS(aidx, ar);
        const reproj_result r = bidir(SW, SI, 0, EPS_1_LOW_RES, EPS_2_LOW_RES, aidx, idx, res, s->alpha, apcs, s, vf, vb);
        if (!best.valid)
            best = r;
        else if (r.valid)
        {
            const int similar = fabsf(depth_to_z(best.depth) - depth_to_z(r.depth)) < EPS_2_LOW_RES;
            const int choose_new = (!similar && r.depth < best.depth) || (similar && r.priority >= best.priority && r.error < best.error);
            if (choose_new)
                best = r;
        }
    }
    if (best.valid)
    {
        int choose_aux = !m.valid;
        if (m.valid && !best.visible_in_main)
        {
            const int similar = fabsf(depth_to_z(best.depth) - depth_to_z(m.depth)) < EPS_2_LOW_RES;
            choose_aux = !similar && best.depth < m.depth;
        }
        if (choose_aux)
            memcpy(o, &best.color, 4);
    }
}

/* ---- timewarp (mode 4), src/renderer.cu:467-522,615-629 ---- */

typedef struct { float x, y, z; } v3f;

static float dot3(v3f a, v3f b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }           /* glm-subset order */
static float dot4(f4 a, f4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
static v3f normalize3(v3f v)
{
    const float s = 1.0f / sqrtf(dot3(v, v));
    v3f r = {v.x * s, v.y * s, v.z * s};
    return r;
}
static f4 normalize4(f4 v)
{
    const float s = 1.0f / sqrtf(dot4(v, v));
    f4 r = {v.x * s, v.y * s, v.z * s, v.w * s};
    return r;
}

/* Mean of the forward keyframe's NDC z (ImageBuffer::average, src/util/image_buffer.cu:80-100).
 * The reference adds with a float atomicAdd in an unspecified order; here every row is summed
 * left to right in double, the rows top to bottom in double, and the total is rounded to float
 * and divided by the pixel count in float, as the reference's final division does. */
static float mean_z(const float *z, uint32_t w, uint32_t h)
{
    double total = 0.0;
    for (uint32_t y = 0; y < h; y++)
    {
        double row = 0.0;
        for (uint32_t x = 0; x < w; x++)
            row += (double)z[(size_t)y * w + x];
        total += row;
    }
    return (float)total / (float)(w * h);
}

static void timewarp_pixel(const oracle_render_info *s, const oracle_view *to, const oracle_view *aux, float depth_to, uint32_t x, uint32_t y,
                           uint8_t *out)
{
    const u2 res = {s->width, s->height}, px = {x, y};
    const f2 pcs = pixel2CS(px, res);
    const f4 near_cs = {pcs.x, pcs.y, 0.0f, 1.0f}, far_cs = {pcs.x, pcs.y, 1.0f, 1.0f};
    const f4 near_ws = project(s->inv_viewproj, near_cs), far_ws = project(s->inv_viewproj, far_cs);
    const v3f ro = {near_ws.x, near_ws.y, near_ws.z};
    const v3f rd = normalize3((v3f){far_ws.x - near_ws.x, far_ws.y - near_ws.y, far_ws.z - near_ws.z});
    const f4 center_cs = {0.0f, 0.0f, depth_to, 1.0f};
    const f4 center_ws = project(to->inv_viewproj, center_cs);
    const f4 campos = {to->inv_viewproj[12], to->inv_viewproj[13], to->inv_viewproj[14], to->inv_viewproj[15]}; /* inv_viewproj_mat_to[3] */
    const f4 vd4 = normalize4((f4){center_ws.x - campos.x, center_ws.y - campos.y, center_ws.z - campos.z, center_ws.w - campos.w});
    const v3f n = {vd4.x, vd4.y, vd4.z};
    const v3f pp = {campos.x, campos.y, campos.z};
    const float denom = dot3(rd, n);
    if (fabsf(denom) < 1e-6f) /* the ray is parallel to the plane: no write */
        return;
    const float t = dot3((v3f){pp.x - ro.x, pp.y - ro.y, pp.z - ro.z}, n) / denom;
    const f4 hit = {ro.x + t * rd.x, ro.y + t * rd.y, ro.z + t * rd.z, 1.0f};
    const f4 pc = project(to->viewproj, hit);
    const f2 pcxy = {pc.x, pc.y};
    const u2 tres = {to->width, to->height};
    i2 pix = CS2pixel(pcxy, tres);
    const oracle_view *src = to;
    u2 sres = tres;
    if (!in_range(pix, tres) && aux)
    {
        const f4 pa = project(aux->viewproj, hit);
        const f2 paxy = {pa.x, pa.y};
        sres.x = aux->width;
        sres.y = aux->height;
        pix = CS2pixel(paxy, sres);
        src = aux;
    }
    /* clamp(pixel, 0, res - 1), include/util/helper_math.h clamp(int2, int2, int2) */
    pix.x = pix.x < 0 ? 0 : (pix.x > (int32_t)sres.x - 1 ? (int32_t)sres.x - 1 : pix.x);
    pix.y = pix.y < 0 ? 0 : (pix.y > (int32_t)sres.y - 1 ? (int32_t)sres.y - 1 : pix.y);
    memcpy(out, src->color + 4 * ((size_t)pix.y * sres.x + (uint32_t)pix.x), 4);
}

static int oracle_timewarp(const oracle_frame *frame, const oracle_render_info *s, uint8_t *out_rgba, int nt)
{
    const float depth_to = mean_z(frame->fwd.z, frame->fwd.width, frame->fwd.height);
    const oracle_view *aux = frame->num_aux > 0 ? &frame->aux_curr[0] : NULL;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int32_t y = 0; y < (int32_t)s->height; y++)
        for (uint32_t x = 0; x < s->width; x++)
            timewarp_pixel(s, &frame->fwd, aux, depth_to, x, (uint32_t)y, out_rgba + 4 * ((size_t)y * s->width + x));
    return 0;
}

static int view_ok(const oracle_view *v)
{
    if (!v || !v->color || !v->z || v->width == 0 || v->height == 0 || v->width > 65535u || v->height > 65535u)
        return 0;
    if (v->shadow_color_a && !v->shadow_info)
        return 0;
    return 1;
}

int oracle_render(const oracle_frame *frame, const oracle_render_info *s, uint8_t *out_rgba, oracle_view_out *outs, int nthreads)
{
    if (!frame || !s || !out_rgba || s->mode < 0 || s->mode > 4)
        return -1;
    /* shadow levels sit at bits 2i of a 32-bit field: more than 16 sub-frames
     * would shift past its width (undefined in the reference) */
    if (s->shadow_frames_per_anchor < 0 || s->shadow_frames_per_anchor > 16)
        return -1;
    if (!view_ok(&frame->fwd) || !view_ok(&frame->bwd) || frame->num_aux < 0)
        return -1;
    const u2 res = {s->width, s->height};
    if (frame->fwd.width != res.x || frame->fwd.height != res.y || frame->bwd.width != res.x || frame->bwd.height != res.y)
        return -1;
    const int n_aux = frame->num_aux;
    for (int i = 0; i < n_aux; i++)
    {
        const oracle_view *a = &frame->aux_curr[i], *b = &frame->aux_next[i];
        if (!view_ok(a) || !view_ok(b) || a->width != b->width || a->height != b->height)
            return -1;
        if (a->width > res.x || a->height > res.y)
            return -1;
        if ((res.x - 1) / (res.x / a->width) >= a->width || (res.y - 1) / (res.y / a->height) >= a->height)
            return -1;
    }
#ifdef _OPENMP
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    const int nt = 1;
    (void)nthreads;
#endif
    if (s->mode == 4) /* TIMEWARP returns before any splatting, src/renderer.cu:615-629 */
        return oracle_timewarp(frame, s, out_rgba, nt);
    const int n_views = 2 + 2 * n_aux;
    view_ctx *views = (view_ctx *)calloc((size_t)n_views, sizeof(view_ctx));
    void **scratch = (void **)calloc((size_t)n_views * 3, sizeof(void *));
    if (!views || !scratch)
    {
        free(views);
        free(scratch);
        return -1;
    }
    int rc = 0;
    const float alpha = s->alpha;
    for (int k = 0; k < n_views; k++)
    {
        view_ctx *c = &views[k];
        if (k < 2)
        {
            c->v = k == 0 ? &frame->fwd : &frame->bwd;
            c->forward = k == 0;
            c->priority = 0;
            c->vp_to = (k == 0 ? frame->bwd.viewproj : frame->fwd.viewproj);
        }
        else
        {
            const int i = (k - 2) / 2;
            const int fw = ((k - 2) % 2) == 0;
            c->v = fw ? &frame->aux_curr[i] : &frame->aux_next[i];
            c->forward = fw;
            c->priority = frame->aux_priority ? frame->aux_priority[i] : 0;
            c->vp_to = fw ? frame->aux_next[i].viewproj : frame->aux_curr[i].viewproj;
        }
        c->weight = c->forward ? alpha : 1.0f - alpha;
        c->vp_from_main = c->forward ? frame->fwd.viewproj : frame->bwd.viewproj;
        c->dims.x = c->v->width;
        c->dims.y = c->v->height;
        const size_t n = (size_t)c->dims.x * c->dims.y;
        c->splat = outs && outs[k].splat ? outs[k].splat : (uint64_t *)(scratch[3 * k] = malloc(n * 8));
        c->cam_ff = outs && outs[k].cam_ff ? outs[k].cam_ff : (float *)(scratch[3 * k + 1] = malloc(n * 16));
        c->full_ff = outs && outs[k].full_ff ? outs[k].full_ff : (float *)(scratch[3 * k + 2] = malloc(n * 16));
        if (!c->splat || !c->cam_ff || !c->full_ff)
            rc = -1;
    }
    if (rc == 0)
    {
        const int linear = s->mode == 1;
        for (int k = 0; k < n_views; k++)
        {
            const view_ctx *c = &views[k];
            memset(c->splat, SPLAT_INIT_BYTE, (size_t)c->dims.x * c->dims.y * 8);
#pragma omp parallel for schedule(static) num_threads(nt)
            for (int32_t y = 0; y < (int32_t)c->dims.y; y++)
                for (uint32_t x = 0; x < c->dims.x; x++)
                    splat_pixel(c, s->viewproj, linear, x, (uint32_t)y);
        }
        int SW = 1, SI = 3, mav = 0; /* modes 0 and 2, src/renderer.cu:678-681 */
        if (s->mode == 3)
            SI = 0; /* :682-685 */
        else if (s->mode == 1)
        {
            SW = 3; /* :686-689 */
            SI = 5;
            mav = 1;
        }
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int32_t y = 0; y < (int32_t)res.y; y++)
            for (uint32_t x = 0; x < res.x; x++)
                reproj_pixel(s, views, n_aux, SW, SI, mav, x, (uint32_t)y, out_rgba);
    }
    for (int k = 0; k < n_views * 3; k++)
        free(scratch[k]);
    free(scratch);
    free(views);
    return rc;
}
