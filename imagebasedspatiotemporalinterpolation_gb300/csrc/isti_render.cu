// Per-frame interpolation path on GB300: init, splat and bidirectional
// reprojection kernels, and the C ABI of include/isti.h.
//
// Reference: src/renderer.cu (DerThomy/ImageBasedSpatioTemporalInterpolation).
//
// A launch sequence renders a batch of 1..ISTI_MAX_BATCH_FRAMES client frames
// of one keyframe pair (isti_render is a batch of one).
//
// Layout in HBM (renderer-owned arena, one allocation):
//   [splat keys, u64/px: frame-major, every view][cam flow f32x4/px: frame-major, every view]
//   [full flow f32x4/px, every view][pixel->clip tables, (w + h) f32 per view]
// Pixel inputs are caller-owned device images (include/isti.h).
//
// Launches per batch (nothing blocks the host):
//  1. init:  every key <- 0xfefe...fe (the reference's cudaMemset(0xfe),
//            src/renderer.cu:632-638) and the pixel->clip tables;
//  2. splat: blockIdx.z = source view; per source pixel the keyframe part
//            (world positions, flow to the other keyframe, visibility in the
//            main view) once, then per frame the client-camera projection,
//            flow store and 64-bit atomicMin;
//  3. reprojection: a block covers 2 rows x 32 output pixels with one warp
//            per source view (view = threadIdx.y).  Phase 1: each thread runs
//            window initialisation + iterative search + reprojection error
//            for its view and both rows, interleaved, for every frame.
//            Phase 2: the (frame, row) tasks are spread over the warps; each
//            chooses the direction per camera and the winning camera and
//            computes the colour (second chance, soft shadows) only for the
//            result that is written.  The reference colours every camera's
//            result (src/renderer.cu:378-396,436); only the written one is
//            observable and colour never feeds a choice, so the output is
//            identical.  Phase 3 writes chained outputs.
#include "isti.h"
#include "isti_device.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace isti
{
constexpr int MAX_VIEWS = 2 + 2 * ISTI_MAX_AUX_CAMS;
constexpr int MAX_FRAMES = ISTI_MAX_BATCH_FRAMES;
constexpr int ROWS = 2; // output rows per reprojection block
constexpr float FLT_MAX_F = 3.402823466e+38f;

struct DevView
{
    const uint32_t *color; // RGBA8 packed, R in bits 0-7
    const float *z;
    const void *motion;
    const uint32_t *sha, *shb, *shi;
    unsigned long long *splat; // frame 0; frame k at + k * FrameParams::key_stride
    float4 *cam_ff;            // frame 0; frame k at + k * FrameParams::cam_stride
    float4 *full_ff;
    float *lut;                // pixel2CS tables: x at [0, w), y at [w, w + h)
    uint32_t w, h;
    uint32_t sx, sy;           // output pixels per view pixel (aux_idx = idx / s, src/renderer.cu:433)
    int32_t motion_fmt;
    int32_t forward;
    int32_t priority;
    float err_sx, err_sy;      // res / min(res.x, res.y), computeReprojError scale (src/renderer.cu:213)
    float inv_vp[16];          // this view's inverse viewproj
    float vp_to[16];           // the other keyframe's viewproj (same camera)
    float vp_main[16];         // main camera viewproj at this keyframe (visible_in_main test)
};

// Per-frame settings (RenderInfo / AdditionalRenderInfo, include/renderer.h:18-35)
struct FrameCfg
{
    float alpha;
    int32_t fpa, sfpa, no_shadows;
};

struct FrameParams
{
    DevView v[MAX_VIEWS];
    float cam_vp[MAX_FRAMES][16];
    uint32_t *out[MAX_FRAMES];
    FrameCfg f[MAX_FRAMES];
    size_t key_stride; // elements between frames in the key block
    size_t cam_stride; // elements between frames in the cam-flow block
    ulonglong2 *keys;  // the whole key block (16-byte units) for the init kernel
    size_t key_units;
    uint32_t out_w, out_h;
    int32_t n_views, n_aux, n_frames, linear, chain;
};

// ---- border-addressed loads: zero outside the image (cudaAddressModeBorder) ----

__device__ __forceinline__ float ld_f(const float *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (y * w + x)) : 0.0f;
}
__device__ __forceinline__ float4 ld_f4(const float4 *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (y * w + x)) : make_float4(0.f, 0.f, 0.f, 0.f);
}
__device__ __forceinline__ uint32_t ld_c(const uint32_t *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (y * w + x)) : 0u;
}

__device__ __forceinline__ float4 load_motion(const DevView &v, uint32_t idx)
{
    if (v.motion_fmt == ISTI_MOTION_F32X4)
        return __ldg(static_cast<const float4 *>(v.motion) + idx);
    if (v.motion_fmt == ISTI_MOTION_F16X3)
    {
        const __half *m = static_cast<const __half *>(v.motion) + 3 * (size_t)idx;
        return make_float4(__half2float(m[0]), __half2float(m[1]), __half2float(m[2]), 0.0f);
    }
    return make_float4(0.f, 0.f, 0.f, 0.f);
}

// pixel2CS of pixel (x, y) of view v from its tables; direct formula outside the image
__device__ __forceinline__ float2 view_pixel2cs(const DevView &v, uint32_t x, uint32_t y)
{
    if (x < v.w && y < v.h)
        return make_float2(__ldg(v.lut + x), __ldg(v.lut + v.w + y));
    return pixel2cs(x, y, v.w, v.h);
}

// ---- key initialisation (cudaMemset 0xfe, src/renderer.cu:632-638) + pixel->clip tables ----

__global__ void __launch_bounds__(256) init_kernel(const __grid_constant__ FrameParams p)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const ulonglong2 empty = make_ulonglong2(SPLAT_EMPTY, SPLAT_EMPTY);
    for (size_t i = t; i < p.key_units; i += stride)
        p.keys[i] = empty;
    if (t < 65536)
        for (int k = 0; k < p.n_views; k++)
        {
            const DevView &v = p.v[k];
            if (t < v.w)
                v.lut[t] = pixel2cs((uint32_t)t, 0, v.w, 1).x;
            if (t < v.h)
                v.lut[v.w + t] = pixel2cs(0, (uint32_t)t, 1, v.h).y;
        }
}

// ---- computeFlowFields_sortedSplatting_kernel, src/renderer.cu:76-146 ----

__global__ void __launch_bounds__(256) splat_kernel(const __grid_constant__ FrameParams p)
{
    const DevView &v = p.v[blockIdx.z];
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= v.w || y >= v.h)
        return;
    const uint32_t idx = y * v.w + x;

    // keyframe part, independent of the client camera
    const float z_from = __ldg(v.z + idx);
    const float4 om = load_motion(v, idx);
    const float pcx = __ldg(v.lut + x), pcy = __ldg(v.lut + v.w + y); // pixel2CS(idx2D, resolution)
    const float4 cs_from = make_float4(pcx, pcy, z_from, 1.0f);
    const float4 ws_from = project(v.inv_vp, cs_from);
    const float4 moved = make_float4(__fadd_rn(pcx, om.x), __fadd_rn(pcy, om.y), __fadd_rn(z_from, om.z), 1.0f);
    const float4 ws_to = project(v.inv_vp, moved);

    // visible_in_main: WS2CS(posWS_from, viewproj_mat_from_main) inside +-(1 - 1e-3), src/renderer.cu:104-107
    const float4 cm = matvec(v.vp_main, ws_from);
    const float lim = 1.0f - 1e-3f;
    const bool visible = quotient_inside(cm.x, cm.w, lim) && quotient_inside(cm.y, cm.w, lim) && quotient_inside(cm.z, cm.w, lim);
    const float vis = visible ? 1.0f : 0.0f;

    const float4 cs_to = project(v.vp_to, ws_to);
    const float fmx = __fsub_rn(cs_to.x, cs_from.x), fmy = __fsub_rn(cs_to.y, cs_from.y), fmz = __fsub_rn(cs_to.z, cs_from.z);
    v.full_ff[idx] = make_float4(fmx, fmy, fmz, vis);
    const float4 d_ws = make_float4(__fsub_rn(ws_to.x, ws_from.x), __fsub_rn(ws_to.y, ws_from.y), __fsub_rn(ws_to.z, ws_from.z),
                                    __fsub_rn(ws_to.w, ws_from.w));

    // client-camera part, per frame
    for (int k = 0; k < p.n_frames; k++)
    {
        const float wg = v.forward ? p.f[k].alpha : __fsub_rn(1.0f, p.f[k].alpha);
        unsigned long long *keys = v.splat + k * p.key_stride;
        float4 *cam = v.cam_ff + k * p.cam_stride;
        if (!p.linear)
        {
            const float4 scaled = make_float4(__fadd_rn(ws_from.x, __fmul_rn(wg, d_ws.x)), __fadd_rn(ws_from.y, __fmul_rn(wg, d_ws.y)),
                                              __fadd_rn(ws_from.z, __fmul_rn(wg, d_ws.z)), __fadd_rn(ws_from.w, __fmul_rn(wg, d_ws.w)));
            const float4 pc = project(p.cam_vp[k], scaled);
            cam[idx] = make_float4(__fsub_rn(pc.x, cs_from.x), __fsub_rn(pc.y, cs_from.y), __fsub_rn(pc.z, cs_from.z), vis);
            const float depth_cam = z_to_depth(pc.z);
            const int2 pix = cs2pixel(pc.x, pc.y, v.w, v.h);
            if (in_range(pix, v.w, v.h) && !(depth_cam < 0.0f))
                atomicMin(keys + ((uint32_t)pix.y * v.w + (uint32_t)pix.x), encode_key(depth_cam, x, y));
        }
        else
        {
            cam[idx] = make_float4(__fmul_rn(fmx, wg), __fmul_rn(fmy, wg), __fmul_rn(fmz, wg), vis);
            atomicMin(keys + idx, encode_key(z_to_depth(z_from), x, y));
        }
    }
}

// ---- colour: colorFromShadow / secondChanceAndBlend_kernel, src/renderer.cu:217-327 ----

// colorFromShadow (level-index form), src/renderer.cu:217-268
__device__ uint32_t color_from_shadow_idx(uint32_t sidx, int32_t sfpa, const DevView &v, uint32_t px, uint32_t py)
{
    const uint32_t main_color = ld_c(v.color, px, py, v.w, v.h);
    if (sidx < (uint32_t)sfpa && sidx > 0)
    {
        const uint32_t si = ld_c(v.shi, px, py, v.w, v.h);
        const uint32_t bf = ((si & 255u) << 16) | (((si >> 8) & 255u) << 8) | ((si >> 16) & 255u);
        if (v.shb != nullptr && bf != 0)
        {
            const int32_t init_val = (int32_t)(bf & SOFTSHADOW_VAL_MASK);
            const int32_t my_val = (int32_t)((bf >> (SOFTSHADOW_BITS * sidx)) & SOFTSHADOW_VAL_MASK);
            int32_t mn = (int32_t)SOFTSHADOW_VAL_MASK, mx = 0;
            for (int32_t i = 0; i < sfpa; i++)
            {
                const int32_t lv = (int32_t)((bf >> (SOFTSHADOW_BITS * (uint32_t)i)) & SOFTSHADOW_VAL_MASK);
                mn = min(mn, lv);
                mx = max(mx, lv);
            }
            const float t = __fdiv_rn((float)(my_val - mn), (float)(mx - mn));
            const uint32_t cmin = mn == init_val ? main_color : ld_c(v.sha, px, py, v.w, v.h);
            const uint32_t cmax = mx == init_val ? main_color : ld_c(v.shb, px, py, v.w, v.h);
            // (float)(1.0 - (double)t): t is k / d with d in {1, 2, 3} (or NaN), for which the
            // double difference is exact, so one float subtraction rounds identically.
            const float omt = __fsub_rn(1.0f, t);
            uint32_t r = 255u << 24;
#pragma unroll
            for (int c = 0; c < 3; c++)
            {
                const float a = (float)((cmin >> (8 * c)) & 255u), b = (float)((cmax >> (8 * c)) & 255u);
                r |= cvt_u8(__fadd_rn(__fmul_rn(a, omt), __fmul_rn(b, t))) << (8 * c);
            }
            return r;
        }
    }
    return main_color;
}

struct ShadowFrames
{
    uint32_t frame_idx, sfx, sfy;
    float sft;
};

// frame_idx / shadow sub-frames, src/renderer.cu:359-364
__device__ __forceinline__ ShadowFrames shadow_frames(const FrameCfg &c)
{
    ShadowFrames sf;
    const float fa = __fmul_rn((float)c.fpa, c.alpha);
    const float sa = __fmul_rn((float)c.sfpa, c.alpha);
    sf.frame_idx = __float2uint_rn(fa);
    sf.sfx = __float2uint_rd(__fadd_rn(sa, 1e-9f));
    sf.sfy = __float2uint_ru(__fsub_rn(sa, 1e-9f));
    sf.sft = __fsub_rn(sa, (float)sf.sfx);
    return sf;
}

// colorFromShadow (two sub-frame form), src/renderer.cu:270-295
__device__ uint32_t color_from_shadow(const ShadowFrames &sf, const FrameCfg &c, const DevView &v, uint32_t px, uint32_t py)
{
    if (c.no_shadows || sf.sfx >= (uint32_t)c.sfpa || sf.sfy == 0 || v.sha == nullptr)
        return ld_c(v.color, px, py, v.w, v.h);
    const int32_t sfpa = c.sfpa;
    const uint32_t vx = (uint32_t)(v.forward ? (int32_t)sf.sfx : sfpa - (int32_t)sf.sfx);
    const uint32_t vy = (uint32_t)(v.forward ? (int32_t)sf.sfy : sfpa - (int32_t)sf.sfy);
    if (vx == vy || vy >= (uint32_t)sfpa)
        return color_from_shadow_idx(vx, sfpa, v, px, py);
    if (vx >= (uint32_t)sfpa)
        return color_from_shadow_idx(vy, sfpa, v, px, py);
    const uint32_t a = color_from_shadow_idx(vx, sfpa, v, px, py);
    const uint32_t b = color_from_shadow_idx(vy, sfpa, v, px, py);
    return lerp_color_u8(a, b, sf.sft);
}

// secondChanceAndBlend_kernel<EPS_2>, src/renderer.cu:297-327
__device__ uint32_t second_chance(float weight, const ShadowFrames &sf, const FrameCfg &c, uint32_t sx, uint32_t sy, const DevView &from,
                                  const DevView &to, float eps2)
{
    const float4 m_ft = ld_f4(from.full_ff, sx, sy, from.w, from.h);
    const float2 spcs = view_pixel2cs(from, sx, sy);
    const float sz = ld_f(from.z, sx, sy, from.w, from.h);
    const float pcx = __fadd_rn(spcs.x, m_ft.x), pcy = __fadd_rn(spcs.y, m_ft.y), pcz = __fadd_rn(sz, m_ft.z);
    const int2 pp = cs2pixel(pcx, pcy, to.w, to.h);

    uint32_t out = color_from_shadow(sf, c, from, sx, sy);
    if (sf.frame_idx >= (uint32_t)c.fpa)
        return out;
    if (in_range(pp, to.w, to.h))
    {
        const uint32_t pi = (uint32_t)pp.y * to.w + (uint32_t)pp.x;
        const float az = __ldg(to.z + pi);
        const float4 m_tf = __ldg(to.full_ff + pi);
        const float dx = __fsub_rn(m_ft.x, -m_tf.x), dy = __fsub_rn(m_ft.y, -m_tf.y), dz = __fsub_rn(m_ft.z, -m_tf.z);
        if (sqrt_less(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)), EPS_3) &&
            fabsf(__fsub_rn(az, pcz)) < eps2)
            out = lerp_color_u8(color_from_shadow(sf, c, to, pp.x, pp.y), out, weight);
    }
    return out;
}

// ---- bidirectional reprojection, src/renderer.cu:148-465 ----

// One direction of one camera for one output pixel: window init + search + error.
struct DirRes
{
    float error;  // FLT_MAX when not searched
    float depth;  // searched depth, else the window-initialisation depth
    uint32_t src; // source pixel, x << 16 | y
    uint32_t vis; // visible_in_main
};

// Result of bidirectionalReprojection for one camera (src/renderer.cu:366-397), without its colour.
struct CamRes
{
    bool valid;
    bool vis;
    bool blend;      // always-valid 50/50 blend of both directions
    int32_t priority;
    float error;     // indeterminate in the reference for the blend; 0 here
    float depth;
    int32_t dir;     // 0 forward keyframe, 1 backward keyframe
    uint32_t src;
};

template <int SW>
struct Tile
{
    static constexpr int W = 32 + 2 * SW;
    static constexpr int H = ROWS + 2 * SW;
};

__device__ __forceinline__ CamRes cam_result(const DirRes &f, const DirRes &b, const DevView &vf, const DevView &vb, float eps1, float eps2,
                                             bool always_valid)
{
    CamRes r;
    r.valid = false;
    r.vis = false;
    r.blend = false;
    r.priority = 0;
    r.error = 0.0f;
    r.depth = 0.0f;
    r.dir = 0;
    r.src = 0;
    if (f.error < eps1 || b.error < eps1)
    {
        const bool both = f.error < eps1 && b.error < eps1;
        const bool similar = fabsf(__fsub_rn(depth_to_z(f.depth), depth_to_z(b.depth))) < eps2;
        const bool choose_fwd = (both && !similar && f.depth < b.depth) || ((!both || similar) && f.error < b.error);
        r.valid = true;
        if (choose_fwd)
        {
            r.vis = f.vis || (both && similar && b.vis);
            r.priority = vf.priority;
            r.error = f.error;
            r.depth = f.depth;
            r.dir = 0;
            r.src = f.src;
        }
        else
        {
            r.vis = b.vis || (both && similar && f.vis);
            r.priority = vb.priority;
            r.error = b.error;
            r.depth = b.depth;
            r.dir = 1;
            r.src = b.src;
        }
    }
    else if (always_valid)
    {
        r.valid = true;
        r.blend = true;
    }
    return r;
}

// Chooses among the cameras of one output pixel and returns the colour to
// write (false: keep the previous output), src/renderer.cu:400-465.
// res points at the [n_views][32] results of this pixel's row and frame.
template <bool MAV>
__device__ __forceinline__ bool resolve_pixel(const DirRes *res, int lane, const FrameParams &p, const FrameCfg &c, uint32_t &color)
{
    const CamRes m = cam_result(res[lane], res[32 + lane], p.v[0], p.v[1], EPS_1_FULL_RES, EPS_2_FULL_RES, MAV);
    CamRes best;
    best.valid = false;
    best.vis = false;
    best.priority = 0;
    best.error = 0.0f;
    best.depth = 0.0f;
    int best_cam = 0;
    const int n_cams = p.n_views / 2;
    for (int cam = 1; cam < n_cams; cam++)
    {
        const CamRes r = cam_result(res[(2 * cam) * 32 + lane], res[(2 * cam + 1) * 32 + lane], p.v[2 * cam], p.v[2 * cam + 1], EPS_1_LOW_RES,
                                    EPS_2_LOW_RES, false);
        bool take = !best.valid;
        if (best.valid && r.valid)
        {
            const bool similar = fabsf(__fsub_rn(depth_to_z(best.depth), depth_to_z(r.depth))) < EPS_2_LOW_RES;
            take = (!similar && r.depth < best.depth) || (similar && r.priority >= best.priority && r.error < best.error);
        }
        if (take)
        {
            best = r;
            best_cam = cam;
        }
    }
    int cam = -1;
    CamRes fin = m;
    if (m.valid)
        cam = 0;
    if (best.valid)
    {
        bool choose_aux = !m.valid;
        if (m.valid && !best.vis)
        {
            const bool similar = fabsf(__fsub_rn(depth_to_z(best.depth), depth_to_z(m.depth))) < EPS_2_LOW_RES;
            choose_aux = !similar && best.depth < m.depth;
        }
        if (choose_aux)
        {
            cam = best_cam;
            fin = best;
        }
    }
    if (cam < 0)
        return false; // temporal hole filling: keep the previous output (src/renderer.cu:416-419,462-463)

    const ShadowFrames sf = shadow_frames(c);
    const DevView &vf = p.v[2 * cam], &vb = p.v[2 * cam + 1];
    const float eps2 = cam == 0 ? EPS_2_FULL_RES : EPS_2_LOW_RES;
    const float oma = __fsub_rn(1.0f, c.alpha);
    if (fin.blend)
    {
        const DirRes &f = res[lane], &b = res[32 + lane];
        const uint32_t cf = second_chance(oma, sf, c, f.src >> 16, f.src & 0xFFFFu, vf, vb, eps2);
        const uint32_t cb = second_chance(c.alpha, sf, c, b.src >> 16, b.src & 0xFFFFu, vb, vf, eps2);
        color = lerp_color_u8(cf, cb, 0.5f);
    }
    else if (fin.dir == 0)
        color = second_chance(oma, sf, c, fin.src >> 16, fin.src & 0xFFFFu, vf, vb, eps2);
    else
        color = second_chance(c.alpha, sf, c, fin.src >> 16, fin.src & 0xFFFFu, vb, vf, eps2);
    return true;
}

// Upper bound for the window comparison, from the depth bits l of the current lowest key.
// The reference replaces the lowest entry by a candidate c with c > 0 when
//   !isfinite(l) || l < 0 || c < l            (src/renderer.cu:167)
// For c > 0 (bits in [1, 0x7f800000], +inf included) this is c_bits < bound(l_bits):
//   l = +-inf, NaN, or negative non-zero  -> always true  -> bound 0xffffffff;
//   l = -0.0                              -> always false -> bound 0;
//   l in [+0, +max finite]                -> c < l, monotonic in the bits -> bound l_bits.
__device__ __forceinline__ uint32_t key_bound(uint32_t l)
{
    return l == 0x80000000u ? 0u : (l >= 0x7f800000u ? 0xffffffffu : l);
}

// initializeSearchFromSplatting<SW> on a shared-memory tile, src/renderer.cu:148-175, same
// scan order.  Tile row `row` holds the view row of this pixel; keys outside the view read
// as 0 (depth +0.0), which the window never selects, exactly like the reference's skipped
// out-of-range neighbours.  Returns the selected raw key.
template <int SW>
__device__ __forceinline__ unsigned long long window_key(const unsigned long long *tile, int row, int col)
{
    using T = Tile<SW>;
    unsigned long long best = tile[row * T::W + col];
    uint32_t bound = key_bound((uint32_t)(best >> 32));
#pragma unroll
    for (int yo = -SW; yo <= SW; yo++)
#pragma unroll
        for (int xo = -SW; xo <= SW; xo++)
        {
            const unsigned long long c = tile[(row + yo) * T::W + col + xo];
            const uint32_t cb = (uint32_t)(c >> 32);
            if (cb - 1u < 0x7f800000u && cb < bound) // c > 0 && (the reference's replacement test)
            {
                best = c;
                bound = key_bound(cb);
            }
        }
    return best;
}

// bidirectionalReprojection_kernel<SW, SI, MAIN_ALWAYS_VALID>, src/renderer.cu:400-465
// block = (32, n_views): output rows ROWS * blockIdx.y + {0, 1}, 32 pixels each, one warp per source view.
// Phase 1 takes G frames at a time, so each thread has ROWS x G independent search chains in flight.
template <int SW, int SI, bool MAV, int G>
__global__ void __launch_bounds__(32 * MAX_VIEWS) reproj_kernel(const __grid_constant__ FrameParams p)
{
    using T = Tile<SW>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int nv = p.n_views, nf = p.n_frames;
    DirRes *res = reinterpret_cast<DirRes *>(smem);                        // [nf][ROWS][nv][32]
    uint32_t *cols = reinterpret_cast<uint32_t *>(res + nf * ROWS * nv * 32); // [nf][ROWS][32]
    uint32_t *valid = cols + nf * ROWS * 32;                               // [nf][ROWS][32]
    unsigned long long *tiles = reinterpret_cast<unsigned long long *>(valid + nf * ROWS * 32); // [nv][G][H][W]

    const int lane = threadIdx.x, vw = threadIdx.y;
    const uint32_t x0 = blockIdx.x * 32, x = x0 + lane, y0 = blockIdx.y * ROWS;
    const bool xok = x < p.out_w;
    {
        const DevView &v = p.v[vw];
        const uint32_t ix = v.sx == 1 ? x : x / v.sx, tx0 = v.sx == 1 ? x0 : x0 / v.sx;
        const uint32_t iy0 = v.sy == 1 ? y0 : y0 / v.sy, iy1 = v.sy == 1 ? y0 + 1 : (y0 + 1) / v.sy;
        const bool ok0 = xok, ok1 = xok && y0 + 1 < p.out_h;
        const bool fwd = (vw & 1) == 0;
        unsigned long long *tile = tiles + vw * (G * T::H * T::W);
        const int col = (int)(ix - tx0) + SW;
        const int wrow[ROWS] = {SW, (int)(iy1 - iy0) + SW}; // tile row of each output row's window centre
        const bool rok[ROWS] = {ok0, ok1};
        // pixel2CS of the output pixels in the main view (the search target) and in this view (the error)
        const DevView &v0 = p.v[0];
        const uint32_t xc = min(x, p.out_w - 1), y1c = min(y0 + 1, p.out_h - 1);
        const float qx = __ldg(v0.lut + xc);
        const float qy[ROWS] = {__ldg(v0.lut + v0.w + y0), __ldg(v0.lut + v0.w + y1c)};
        const float pcx = __ldg(v.lut + min(ix, v.w - 1));
        const float pcy[ROWS] = {__ldg(v.lut + v.w + iy0), __ldg(v.lut + v.w + min(iy1, v.h - 1))};
        const uint32_t vwid = v.w, vhei = v.h;
#pragma unroll 1
        for (int k0 = 0; k0 < nf; k0 += G)
        {
            __syncwarp();
#pragma unroll
            for (int g = 0; g < G; g++)
            {
                if (k0 + g < nf)
                {
                    const unsigned long long *keys = v.splat + (k0 + g) * p.key_stride;
                    unsigned long long *tg = tile + g * (T::H * T::W);
#pragma unroll
                    for (int r = 0; r < T::H; r++)
                    {
                        const uint32_t gy = iy0 - SW + r;
                        const bool row_ok = gy < vhei;
                        for (int c = lane; c < T::W; c += 32)
                        {
                            const uint32_t gx = tx0 - SW + c;
                            tg[r * T::W + c] = (row_ok && gx < vwid) ? __ldg(keys + (gy * vwid + gx)) : 0ull;
                        }
                    }
                }
            }
            __syncwarp();

            bool s[G][ROWS];
            uint32_t ax[G][ROWS], ay[G][ROWS];
            float d_init[G][ROWS];
            const float4 *cam[G];
#pragma unroll
            for (int g = 0; g < G; g++)
            {
                const int k = min(k0 + g, nf - 1);
                const bool search_ok = (k0 + g < nf) && (!fwd || p.f[k].alpha < 1.0f);
                cam[g] = v.cam_ff + k * p.cam_stride;
#pragma unroll
                for (int r = 0; r < ROWS; r++)
                {
                    const unsigned long long lo = window_key<SW>(tile + g * (T::H * T::W), wrow[r], col);
                    d_init[g][r] = __uint_as_float((uint32_t)(lo >> 32));
                    ax[g][r] = ((uint32_t)lo) >> 16;
                    ay[g][r] = (uint32_t)lo & 0xFFFFu;
                    s[g][r] = rok[r] && search_ok && d_init[g][r] > 0.0f;
                }
            }
            // iterativeSearch<SI>, src/renderer.cu:177-202, all chains interleaved.  The start is a
            // splatted source pixel and every accepted step is in range: no border handling needed.
#pragma unroll
            for (int i = 0; i < SI; i++)
            {
                float4 m[G][ROWS];
#pragma unroll
                for (int g = 0; g < G; g++)
#pragma unroll
                    for (int r = 0; r < ROWS; r++)
                        m[g][r] = s[g][r] ? __ldg(cam[g] + (ay[g][r] * vwid + ax[g][r])) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int g = 0; g < G; g++)
#pragma unroll
                    for (int r = 0; r < ROWS; r++)
                    {
                        const int2 t = cs2pixel(__fsub_rn(qx, m[g][r].x), __fsub_rn(qy[r], m[g][r].y), vwid, vhei);
                        if (s[g][r] && in_range(t, vwid, vhei))
                        {
                            ax[g][r] = (uint32_t)t.x;
                            ay[g][r] = (uint32_t)t.y;
                        }
                    }
            }
            // final flow, depth and computeReprojError, src/renderer.cu:338-341, 204-215
            float4 m[G][ROWS];
            float zz[G][ROWS], fx[G][ROWS], fy[G][ROWS];
#pragma unroll
            for (int g = 0; g < G; g++)
#pragma unroll
                for (int r = 0; r < ROWS; r++)
                {
                    m[g][r] = make_float4(0.f, 0.f, 0.f, 0.f);
                    zz[g][r] = fx[g][r] = fy[g][r] = 0.f;
                    if (s[g][r])
                    {
                        const uint32_t si = ay[g][r] * vwid + ax[g][r];
                        m[g][r] = __ldg(cam[g] + si);
                        zz[g][r] = __ldg(v.z + si);
                        fx[g][r] = __ldg(v.lut + ax[g][r]);
                        fy[g][r] = __ldg(v.lut + vwid + ay[g][r]);
                    }
                }
#pragma unroll
            for (int g = 0; g < G; g++)
            {
                if (k0 + g >= nf)
                    break;
#pragma unroll
                for (int r = 0; r < ROWS; r++)
                {
                    DirRes d;
                    d.error = FLT_MAX_F;
                    d.depth = d_init[g][r];
                    d.vis = 0;
                    if (s[g][r])
                    {
                        d.depth = z_to_depth(__fadd_rn(zz[g][r], m[g][r].z));
                        const float ex = __fmul_rn(__fsub_rn(__fadd_rn(fx[g][r], m[g][r].x), pcx), v.err_sx);
                        const float ey = __fmul_rn(__fsub_rn(__fadd_rn(fy[g][r], m[g][r].y), pcy[r]), v.err_sy);
                        d.error = __fsqrt_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)));
                        d.vis = m[g][r].w > 0.0f;
                    }
                    d.src = (ax[g][r] << 16) | ay[g][r];
                    res[(((k0 + g) * ROWS + r) * nv + vw) * 32 + lane] = d;
                }
            }
        }
    }
    __syncthreads();

    // phase 2: (frame, row) tasks over the warps
#pragma unroll 1
    for (int t = vw; t < nf * ROWS; t += nv)
    {
        const int k = t / ROWS, r = t % ROWS;
        const uint32_t y = y0 + r;
        uint32_t color = 0;
        const bool ok = xok && y < p.out_h && resolve_pixel<MAV>(res + t * nv * 32, lane, p, p.f[k], color);
        if (!p.chain)
        {
            if (ok)
                p.out[k][y * p.out_w + x] = color;
        }
        else
        {
            cols[t * 32 + lane] = color;
            valid[t * 32 + lane] = ok ? 1u : 0u;
        }
    }
    if (!p.chain)
        return;
    __syncthreads();
    // phase 3: one persistent buffer per row, starting as out[0], copied to out[k] after frame k
    if (vw >= ROWS)
        return;
    const uint32_t y = y0 + vw;
    if (!xok || y >= p.out_h)
        return;
    uint32_t run = 0;
    for (int k = 0; k < nf; k++)
    {
        uint32_t *o = p.out[k] + (y * p.out_w + x);
        const int t = k * ROWS + vw;
        if (k == 0)
            run = *o;
        if (valid[t * 32 + lane])
        {
            run = cols[t * 32 + lane];
            *o = run;
        }
        else if (k > 0)
            *o = run;
    }
}

template <int SW, int G>
constexpr size_t reproj_smem(int n_views, int n_frames)
{
    return (size_t)n_frames * ROWS * (n_views * 32 * sizeof(DirRes) + 2 * 32 * sizeof(uint32_t)) +
           (size_t)n_views * G * Tile<SW>::H * Tile<SW>::W * sizeof(unsigned long long);
}
} // namespace isti

// ============================ host side ============================

struct isti_renderer
{
    int device = 0;
    void *arena = nullptr;
    size_t arena_bytes = 0;
    isti::FrameParams last{};
    bool has_frame = false;
    // stage timing: 4 events per timed call (before init, after init, after splat, after reproj)
    bool timing = false;
    std::vector<cudaEvent_t> events;
    std::vector<int32_t> event_frames;
    size_t events_used = 0;
    int32_t timed_launches = 0;
};

namespace
{
thread_local std::string g_last_error;

isti_status fail(isti_status s, const std::string &msg)
{
    g_last_error = msg;
    return s;
}

isti_status cuda_fail(cudaError_t e, const char *what)
{
    return fail(ISTI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

bool view_ok(const isti_view &v, std::string &why)
{
    if (v.width == 0 || v.height == 0 || v.width > 65535u || v.height > 65535u)
        return why = "view size must be 1..65535", false;
    if (!v.color || !v.z)
        return why = "view color and z are required", false;
    if (v.motion_format != ISTI_MOTION_NONE && v.motion_format != ISTI_MOTION_F32X4 && v.motion_format != ISTI_MOTION_F16X3)
        return why = "unknown motion_format", false;
    if (v.motion_format != ISTI_MOTION_NONE && !v.motion)
        return why = "motion pointer is NULL", false;
    if (v.motion_format == ISTI_MOTION_F32X4 && (reinterpret_cast<uintptr_t>(v.motion) & 15u))
        return why = "F32X4 motion must be 16-byte aligned", false;
    if (reinterpret_cast<uintptr_t>(v.color) & 3u)
        return why = "color must be 4-byte aligned", false;
    if (v.shadow_color_a && !v.shadow_info)
        return why = "shadow_info is required with shadow_color_a", false;
    return true;
}

// Checks a batch (the reference's implicit contract, made explicit) and
// returns its source views in kernel order.
isti_status validate(int n_frames, void *const *outs, const isti_render_info *infos, const isti_frame_data *frame, const isti_view **views,
                     int &n_views)
{
    if (n_frames < 1 || n_frames > ISTI_MAX_BATCH_FRAMES)
        return fail(ISTI_ERR_INVALID_ARG, "n_frames must be 1..ISTI_MAX_BATCH_FRAMES");
    const isti_render_info *info = &infos[0];
    for (int k = 0; k < n_frames; k++)
    {
        const isti_render_info &f = infos[k];
        if (!outs[k])
            return fail(ISTI_ERR_INVALID_ARG, "NULL output buffer");
        if (reinterpret_cast<uintptr_t>(outs[k]) & 3u)
            return fail(ISTI_ERR_INVALID_ARG, "output buffers must be 4-byte aligned");
        if (f.mode == ISTI_MODE_TIMEWARP)
            return fail(ISTI_ERR_UNSUPPORTED, "timewarp mode is not implemented");
        if (f.mode < 0 || f.mode > ISTI_MODE_TIMEWARP)
            return fail(ISTI_ERR_INVALID_ARG, "unknown render mode");
        if (f.shadow_frames_per_anchor < 0 || f.shadow_frames_per_anchor > 16)
            return fail(ISTI_ERR_INVALID_ARG, "shadow_frames_per_anchor must be 0..16");
        if (f.width != info->width || f.height != info->height || f.mode != info->mode)
            return fail(ISTI_ERR_INVALID_ARG, "all frames of a batch need the same resolution and mode");
    }
    std::string why;
    if (!view_ok(frame->fwd, why) || !view_ok(frame->bwd, why))
        return fail(ISTI_ERR_INVALID_ARG, why);
    if (frame->fwd.width != info->width || frame->fwd.height != info->height || frame->bwd.width != info->width ||
        frame->bwd.height != info->height)
        return fail(ISTI_ERR_INVALID_ARG, "render resolution must equal the main keyframes' resolution");
    const int n_aux = frame->num_aux;
    if (n_aux < 0 || n_aux > ISTI_MAX_AUX_CAMS)
        return fail(ISTI_ERR_INVALID_ARG, "num_aux out of range");
    if (n_aux > 0 && (!frame->aux_curr || !frame->aux_next))
        return fail(ISTI_ERR_INVALID_ARG, "aux views are NULL");
    for (int i = 0; i < n_aux; i++)
    {
        const isti_view &a = frame->aux_curr[i], &b = frame->aux_next[i];
        if (!view_ok(a, why) || !view_ok(b, why))
            return fail(ISTI_ERR_INVALID_ARG, why);
        if (a.width != b.width || a.height != b.height)
            return fail(ISTI_ERR_INVALID_ARG, "aux curr/next sizes differ");
        // aux_idx = idx / (res / aux_res) must stay inside the aux image (src/renderer.cu:425,433)
        if (a.width > info->width || a.height > info->height || (info->width - 1) / (info->width / a.width) >= a.width ||
            (info->height - 1) / (info->height / a.height) >= a.height)
            return fail(ISTI_ERR_INVALID_ARG, "aux resolution incompatible with the render resolution");
    }
    n_views = 2 + 2 * n_aux;
    views[0] = &frame->fwd;
    views[1] = &frame->bwd;
    for (int i = 0; i < n_aux; i++)
    {
        views[2 + 2 * i] = &frame->aux_curr[i];
        views[3 + 2 * i] = &frame->aux_next[i];
    }
    return ISTI_OK;
}

struct Layout
{
    size_t key_frame_bytes, cam_frame_bytes; // one frame, every view
    size_t key_bytes, cam_bytes, ff_bytes, lut_bytes, total;
};

Layout layout_of(const isti_view *const *views, int n_views, int n_frames)
{
    Layout l{};
    for (int k = 0; k < n_views; k++)
    {
        const size_t px = (size_t)views[k]->width * views[k]->height;
        l.key_frame_bytes += align_up(px * 8, 256);
        l.cam_frame_bytes += align_up(px * 16, 256);
        l.lut_bytes += align_up((size_t)(views[k]->width + views[k]->height) * 4, 256);
    }
    l.ff_bytes = l.cam_frame_bytes;
    l.key_bytes = l.key_frame_bytes * n_frames;
    l.cam_bytes = l.cam_frame_bytes * n_frames;
    l.total = l.key_bytes + l.cam_bytes + l.ff_bytes + l.lut_bytes;
    return l;
}

// Fills the kernel parameters for one batch whose intermediates live at `base`.
void fill_params(isti::FrameParams &p, int n_frames, void *const *outs, const isti_render_info *infos, const isti_frame_data *frame,
                 const isti_view *const *views, int n_views, const Layout &l, char *base, bool chain)
{
    std::memset(&p, 0, sizeof p);
    const isti_render_info &info = infos[0];
    size_t off_key = 0, off_cam = l.key_bytes, off_full = l.key_bytes + l.cam_bytes, off_lut = l.key_bytes + l.cam_bytes + l.ff_bytes;
    for (int k = 0; k < n_views; k++)
    {
        const bool fw = (k % 2) == 0;
        const isti_view &v = *views[k];
        isti::DevView &d = p.v[k];
        d.color = static_cast<const uint32_t *>(v.color);
        d.z = v.z;
        d.motion = v.motion_format == ISTI_MOTION_NONE ? nullptr : v.motion;
        d.motion_fmt = v.motion_format;
        d.sha = static_cast<const uint32_t *>(v.shadow_color_a);
        d.shb = static_cast<const uint32_t *>(v.shadow_color_b);
        d.shi = static_cast<const uint32_t *>(v.shadow_info);
        d.w = v.width;
        d.h = v.height;
        d.sx = k < 2 ? 1u : info.width / v.width;
        d.sy = k < 2 ? 1u : info.height / v.height;
        d.forward = fw ? 1 : 0;
        d.priority = (k < 2 || !frame->aux_priority) ? 0 : frame->aux_priority[(k - 2) / 2];
        const uint32_t mn = v.width < v.height ? v.width : v.height;
        d.err_sx = (float)v.width / (float)mn;
        d.err_sy = (float)v.height / (float)mn;
        const float *vp_to = (k < 2) ? (fw ? frame->bwd.viewproj : frame->fwd.viewproj)
                                     : (fw ? frame->aux_next[(k - 2) / 2].viewproj : frame->aux_curr[(k - 2) / 2].viewproj);
        const float *vp_main = fw ? frame->fwd.viewproj : frame->bwd.viewproj;
        std::memcpy(d.inv_vp, v.inv_viewproj, sizeof d.inv_vp);
        std::memcpy(d.vp_to, vp_to, sizeof d.vp_to);
        std::memcpy(d.vp_main, vp_main, sizeof d.vp_main);
        const size_t px = (size_t)v.width * v.height;
        d.splat = reinterpret_cast<unsigned long long *>(base + off_key);
        d.cam_ff = reinterpret_cast<float4 *>(base + off_cam);
        d.full_ff = reinterpret_cast<float4 *>(base + off_full);
        d.lut = reinterpret_cast<float *>(base + off_lut);
        off_key += align_up(px * 8, 256);
        off_cam += align_up(px * 16, 256);
        off_full += align_up(px * 16, 256);
        off_lut += align_up((size_t)(v.width + v.height) * 4, 256);
    }
    for (int k = 0; k < n_frames; k++)
    {
        std::memcpy(p.cam_vp[k], infos[k].viewproj, sizeof p.cam_vp[k]);
        p.out[k] = static_cast<uint32_t *>(outs[k]);
        p.f[k].alpha = infos[k].alpha;
        p.f[k].fpa = infos[k].frames_per_anchor;
        p.f[k].sfpa = infos[k].shadow_frames_per_anchor;
        p.f[k].no_shadows = infos[k].no_shadows ? 1 : 0;
    }
    p.key_stride = l.key_frame_bytes / sizeof(unsigned long long);
    p.cam_stride = l.cam_frame_bytes / sizeof(float4);
    p.keys = reinterpret_cast<ulonglong2 *>(base);
    p.key_units = l.key_bytes / sizeof(ulonglong2);
    p.out_w = info.width;
    p.out_h = info.height;
    p.n_views = n_views;
    p.n_aux = frame->num_aux;
    p.n_frames = n_frames;
    p.linear = info.mode == ISTI_MODE_BACKWARD_BIDIRECTIONAL ? 1 : 0;
    p.chain = chain ? 1 : 0;
}

template <int SW, int SI, bool MAV, int G>
cudaError_t launch_reproj_g(const isti::FrameParams &p, cudaStream_t stream)
{
    const size_t smem = isti::reproj_smem<SW, G>(p.n_views, p.n_frames); // beyond 48 KiB for large batches
    if (smem > 48 * 1024)
    {
        cudaError_t e = cudaFuncSetAttribute(isti::reproj_kernel<SW, SI, MAV, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    const dim3 gr((p.out_w + 31) / 32, (p.out_h + isti::ROWS - 1) / isti::ROWS);
    isti::reproj_kernel<SW, SI, MAV, G><<<gr, dim3(32, p.n_views), smem, stream>>>(p);
    return cudaGetLastError();
}

// One frame searched at a time: measured on GB300 (1080p, 6 views, 3 frames), searching
// 2 or 3 frames together raises the register count to 64-92 and the launch time by ~65 %.
template <int SW, int SI, bool MAV>
cudaError_t launch_reproj(const isti::FrameParams &p, cudaStream_t stream)
{
    return launch_reproj_g<SW, SI, MAV, 1>(p, stream);
}

// Enqueues the three kernels of one batch; events (optional) are recorded after init and splat.
cudaError_t launch_batch(const isti::FrameParams &p, int mode, cudaStream_t stream, cudaEvent_t after_init, cudaEvent_t after_splat)
{
    uint32_t max_w = 0, max_h = 0;
    for (int k = 0; k < p.n_views; k++)
    {
        max_w = p.v[k].w > max_w ? p.v[k].w : max_w;
        max_h = p.v[k].h > max_h ? p.v[k].h : max_h;
    }
    // init: about 8 x 16-byte stores per thread, at least enough threads for the tables (<= 65535 entries)
    size_t init_blocks = (p.key_units + 8 * 256 - 1) / (8 * 256);
    if (init_blocks < 256)
        init_blocks = 256;
    if (init_blocks > 152 * 64)
        init_blocks = 152 * 64;
    isti::init_kernel<<<(unsigned)init_blocks, 256, 0, stream>>>(p);
    if (after_init)
        cudaEventRecord(after_init, stream);
    const dim3 gs((max_w + 31) / 32, (max_h + 7) / 8, p.n_views);
    isti::splat_kernel<<<gs, dim3(32, 8), 0, stream>>>(p);
    if (after_splat)
        cudaEventRecord(after_splat, stream);
    switch (mode)
    {
    case ISTI_MODE_OURS:
    case ISTI_MODE_BACKWARD_UNIDIRECTIONAL:
        return launch_reproj<1, 3, false>(p, stream);
    case ISTI_MODE_SPLATTING:
        return launch_reproj<1, 0, false>(p, stream);
    case ISTI_MODE_BACKWARD_BIDIRECTIONAL:
        return launch_reproj<3, 5, true>(p, stream);
    }
    return cudaGetLastError();
}

isti_status render_batch(isti_renderer *r, int n_frames, void *const *outs, const isti_render_info *infos, const isti_frame_data *frame,
                         bool chain, cudaStream_t stream)
{
    const isti_view *views[isti::MAX_VIEWS];
    int n_views = 0;
    isti_status st = validate(n_frames, outs, infos, frame, views, n_views);
    if (st != ISTI_OK)
        return st;
    const Layout l = layout_of(views, n_views, n_frames);

    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (cur != r->device)
        return fail(ISTI_ERR_INVALID_ARG, "renderer was created on another device");
    if (l.total > r->arena_bytes)
    {
        if (r->arena)
        {
            e = cudaFree(r->arena);
            r->arena = nullptr;
            r->arena_bytes = 0;
            if (e != cudaSuccess)
                return cuda_fail(e, "cudaFree");
        }
        e = cudaMalloc(&r->arena, l.total);
        if (e != cudaSuccess)
        {
            r->arena = nullptr;
            return e == cudaErrorMemoryAllocation ? fail(ISTI_ERR_OOM, "cudaMalloc of the renderer arena failed") : cuda_fail(e, "cudaMalloc");
        }
        r->arena_bytes = l.total;
    }
    char *base = static_cast<char *>(r->arena);
    fill_params(r->last, n_frames, outs, infos, frame, views, n_views, l, base, chain);

    cudaEvent_t *ev = nullptr;
    if (r->timing)
    {
        if (r->events_used + 4 > r->events.size())
            for (int i = 0; i < 4; i++)
            {
                cudaEvent_t x;
                e = cudaEventCreate(&x);
                if (e != cudaSuccess)
                    return cuda_fail(e, "cudaEventCreate");
                r->events.push_back(x);
            }
        r->event_frames.resize(r->events.size() / 4);
        r->event_frames[r->events_used / 4] = n_frames;
        ev = &r->events[r->events_used];
        r->events_used += 4;
        r->timed_launches += 3;
        cudaEventRecord(ev[0], stream);
    }
    e = launch_batch(r->last, infos[0].mode, stream, ev ? ev[1] : nullptr, ev ? ev[2] : nullptr);
    if (ev)
        cudaEventRecord(ev[3], stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    r->has_frame = true;
    return ISTI_OK;
}
} // namespace

extern "C" {

int32_t isti_abi_version(void) { return ISTI_ABI_VERSION; }

const char *isti_last_error(void) { return g_last_error.c_str(); }

const char *isti_status_string(isti_status s)
{
    switch (s)
    {
    case ISTI_OK: return "ok";
    case ISTI_ERR_INVALID_ARG: return "invalid argument";
    case ISTI_ERR_OOM: return "out of device memory";
    case ISTI_ERR_CUDA: return "CUDA error";
    case ISTI_ERR_TIMEOUT: return "timeout";
    case ISTI_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

isti_status isti_renderer_create(isti_renderer **out)
{
    if (!out)
        return fail(ISTI_ERR_INVALID_ARG, "out is NULL");
    isti_renderer *r = new (std::nothrow) isti_renderer();
    if (!r)
        return fail(ISTI_ERR_OOM, "host allocation failed");
    cudaError_t e = cudaGetDevice(&r->device);
    if (e != cudaSuccess)
    {
        delete r;
        return cuda_fail(e, "cudaGetDevice");
    }
    *out = r;
    return ISTI_OK;
}

isti_status isti_renderer_destroy(isti_renderer *r)
{
    if (!r)
        return ISTI_OK;
    isti_status s = ISTI_OK;
    for (cudaEvent_t ev : r->events)
        cudaEventDestroy(ev);
    if (r->arena)
    {
        cudaError_t e = cudaFree(r->arena);
        if (e != cudaSuccess)
            s = cuda_fail(e, "cudaFree");
    }
    delete r;
    return s;
}

isti_status isti_render(isti_renderer *r, void *out_rgba, const isti_render_info *info, const isti_frame_data *frame, void *stream)
{
    if (!r || !out_rgba || !info || !frame)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    void *outs[1] = {out_rgba};
    return render_batch(r, 1, outs, info, frame, false, static_cast<cudaStream_t>(stream));
}

isti_status isti_render_batch(isti_renderer *r, int32_t n_frames, void *const *out_rgba, const isti_render_info *infos,
                              const isti_frame_data *frame, int32_t chain_outputs, void *stream)
{
    if (!r || !out_rgba || !infos || !frame)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    return render_batch(r, n_frames, out_rgba, infos, frame, chain_outputs != 0, static_cast<cudaStream_t>(stream));
}

isti_status isti_renderer_enable_timing(isti_renderer *r, int32_t on)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "renderer is NULL");
    r->timing = on != 0;
    return ISTI_OK;
}

isti_status isti_renderer_timing(isti_renderer *r, isti_timing *out)
{
    if (!r || !out)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    std::memset(out, 0, sizeof *out);
    for (size_t i = 0; i + 4 <= r->events_used; i += 4)
    {
        cudaError_t e = cudaEventSynchronize(r->events[i + 3]);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaEventSynchronize");
        float a = 0.f, b = 0.f, c = 0.f;
        cudaEventElapsedTime(&a, r->events[i], r->events[i + 1]);
        cudaEventElapsedTime(&b, r->events[i + 1], r->events[i + 2]);
        cudaEventElapsedTime(&c, r->events[i + 2], r->events[i + 3]);
        out->init_ms += a;
        out->splat_ms += b;
        out->reproj_ms += c;
        out->frames += r->event_frames[i / 4];
    }
    out->kernel_launches = r->timed_launches;
    r->events_used = 0;
    r->timed_launches = 0;
    return ISTI_OK;
}

isti_status isti_renderer_view_buffers(const isti_renderer *r, int32_t view, const uint64_t **splat, const float **cam_ff,
                                       const float **full_ff, uint32_t *width, uint32_t *height)
{
    if (!r || !r->has_frame)
        return fail(ISTI_ERR_INVALID_ARG, "no frame rendered yet");
    const int nv = r->last.n_views;
    if (view < 0 || view >= nv * r->last.n_frames)
        return fail(ISTI_ERR_INVALID_ARG, "view index out of range");
    const int k = view / nv;
    const isti::DevView &d = r->last.v[view % nv];
    if (splat)
        *splat = reinterpret_cast<const uint64_t *>(d.splat + k * r->last.key_stride);
    if (cam_ff)
        *cam_ff = reinterpret_cast<const float *>(d.cam_ff + k * r->last.cam_stride);
    if (full_ff)
        *full_ff = reinterpret_cast<const float *>(d.full_ff);
    if (width)
        *width = d.w;
    if (height)
        *height = d.h;
    return ISTI_OK;
}

} // extern "C"

// ============================ rendering without allocation ============================
//
// isti_render_noalloc serves callers that may not allocate device memory while
// they run (a host whose device budget is reserved up front by its own pool, a
// real-time loop where cudaMalloc/cudaFree can synchronise the device).  Its
// intermediates live in g_noalloc_scratch below instead of a renderer arena;
// the kernels are the ones isti_render launches.

namespace
{
// Fixed scratch for isti_render_noalloc: ISTI_NOALLOC_SCRATCH_BYTES (64 MiB), loaded
// with the module on every GPU that uses the library and kept until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[ISTI_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device.  In host code the
// array's name only denotes a host-side shadow, so the address is looked up once
// per device (with that device current) and cached.
isti_status noalloc_scratch(int device, char **out)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return fail(ISTI_ERR_UNSUPPORTED, "device ordinal beyond the no-allocation scratch table");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device])
    {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[device] = p;
    }
    *out = static_cast<char *>(g_noalloc_ptr[device]);
    return ISTI_OK;
}
} // namespace

extern "C" isti_status isti_render_noalloc(void *out_rgba, const isti_render_info *info, const isti_frame_data *frame, void *stream_ptr)
{
    if (!out_rgba || !info || !frame)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    void *outs[1] = {out_rgba};
    const isti_view *views[isti::MAX_VIEWS];
    int n_views = 0;
    isti_status st = validate(1, outs, info, frame, views, n_views);
    if (st != ISTI_OK)
        return st;
    const Layout l = layout_of(views, n_views, 1);
    if (l.total > ISTI_NOALLOC_SCRATCH_BYTES)
        return fail(ISTI_ERR_INVALID_ARG, "frame needs " + std::to_string(l.total) + " bytes of scratch; isti_render_noalloc holds at most " +
                                              std::to_string((size_t)ISTI_NOALLOC_SCRATCH_BYTES) + " (use isti_render for larger frames)");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    char *base = nullptr;
    st = noalloc_scratch(device, &base);
    if (st != ISTI_OK)
        return st;
    isti::FrameParams p;
    fill_params(p, 1, outs, info, frame, views, n_views, l, base, false);
    // The array keeps the previous call's contents: the init kernel resets every key to
    // the reference's empty value (all bytes 0xfe) and rewrites the tables; the flow
    // fields are fully rewritten by the splat kernel before the reprojection reads them.
    e = launch_batch(p, info->mode, static_cast<cudaStream_t>(stream_ptr), nullptr, nullptr);
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    return ISTI_OK;
}
