// Per-frame interpolation path on GB300: splat kernel + bidirectional
// reprojection kernel, and the C ABI of include/isti.h.
//
// Reference: src/renderer.cu (DerThomy/ImageBasedSpatioTemporalInterpolation).
//
// Layout in HBM (renderer-owned arena, one allocation):
//   [splat keys of every view, u64 per pixel][cam flow f32x4 per pixel, every view][full flow f32x4, every view]
// The key block is contiguous so one memset initialises all views.
// Pixel inputs are caller-owned device images (include/isti.h).
//
// Launches per frame: 1 memset + 1 splat launch (all 2 + 2 * n_aux source
// views, blockIdx.z = view) + 1 reprojection launch (one thread per output
// pixel).  Nothing blocks the host.
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

struct DevView
{
    const uint32_t *color;  // RGBA8 packed, R in bits 0-7
    const float *z;
    const void *motion;
    const uint32_t *sha, *shb, *shi;
    unsigned long long *splat;
    float4 *cam_ff;
    float4 *full_ff;
    uint32_t w, h;
    int32_t motion_fmt;
    int32_t forward;
    int32_t priority;
    float weight;
    float err_sx, err_sy;   // res / min(res.x, res.y), computeReprojError scale (src/renderer.cu:213)
    float inv_vp[16];       // this view's inverse viewproj
    float vp_to[16];        // the other keyframe's viewproj (same camera)
    float vp_main[16];      // main camera viewproj at this keyframe (visible_in_main test)
};

struct FrameParams
{
    DevView v[MAX_VIEWS];
    float cam_vp[16];
    uint32_t *out;
    uint32_t out_w, out_h;
    float alpha;
    int32_t n_views, n_aux;
    int32_t fpa, sfpa, no_shadows, linear;
};

// ---- border-addressed loads: zero outside the image (cudaAddressModeBorder) ----

__device__ __forceinline__ float ld_f(const float *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (size_t)y * w + x) : 0.0f;
}
__device__ __forceinline__ float4 ld_f4(const float4 *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (size_t)y * w + x) : make_float4(0.f, 0.f, 0.f, 0.f);
}
__device__ __forceinline__ uint32_t ld_c(const uint32_t *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (size_t)y * w + x) : 0u;
}

__device__ __forceinline__ float4 load_motion(const DevView &v, size_t idx)
{
    if (v.motion_fmt == ISTI_MOTION_F32X4)
        return __ldg(static_cast<const float4 *>(v.motion) + idx);
    if (v.motion_fmt == ISTI_MOTION_F16X3)
    {
        const __half *m = static_cast<const __half *>(v.motion) + 3 * idx;
        return make_float4(__half2float(m[0]), __half2float(m[1]), __half2float(m[2]), 0.0f);
    }
    return make_float4(0.f, 0.f, 0.f, 0.f);
}

// ---- computeFlowFields_sortedSplatting_kernel, src/renderer.cu:76-146 ----

__global__ void __launch_bounds__(256) splat_kernel(const __grid_constant__ FrameParams p)
{
    const DevView &v = p.v[blockIdx.z];
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= v.w || y >= v.h)
        return;
    const size_t idx = (size_t)y * v.w + x;

    const float z_from = __ldg(v.z + idx);
    const float4 om = load_motion(v, idx);
    const float2 pcs = pixel2cs(x, y, v.w, v.h);
    const float4 cs_from = make_float4(pcs.x, pcs.y, z_from, 1.0f);
    const float4 ws_from = project(v.inv_vp, cs_from);
    const float4 moved = make_float4(__fadd_rn(pcs.x, om.x), __fadd_rn(pcs.y, om.y), __fadd_rn(z_from, om.z), 1.0f);
    const float4 ws_to = project(v.inv_vp, moved);

    const float4 cm = project(v.vp_main, ws_from);
    const float lim = 1.0f - 1e-3f;
    const bool visible = cm.x > -lim && cm.x < lim && cm.y > -lim && cm.y < lim && cm.z > -lim && cm.z < lim;
    const float vis = visible ? 1.0f : 0.0f;

    const float wg = v.weight;
    const float4 scaled = make_float4(__fadd_rn(ws_from.x, __fmul_rn(wg, __fsub_rn(ws_to.x, ws_from.x))),
                                      __fadd_rn(ws_from.y, __fmul_rn(wg, __fsub_rn(ws_to.y, ws_from.y))),
                                      __fadd_rn(ws_from.z, __fmul_rn(wg, __fsub_rn(ws_to.z, ws_from.z))),
                                      __fadd_rn(ws_from.w, __fmul_rn(wg, __fsub_rn(ws_to.w, ws_from.w))));
    const float4 cs_to = project(v.vp_to, ws_to);
    const float fmx = __fsub_rn(cs_to.x, cs_from.x), fmy = __fsub_rn(cs_to.y, cs_from.y), fmz = __fsub_rn(cs_to.z, cs_from.z);
    v.full_ff[idx] = make_float4(fmx, fmy, fmz, vis);

    float depth = z_to_depth(z_from);
    uint32_t tx = x, ty = y;
    if (!p.linear)
    {
        const float4 pc = project(p.cam_vp, scaled);
        v.cam_ff[idx] = make_float4(__fsub_rn(pc.x, cs_from.x), __fsub_rn(pc.y, cs_from.y), __fsub_rn(pc.z, cs_from.z), vis);
        const float depth_cam = z_to_depth(pc.z);
        const int2 pix = cs2pixel(pc.x, pc.y, v.w, v.h);
        if (!in_range(pix, v.w, v.h) || depth_cam < 0.0f)
            return;
        depth = depth_cam;
        tx = (uint32_t)pix.x;
        ty = (uint32_t)pix.y;
    }
    else
    {
        v.cam_ff[idx] = make_float4(__fmul_rn(fmx, wg), __fmul_rn(fmy, wg), __fmul_rn(fmz, wg), vis);
    }
    atomicMin(v.splat + (size_t)ty * v.w + tx, encode_key(depth, x, y));
}

// ---- bidirectional reprojection, src/renderer.cu:148-465 ----

struct Result
{
    bool valid;
    bool vis;
    int32_t priority;
    float error;
    float depth;
    uint32_t color;
};

// initializeSearchFromSplatting<W>, src/renderer.cu:148-175
template <int W>
__device__ __forceinline__ KeyInfo init_search(uint32_t ix, uint32_t iy, const DevView &v)
{
    const unsigned long long *sp = v.splat;
    KeyInfo lowest = decode_key(__ldg(sp + (size_t)iy * v.w + ix));
#pragma unroll
    for (int yo = -W; yo <= W; yo++)
#pragma unroll
        for (int xo = -W; xo <= W; xo++)
        {
            const int2 n = make_int2((int)ix + xo, (int)iy + yo);
            if (!in_range(n, v.w, v.h))
                continue;
            const KeyInfo cur = decode_key(__ldg(sp + (size_t)n.y * v.w + n.x));
            if (cur.depth > 0.0f && (!isfinite(lowest.depth) || lowest.depth < 0.0f || cur.depth < lowest.depth))
                lowest = cur;
        }
    return lowest;
}

// iterativeSearch<N>, src/renderer.cu:177-202
template <int N>
__device__ __forceinline__ void iterative_search(uint32_t &sx, uint32_t &sy, float2 q, const DevView &v)
{
#pragma unroll
    for (int i = 0; i < N; i++)
    {
        const float4 m = ld_f4(v.cam_ff, sx, sy, v.w, v.h);
        const int2 t = cs2pixel(__fsub_rn(q.x, m.x), __fsub_rn(q.y, m.y), v.w, v.h);
        if (!in_range(t, v.w, v.h))
            continue;
        sx = (uint32_t)t.x;
        sy = (uint32_t)t.y;
    }
}

// computeReprojError, src/renderer.cu:204-215
__device__ __forceinline__ float reproj_error(uint32_t sx, uint32_t sy, const DevView &v, float2 pcs, float4 m)
{
    const float2 pf = pixel2cs(sx, sy, v.w, v.h);
    float ex = __fsub_rn(__fadd_rn(pf.x, m.x), pcs.x);
    float ey = __fsub_rn(__fadd_rn(pf.y, m.y), pcs.y);
    ex = __fmul_rn(ex, v.err_sx);
    ey = __fmul_rn(ey, v.err_sy);
    return __fsqrt_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)));
}

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

// colorFromShadow (two sub-frame form), src/renderer.cu:270-295
__device__ uint32_t color_from_shadow(uint32_t sfx, uint32_t sfy, float sft, const FrameParams &p, const DevView &v, uint32_t px,
                                      uint32_t py)
{
    if (p.no_shadows || sfx >= (uint32_t)p.sfpa || sfy == 0 || v.sha == nullptr)
        return ld_c(v.color, px, py, v.w, v.h);
    const int32_t sfpa = p.sfpa;
    const uint32_t vx = (uint32_t)(v.forward ? (int32_t)sfx : sfpa - (int32_t)sfx);
    const uint32_t vy = (uint32_t)(v.forward ? (int32_t)sfy : sfpa - (int32_t)sfy);
    if (vx == vy || vy >= (uint32_t)sfpa)
        return color_from_shadow_idx(vx, sfpa, v, px, py);
    if (vx >= (uint32_t)sfpa)
        return color_from_shadow_idx(vy, sfpa, v, px, py);
    const uint32_t a = color_from_shadow_idx(vx, sfpa, v, px, py);
    const uint32_t b = color_from_shadow_idx(vy, sfpa, v, px, py);
    return lerp_color_u8(a, b, sft);
}

struct ShadowFrames
{
    uint32_t frame_idx, sfx, sfy;
    float sft;
};

// secondChanceAndBlend_kernel<EPS_2>, src/renderer.cu:297-327
__device__ uint32_t second_chance(float weight, const ShadowFrames &sf, uint32_t sx, uint32_t sy, const FrameParams &p, const DevView &from,
                                  const DevView &to, float eps2)
{
    const float4 m_ft = ld_f4(from.full_ff, sx, sy, from.w, from.h);
    const float2 spcs = pixel2cs(sx, sy, from.w, from.h);
    const float sz = ld_f(from.z, sx, sy, from.w, from.h);
    const float pcx = __fadd_rn(spcs.x, m_ft.x), pcy = __fadd_rn(spcs.y, m_ft.y), pcz = __fadd_rn(sz, m_ft.z);
    const int2 pp = cs2pixel(pcx, pcy, to.w, to.h);

    uint32_t out = color_from_shadow(sf.sfx, sf.sfy, sf.sft, p, from, sx, sy);
    if (sf.frame_idx >= (uint32_t)p.fpa)
        return out;
    if (in_range(pp, to.w, to.h))
    {
        const float az = ld_f(to.z, pp.x, pp.y, to.w, to.h);
        const float4 m_tf = ld_f4(to.full_ff, pp.x, pp.y, to.w, to.h);
        const float dx = __fsub_rn(m_ft.x, -m_tf.x), dy = __fsub_rn(m_ft.y, -m_tf.y), dz = __fsub_rn(m_ft.z, -m_tf.z);
        const float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        if (dist < EPS_3 && fabsf(__fsub_rn(az, pcz)) < eps2)
            out = lerp_color_u8(color_from_shadow(sf.sfx, sf.sfy, sf.sft, p, to, pp.x, pp.y), out, weight);
    }
    return out;
}

// bidirectionalReprojection<SW, SI, ALWAYS_VALID, EPS_1, EPS_2>, src/renderer.cu:329-398
template <int SW, int SI, bool ALWAYS_VALID>
__device__ __forceinline__ Result bidir(uint32_t ix, uint32_t iy, float2 q_full, float2 pcs, const ShadowFrames &sf, const FrameParams &p,
                                        const DevView &fwd, const DevView &bwd, float eps1, float eps2)
{
    float fwd_e = 3.402823466e+38f; // FLT_MAX
    bool fwd_vis = false;
    KeyInfo fi = init_search<SW>(ix, iy, fwd);
    if (fi.depth > 0.0f && p.alpha < 1.0f)
    {
        iterative_search<SI>(fi.sx, fi.sy, q_full, fwd);
        const float4 m = ld_f4(fwd.cam_ff, fi.sx, fi.sy, fwd.w, fwd.h);
        fi.depth = z_to_depth(__fadd_rn(ld_f(fwd.z, fi.sx, fi.sy, fwd.w, fwd.h), m.z));
        fwd_e = reproj_error(fi.sx, fi.sy, fwd, pcs, m);
        fwd_vis = m.w > 0.0f;
    }
    float bwd_e = 3.402823466e+38f;
    bool bwd_vis = false;
    KeyInfo bi = init_search<SW>(ix, iy, bwd);
    if (bi.depth > 0.0f)
    {
        iterative_search<SI>(bi.sx, bi.sy, q_full, bwd);
        const float4 m = ld_f4(bwd.cam_ff, bi.sx, bi.sy, bwd.w, bwd.h);
        bi.depth = z_to_depth(__fadd_rn(ld_f(bwd.z, bi.sx, bi.sy, bwd.w, bwd.h), m.z));
        bwd_e = reproj_error(bi.sx, bi.sy, bwd, pcs, m);
        bwd_vis = m.w > 0.0f;
    }

    Result r;
    r.valid = false;
    r.vis = false;
    r.priority = 0;
    r.error = 0.0f; // indeterminate in the reference for the always-valid blend
    r.depth = 0.0f;
    r.color = 0u;
    if (fwd_e < eps1 || bwd_e < eps1)
    {
        const bool both = fwd_e < eps1 && bwd_e < eps1;
        const bool similar = fabsf(__fsub_rn(depth_to_z(fi.depth), depth_to_z(bi.depth))) < eps2;
        const bool choose_fwd = (both && !similar && fi.depth < bi.depth) || ((!both || similar) && fwd_e < bwd_e);
        r.valid = true;
        if (choose_fwd)
        {
            r.vis = fwd_vis || (both && similar && bwd_vis);
            r.priority = fwd.priority;
            r.error = fwd_e;
            r.depth = fi.depth;
            r.color = second_chance(__fsub_rn(1.0f, p.alpha), sf, fi.sx, fi.sy, p, fwd, bwd, eps2);
        }
        else
        {
            r.vis = bwd_vis || (both && similar && fwd_vis);
            r.priority = bwd.priority;
            r.error = bwd_e;
            r.depth = bi.depth;
            r.color = second_chance(p.alpha, sf, bi.sx, bi.sy, p, bwd, fwd, eps2);
        }
    }
    else if (ALWAYS_VALID)
    {
        r.valid = true;
        const uint32_t cf = second_chance(__fsub_rn(1.0f, p.alpha), sf, fi.sx, fi.sy, p, fwd, bwd, eps2);
        const uint32_t cb = second_chance(p.alpha, sf, bi.sx, bi.sy, p, bwd, fwd, eps2);
        r.color = lerp_color_u8(cf, cb, 0.5f);
    }
    return r;
}

// bidirectionalReprojection_kernel<SW, SI, MAIN_ALWAYS_VALID>, src/renderer.cu:400-465
template <int SW, int SI, bool MAV>
__global__ void __launch_bounds__(256) reproj_kernel(const __grid_constant__ FrameParams p)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.out_w || y >= p.out_h)
        return;

    // frame_idx / shadow sub-frames, src/renderer.cu:359-364
    ShadowFrames sf;
    const float fa = __fmul_rn((float)p.fpa, p.alpha);
    const float sa = __fmul_rn((float)p.sfpa, p.alpha);
    sf.frame_idx = __float2uint_rn(fa);
    sf.sfx = __float2uint_rd(__fadd_rn(sa, 1e-9f));
    sf.sfy = __float2uint_ru(__fsub_rn(sa, 1e-9f));
    sf.sft = __fsub_rn(sa, (float)sf.sfx);

    const float2 pcs = pixel2cs(x, y, p.out_w, p.out_h);
    uint32_t *o = p.out + (size_t)y * p.out_w + x;
    const Result m = bidir<SW, SI, MAV>(x, y, pcs, pcs, sf, p, p.v[0], p.v[1], EPS_1_FULL_RES, EPS_2_FULL_RES);
    if (m.valid)
        *o = m.color;
    if (p.n_aux <= 0)
        return;

    Result best;
    best.valid = false;
    best.vis = false;
    best.priority = 0;
    best.error = 0.0f;
    best.depth = 0.0f;
    best.color = 0u;
    for (int i = 0; i < p.n_aux; i++)
    {
        const DevView &vf = p.v[2 + 2 * i];
        const DevView &vb = p.v[3 + 2 * i];
        const uint32_t ax = x / (p.out_w / vf.w), ay = y / (p.out_h / vf.h);
        const float2 apcs = pixel2cs(ax, ay, vf.w, vf.h);
        const Result r = bidir<SW, SI, false>(ax, ay, pcs, apcs, sf, p, vf, vb, EPS_1_LOW_RES, EPS_2_LOW_RES);
        if (!best.valid)
            best = r;
        else if (r.valid)
        {
            const bool similar = fabsf(__fsub_rn(depth_to_z(best.depth), depth_to_z(r.depth))) < EPS_2_LOW_RES;
            const bool choose_new = (!similar && r.depth < best.depth) || (similar && r.priority >= best.priority && r.error < best.error);
            if (choose_new)
                best = r;
        }
    }
    if (best.valid)
    {
        bool choose_aux = !m.valid;
        if (m.valid && !best.vis)
        {
            const bool similar = fabsf(__fsub_rn(depth_to_z(best.depth), depth_to_z(m.depth))) < EPS_2_LOW_RES;
            choose_aux = !similar && best.depth < m.depth;
        }
        if (choose_aux)
            *o = best.color;
    }
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
    // stage timing: 4 events per timed render (before init, after init, after splat, after reproj)
    bool timing = false;
    std::vector<cudaEvent_t> events;
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

void fill_view(isti::DevView &d, const isti_view &v, int forward, int priority, float weight, const float *vp_to, const float *vp_main)
{
    d.color = static_cast<const uint32_t *>(v.color);
    d.z = v.z;
    d.motion = v.motion_format == ISTI_MOTION_NONE ? nullptr : v.motion;
    d.motion_fmt = v.motion_format;
    d.sha = static_cast<const uint32_t *>(v.shadow_color_a);
    d.shb = static_cast<const uint32_t *>(v.shadow_color_b);
    d.shi = static_cast<const uint32_t *>(v.shadow_info);
    d.w = v.width;
    d.h = v.height;
    d.forward = forward;
    d.priority = priority;
    d.weight = weight;
    const uint32_t mn = v.width < v.height ? v.width : v.height;
    d.err_sx = (float)v.width / (float)mn;
    d.err_sy = (float)v.height / (float)mn;
    std::memcpy(d.inv_vp, v.inv_viewproj, sizeof d.inv_vp);
    std::memcpy(d.vp_to, vp_to, sizeof d.vp_to);
    std::memcpy(d.vp_main, vp_main, sizeof d.vp_main);
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

isti_status isti_render(isti_renderer *r, void *out_rgba, const isti_render_info *info, const isti_frame_data *frame, void *stream_ptr)
{
    if (!r || !out_rgba || !info || !frame)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    if (reinterpret_cast<uintptr_t>(out_rgba) & 3u)
        return fail(ISTI_ERR_INVALID_ARG, "out_rgba must be 4-byte aligned");
    if (info->mode == ISTI_MODE_TIMEWARP)
        return fail(ISTI_ERR_UNSUPPORTED, "timewarp mode is not implemented");
    if (info->mode < 0 || info->mode > ISTI_MODE_TIMEWARP)
        return fail(ISTI_ERR_INVALID_ARG, "unknown render mode");
    if (info->shadow_frames_per_anchor < 0 || info->shadow_frames_per_anchor > 16)
        return fail(ISTI_ERR_INVALID_ARG, "shadow_frames_per_anchor must be 0..16");
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

    const int n_views = 2 + 2 * n_aux;
    const isti_view *views[isti::MAX_VIEWS];
    views[0] = &frame->fwd;
    views[1] = &frame->bwd;
    for (int i = 0; i < n_aux; i++)
    {
        views[2 + 2 * i] = &frame->aux_curr[i];
        views[3 + 2 * i] = &frame->aux_next[i];
    }
    size_t key_bytes = 0, ff_bytes = 0;
    size_t px[isti::MAX_VIEWS];
    for (int k = 0; k < n_views; k++)
    {
        px[k] = (size_t)views[k]->width * views[k]->height;
        key_bytes += align_up(px[k] * 8, 256);
        ff_bytes += align_up(px[k] * 16, 256);
    }
    const size_t need = key_bytes + 2 * ff_bytes;

    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (cur != r->device)
        return fail(ISTI_ERR_INVALID_ARG, "renderer was created on another device");
    if (need > r->arena_bytes)
    {
        if (r->arena)
        {
            e = cudaFree(r->arena);
            r->arena = nullptr;
            r->arena_bytes = 0;
            if (e != cudaSuccess)
                return cuda_fail(e, "cudaFree");
        }
        e = cudaMalloc(&r->arena, need);
        if (e != cudaSuccess)
        {
            r->arena = nullptr;
            return e == cudaErrorMemoryAllocation ? fail(ISTI_ERR_OOM, "cudaMalloc of the renderer arena failed") : cuda_fail(e, "cudaMalloc");
        }
        r->arena_bytes = need;
    }

    isti::FrameParams &p = r->last;
    std::memset(&p, 0, sizeof p);
    char *base = static_cast<char *>(r->arena);
    size_t off_key = 0, off_cam = key_bytes, off_full = key_bytes + ff_bytes;
    const float alpha = info->alpha;
    const float one_minus_alpha = 1.0f - alpha;
    uint32_t max_w = 0, max_h = 0;
    for (int k = 0; k < n_views; k++)
    {
        const bool fw = (k % 2) == 0;
        const isti_view &v = *views[k];
        const float *vp_to = (k < 2) ? (fw ? frame->bwd.viewproj : frame->fwd.viewproj)
                                     : (fw ? frame->aux_next[(k - 2) / 2].viewproj : frame->aux_curr[(k - 2) / 2].viewproj);
        const float *vp_main = fw ? frame->fwd.viewproj : frame->bwd.viewproj;
        const int prio = (k < 2 || !frame->aux_priority) ? 0 : frame->aux_priority[(k - 2) / 2];
        fill_view(p.v[k], v, fw ? 1 : 0, prio, fw ? alpha : one_minus_alpha, vp_to, vp_main);
        p.v[k].splat = reinterpret_cast<unsigned long long *>(base + off_key);
        p.v[k].cam_ff = reinterpret_cast<float4 *>(base + off_cam);
        p.v[k].full_ff = reinterpret_cast<float4 *>(base + off_full);
        off_key += align_up(px[k] * 8, 256);
        off_cam += align_up(px[k] * 16, 256);
        off_full += align_up(px[k] * 16, 256);
        max_w = v.width > max_w ? v.width : max_w;
        max_h = v.height > max_h ? v.height : max_h;
    }
    std::memcpy(p.cam_vp, info->viewproj, sizeof p.cam_vp);
    p.out = static_cast<uint32_t *>(out_rgba);
    p.out_w = info->width;
    p.out_h = info->height;
    p.alpha = alpha;
    p.n_views = n_views;
    p.n_aux = n_aux;
    p.fpa = info->frames_per_anchor;
    p.sfpa = info->shadow_frames_per_anchor;
    p.no_shadows = info->no_shadows ? 1 : 0;
    p.linear = info->mode == ISTI_MODE_BACKWARD_BIDIRECTIONAL ? 1 : 0;

    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
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
        ev = &r->events[r->events_used];
        r->events_used += 4;
        r->timed_launches += 2;
        cudaEventRecord(ev[0], stream);
    }
    e = cudaMemsetAsync(base, 0xfe, key_bytes, stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemsetAsync");
    if (ev)
        cudaEventRecord(ev[1], stream);
    const dim3 blk(32, 8);
    const dim3 gs((max_w + 31) / 32, (max_h + 7) / 8, n_views);
    isti::splat_kernel<<<gs, blk, 0, stream>>>(p);
    if (ev)
        cudaEventRecord(ev[2], stream);
    const dim3 gr((info->width + 31) / 32, (info->height + 7) / 8);
    switch (info->mode)
    {
    case ISTI_MODE_OURS:
    case ISTI_MODE_BACKWARD_UNIDIRECTIONAL:
        isti::reproj_kernel<1, 3, false><<<gr, blk, 0, stream>>>(p);
        break;
    case ISTI_MODE_SPLATTING:
        isti::reproj_kernel<1, 0, false><<<gr, blk, 0, stream>>>(p);
        break;
    case ISTI_MODE_BACKWARD_BIDIRECTIONAL:
        isti::reproj_kernel<3, 5, true><<<gr, blk, 0, stream>>>(p);
        break;
    }
    if (ev)
        cudaEventRecord(ev[3], stream);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    r->has_frame = true;
    return ISTI_OK;
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
        out->frames += 1;
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
    if (view < 0 || view >= r->last.n_views)
        return fail(ISTI_ERR_INVALID_ARG, "view index out of range");
    const isti::DevView &d = r->last.v[view];
    if (splat)
        *splat = reinterpret_cast<const uint64_t *>(d.splat);
    if (cam_ff)
        *cam_ff = reinterpret_cast<const float *>(d.cam_ff);
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
// splat keys and flow fields live in g_noalloc_scratch below instead of a
// renderer arena; the kernels are the ones isti_render launches.

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
    if (reinterpret_cast<uintptr_t>(out_rgba) & 3u)
        return fail(ISTI_ERR_INVALID_ARG, "out_rgba must be 4-byte aligned");
    if (info->mode == ISTI_MODE_TIMEWARP)
        return fail(ISTI_ERR_UNSUPPORTED, "timewarp mode is not implemented");
    if (info->mode < 0 || info->mode > ISTI_MODE_TIMEWARP)
        return fail(ISTI_ERR_INVALID_ARG, "unknown render mode");
    if (info->shadow_frames_per_anchor < 0 || info->shadow_frames_per_anchor > 16)
        return fail(ISTI_ERR_INVALID_ARG, "shadow_frames_per_anchor must be 0..16");
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
        if (a.width > info->width || a.height > info->height || (info->width - 1) / (info->width / a.width) >= a.width ||
            (info->height - 1) / (info->height / a.height) >= a.height)
            return fail(ISTI_ERR_INVALID_ARG, "aux resolution incompatible with the render resolution");
    }

    const int n_views = 2 + 2 * n_aux;
    const isti_view *views[isti::MAX_VIEWS];
    views[0] = &frame->fwd;
    views[1] = &frame->bwd;
    for (int i = 0; i < n_aux; i++)
    {
        views[2 + 2 * i] = &frame->aux_curr[i];
        views[3 + 2 * i] = &frame->aux_next[i];
    }
    size_t key_bytes = 0, ff_bytes = 0, px[isti::MAX_VIEWS];
    for (int k = 0; k < n_views; k++)
    {
        px[k] = (size_t)views[k]->width * views[k]->height;
        key_bytes += align_up(px[k] * 8, 256);
        ff_bytes += align_up(px[k] * 16, 256);
    }
    const size_t need = key_bytes + 2 * ff_bytes;
    if (need > ISTI_NOALLOC_SCRATCH_BYTES)
        return fail(ISTI_ERR_INVALID_ARG, "frame needs " + std::to_string(need) + " bytes of scratch; isti_render_noalloc holds at most " +
                                              std::to_string((size_t)ISTI_NOALLOC_SCRATCH_BYTES) + " (use isti_render for larger frames)");

    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    char *base = nullptr;
    isti_status st = noalloc_scratch(device, &base);
    if (st != ISTI_OK)
        return st;

    isti::FrameParams p;
    std::memset(&p, 0, sizeof p);
    size_t off_key = 0, off_cam = key_bytes, off_full = key_bytes + ff_bytes;
    const float alpha = info->alpha;
    const float one_minus_alpha = 1.0f - alpha;
    uint32_t max_w = 0, max_h = 0;
    for (int k = 0; k < n_views; k++)
    {
        const bool fw = (k % 2) == 0;
        const isti_view &v = *views[k];
        const float *vp_to = (k < 2) ? (fw ? frame->bwd.viewproj : frame->fwd.viewproj)
                                     : (fw ? frame->aux_next[(k - 2) / 2].viewproj : frame->aux_curr[(k - 2) / 2].viewproj);
        const float *vp_main = fw ? frame->fwd.viewproj : frame->bwd.viewproj;
        const int prio = (k < 2 || !frame->aux_priority) ? 0 : frame->aux_priority[(k - 2) / 2];
        fill_view(p.v[k], v, fw ? 1 : 0, prio, fw ? alpha : one_minus_alpha, vp_to, vp_main);
        p.v[k].splat = reinterpret_cast<unsigned long long *>(base + off_key);
        p.v[k].cam_ff = reinterpret_cast<float4 *>(base + off_cam);
        p.v[k].full_ff = reinterpret_cast<float4 *>(base + off_full);
        off_key += align_up(px[k] * 8, 256);
        off_cam += align_up(px[k] * 16, 256);
        off_full += align_up(px[k] * 16, 256);
        max_w = v.width > max_w ? v.width : max_w;
        max_h = v.height > max_h ? v.height : max_h;
    }
    std::memcpy(p.cam_vp, info->viewproj, sizeof p.cam_vp);
    p.out = static_cast<uint32_t *>(out_rgba);
    p.out_w = info->width;
    p.out_h = info->height;
    p.alpha = alpha;
    p.n_views = n_views;
    p.n_aux = n_aux;
    p.fpa = info->frames_per_anchor;
    p.sfpa = info->shadow_frames_per_anchor;
    p.no_shadows = info->no_shadows ? 1 : 0;
    p.linear = info->mode == ISTI_MODE_BACKWARD_BIDIRECTIONAL ? 1 : 0;

    // The array keeps the previous call's contents: every key starts as the
    // reference's empty value (all bytes 0xfe); the flow fields are fully
    // rewritten by the splat kernel before the reprojection reads them.
    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    e = cudaMemsetAsync(base, 0xfe, key_bytes, stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemsetAsync");
    const dim3 blk(32, 8);
    const dim3 gs((max_w + 31) / 32, (max_h + 7) / 8, n_views);
    isti::splat_kernel<<<gs, blk, 0, stream>>>(p);
    const dim3 gr((info->width + 31) / 32, (info->height + 7) / 8);
    switch (info->mode)
    {
    case ISTI_MODE_OURS:
    case ISTI_MODE_BACKWARD_UNIDIRECTIONAL:
        isti::reproj_kernel<1, 3, false><<<gr, blk, 0, stream>>>(p);
        break;
    case ISTI_MODE_SPLATTING:
        isti::reproj_kernel<1, 0, false><<<gr, blk, 0, stream>>>(p);
        break;
    case ISTI_MODE_BACKWARD_BIDIRECTIONAL:
        isti::reproj_kernel<3, 5, true><<<gr, blk, 0, stream>>>(p);
        break;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    return ISTI_OK;
}
