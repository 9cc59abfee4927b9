// Host side of the GB300 interpolation path and the C ABI of include/isti.h.
// Device code: isti_kernels.cuh.  Reference: src/renderer.cu
// (DerThomy/ImageBasedSpatioTemporalInterpolation).
//
// Layout in HBM (renderer-owned arena, one allocation):
//   [splat keys, u64/px: frame-major, every view][cam flow f32x4/px: frame-major, every view]
//   [full flow f32x4/px, every view][pixel->clip tables, (w + h) f32 per view][status word]
// Pixel inputs are caller-owned device images (include/isti.h).
//
// Launches per batch: init, splat, reprojection (isti_kernels.cuh); nothing
// blocks the host.
#include "isti.h"
#include "isti_dataset.h"
#include "isti_arith.h"
#include "isti_kernels.cuh"
#include "isti_launch.cuh"
#include "isti_learned.cuh"
#include "isti_batch.cuh"
#include "isti_unet.h"
#include "isti_train.h"
#include "host/isti_error.hpp"

#include <algorithm>

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

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
    // autotuning of the reprojection launch: one entry per tuned shape class
    bool autotune = false;
    std::vector<isti_tuning> tuned;
    isti::ReprojChoice pinned{}; // isti_renderer_set_reproj_launch (zero fields: the rule's)
    // arithmetic of the kernels (isti_renderer_set_arithmetic)
    int32_t arith = ISTI_ARITH_IEEE;
    // learned render path: its own arena (keys for the fallback tiles, keyframe parts,
    // network input and output, tile flags) and the parameters of its last call
    void *learned_arena = nullptr;
    size_t learned_bytes = 0;
    isti::LearnedParams learned{};
    bool has_learned = false;
    // failure-detection test hook (isti_renderer_test_withhold_tile)
    int32_t withhold_x = -1, withhold_y = -1;
    uint32_t wait_limit = 0;
    // isti_render_pairs: device arena (every pair's intermediates, then the parameter block),
    // pinned staging of the parameter block and the event of its last copy
    void *multi_arena = nullptr;
    size_t multi_bytes = 0;
    int32_t pair_splat_rows = 0, pair_init_kib = 0; // isti_render_pairs unit sizes (0: the defaults)
    int32_t stall_pair = -1;                         // test hook (isti_renderer_test_stall_pair)
    uint32_t stall_spin_limit = 0;
    void *multi_host[2] = {nullptr, nullptr}; // parameter staging: uncaptured calls, captured calls
    size_t multi_host_bytes[2] = {0, 0};
    cudaEvent_t multi_copied = nullptr;
    bool multi_recorded = false; // multi_copied was last recorded outside a stream capture
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

// [keys: frame, view][client flow (x, y): frame, view][client-flow depth: frame, view]
// [keyframe flow: view][visibility: view][pixel->clip tables: view][status word]
struct Layout
{
    size_t key_frame_bytes, cam_frame_bytes, depth_frame_bytes; // one frame, every view
    size_t key_bytes, cam_bytes, depth_bytes, ff_bytes, vis_bytes, lut_bytes, total;
};

constexpr size_t STATUS_BYTES = 256;

Layout layout_of(const isti_view *const *views, int n_views, int n_frames)
{
    Layout l{};
    for (int k = 0; k < n_views; k++)
    {
        const size_t px = (size_t)views[k]->width * views[k]->height;
        l.key_frame_bytes += align_up(px * 8, 256);
        l.cam_frame_bytes += align_up(px * 8, 256);
        l.depth_frame_bytes += align_up(px * 4, 256);
        l.ff_bytes += align_up(px * 16, 256);
        l.vis_bytes += align_up(px, 256);
        l.lut_bytes += align_up((size_t)(views[k]->width + views[k]->height) * 4, 256);
    }
    l.key_bytes = l.key_frame_bytes * n_frames;
    l.cam_bytes = l.cam_frame_bytes * n_frames;
    l.depth_bytes = l.depth_frame_bytes * n_frames;
    l.total = l.key_bytes + l.cam_bytes + l.depth_bytes + l.ff_bytes + l.vis_bytes + l.lut_bytes + STATUS_BYTES;
    return l;
}

// Timewarp (mode 4) needs no splat intermediates: [row sums, double per row of the
// forward keyframe][mean z][status word].
Layout timewarp_layout(const isti_view *const *views)
{
    Layout l{};
    l.total = align_up((size_t)views[0]->height * sizeof(double), 256) + 256 + STATUS_BYTES;
    return l;
}

Layout layout_for(int mode, const isti_view *const *views, int n_views, int n_frames)
{
    return mode == ISTI_MODE_TIMEWARP ? timewarp_layout(views) : layout_of(views, n_views, n_frames);
}

// Fills the kernel parameters for one batch whose intermediates live at `base`.
void fill_params(isti::FrameParams &p, int n_frames, void *const *outs, const isti_render_info *infos, const isti_frame_data *frame,
                 const isti_view *const *views, int n_views, const Layout &l, char *base, bool chain)
{
    std::memset(&p, 0, sizeof p);
    p.withhold_block = -1;
    p.withhold_x = p.withhold_y = -1;
    const isti_render_info &info = infos[0];
    size_t off_key = 0, off_cam = l.key_bytes, off_dep = off_cam + l.cam_bytes, off_full = off_dep + l.depth_bytes;
    size_t off_vis = off_full + l.ff_bytes, off_lut = off_vis + l.vis_bytes;
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
        std::memcpy(d.vp_self, v.viewproj, sizeof d.vp_self);
        const size_t px = (size_t)v.width * v.height;
        d.splat = reinterpret_cast<unsigned long long *>(base + off_key);
        d.cam_xy = l.cam_bytes ? reinterpret_cast<float2 *>(base + off_cam) : nullptr;
        d.cam_depth = l.depth_bytes ? reinterpret_cast<float *>(base + off_dep) : nullptr;
        d.vis = l.vis_bytes ? reinterpret_cast<uint8_t *>(base + off_vis) : nullptr;
        d.full_ff = reinterpret_cast<float4 *>(base + off_full);
        d.lut = reinterpret_cast<float *>(base + off_lut);
        off_key += align_up(px * 8, 256);
        off_cam += align_up(px * 8, 256);
        off_dep += align_up(px * 4, 256);
        off_full += align_up(px * 16, 256);
        off_vis += align_up(px, 256);
        off_lut += align_up((size_t)(v.width + v.height) * 4, 256);
    }
    for (int k = 0; k < n_frames; k++)
    {
        std::memcpy(p.cam_vp[k], infos[k].viewproj, sizeof p.cam_vp[k]);
        std::memcpy(p.cam_ivp[k], infos[k].inv_viewproj, sizeof p.cam_ivp[k]);
        p.out[k] = static_cast<uint32_t *>(outs[k]);
        p.f[k].alpha = infos[k].alpha;
        p.f[k].fpa = infos[k].frames_per_anchor;
        p.f[k].sfpa = infos[k].shadow_frames_per_anchor;
        p.f[k].no_shadows = infos[k].no_shadows ? 1 : 0;
    }
    p.key_stride = l.key_frame_bytes / sizeof(unsigned long long);
    p.cam_stride = l.cam_frame_bytes / sizeof(float2);
    p.depth_stride = l.depth_frame_bytes / sizeof(float);
    p.keys = reinterpret_cast<ulonglong2 *>(base);
    p.key_units = l.key_bytes / sizeof(ulonglong2);
    p.status = reinterpret_cast<int32_t *>(base + l.total - STATUS_BYTES);
    p.out_w = info.width;
    p.out_h = info.height;
    p.n_views = n_views;
    p.n_aux = frame->num_aux;
    p.n_frames = n_frames;
    p.linear = info.mode == ISTI_MODE_BACKWARD_BIDIRECTIONAL ? 1 : 0;
    p.chain = chain ? 1 : 0;
}

bool has_shadows(const isti::FrameParams &p)
{
    for (int k = 0; k < p.n_views; k++)
        if (p.v[k].shi != nullptr)
            return true;
    return false;
}

isti_tuning *find_tuning(isti_renderer *r, int mode, const isti::FrameParams &p)
{
    const int32_t sh = has_shadows(p) ? 1 : 0;
    for (isti_tuning &t : r->tuned)
        if (t.mode == mode && t.n_views == p.n_views && t.n_frames == p.n_frames && t.shadows == sh && t.width == p.out_w &&
            t.height == p.out_h)
            return &t;
    return nullptr;
}

// Times every candidate launch of the reprojection of the batch just enqueued (same inputs,
// same outputs: each run rewrites them identically) and records the fastest for its shape
// class.  One untimed launch per candidate first (module loading), then REPEAT timed ones.
cudaError_t launch_reproj_arith(isti_renderer *r, isti::FrameParams &p, int mode, cudaStream_t stream, isti::ReprojChoice c)
{
    if (r->arith == ISTI_ARITH_REFERENCE_GPU)
        return isti_fm_launch_reproj_mode(&p, mode, stream, c.regs, c.row_pairs, c.plain_tiles);
    return isti::launch_reproj_mode(p, mode, stream, c);
}

isti_status tune_reproj(isti_renderer *r, int mode, cudaStream_t stream)
{
    constexpr int REPEAT = 3;
    isti::FrameParams &p = r->last;
    std::vector<isti::ReprojChoice> cands;
    // chained outputs of several frames allow at most one block row per view (the launch limits them)
    const int max_pairs = p.chain && p.n_frames > 1 ? std::max(1, std::min(3, p.n_views / isti::ROWS)) : 3;
    for (int plain = 0; plain <= 1; plain++) // key tiles by TMA (where the views allow it), or by plain loads
        for (int regs : isti::mode_regs(mode))
            for (int np = 1; np <= max_pairs; np++)
                cands.push_back({regs, np, plain});
    const isti::ReprojChoice rule = isti::rule_choice(isti::mode_window(mode), p);
    std::vector<cudaEvent_t> ev(2 * cands.size(), nullptr);
    cudaError_t e = cudaSuccess;
    for (cudaEvent_t &x : ev)
        if (e == cudaSuccess)
            e = cudaEventCreate(&x);
    for (size_t i = 0; i < cands.size() && e == cudaSuccess; i++)
    {
        e = launch_reproj_arith(r, p, mode, stream, cands[i]);
        if (e == cudaSuccess)
            e = cudaEventRecord(ev[2 * i], stream);
        for (int k = 0; k < REPEAT && e == cudaSuccess; k++)
            e = launch_reproj_arith(r, p, mode, stream, cands[i]);
        if (e == cudaSuccess)
            e = cudaEventRecord(ev[2 * i + 1], stream);
    }
    // leave the renderer's parameters as its chosen launch sets them
    if (e == cudaSuccess)
        e = cudaEventSynchronize(ev.back());
    float best_ms = 0.0f, rule_ms = 0.0f;
    size_t best = 0;
    for (size_t i = 0; i < cands.size() && e == cudaSuccess; i++)
    {
        float ms = 0.0f;
        e = cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
        ms /= REPEAT;
        if (i == 0 || ms < best_ms)
        {
            best_ms = ms;
            best = i;
        }
        if (cands[i].regs == rule.regs && cands[i].row_pairs == rule.row_pairs && cands[i].plain_tiles == rule.plain_tiles)
            rule_ms = ms;
    }
    for (cudaEvent_t x : ev)
        if (x)
            cudaEventDestroy(x);
    if (e != cudaSuccess)
        return cuda_fail(e, "autotuning the reprojection");
    isti_tuning t{};
    t.mode = mode;
    t.n_views = p.n_views;
    t.n_frames = p.n_frames;
    t.shadows = has_shadows(p) ? 1 : 0;
    t.width = p.out_w;
    t.height = p.out_h;
    t.regs = cands[best].regs;
    t.row_pairs = cands[best].row_pairs;
    t.plain_tiles = cands[best].plain_tiles;
    t.best_ms = best_ms;
    t.rule_ms = rule_ms;
    r->tuned.push_back(t);
    return ISTI_OK;
}

isti_status render_batch(isti_renderer *r, int n_frames, void *const *outs, const isti_render_info *infos, const isti_frame_data *frame,
                         bool chain, cudaStream_t stream)
{
    const isti_view *views[isti::MAX_VIEWS];
    int n_views = 0;
    isti_status st = validate(n_frames, outs, infos, frame, views, n_views);
    if (st != ISTI_OK)
        return st;
    const bool timewarp = infos[0].mode == ISTI_MODE_TIMEWARP;
    const Layout l = layout_for(infos[0].mode, views, n_views, n_frames);

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
    r->last.withhold_x = r->withhold_x;
    r->last.withhold_y = r->withhold_y;
    r->last.wait_limit = r->wait_limit;

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
    isti::ReprojChoice choice{};
    const bool pinned = r->pinned.regs || r->pinned.row_pairs || r->pinned.plain_tiles;
    const isti_tuning *tuned = timewarp || pinned ? nullptr : find_tuning(r, infos[0].mode, r->last);
    if (pinned)
        choice = r->pinned;
    else if (tuned)
        choice = {tuned->regs, tuned->row_pairs, tuned->plain_tiles};
    cudaEvent_t ev1 = ev ? ev[1] : nullptr, ev2 = ev ? ev[2] : nullptr;
    if (r->arith == ISTI_ARITH_REFERENCE_GPU)
        e = timewarp ? isti_fm_launch_timewarp(&r->last, base, stream, ev1, ev2)
                     : isti_fm_launch_batch(&r->last, infos[0].mode, stream, ev1, ev2, choice.regs, choice.row_pairs, choice.plain_tiles);
    else
        e = timewarp ? isti::launch_timewarp(r->last, base, stream, ev1, ev2)
                     : isti::launch_batch(r->last, infos[0].mode, stream, ev1, ev2, choice);
    if (ev)
        cudaEventRecord(ev[3], stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    r->has_frame = true;
    if (r->autotune && !timewarp && !tuned && !pinned)
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        e = cudaStreamIsCapturing(stream, &cs);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaStreamIsCapturing");
        if (cs == cudaStreamCaptureStatusNone) // no tuning inside a capture: the class keeps the rule until an uncaptured call
            return tune_reproj(r, infos[0].mode, stream);
    }
    return ISTI_OK;
}
} // namespace

isti_status isti::set_error(isti_status s, const std::string &msg) { return fail(s, msg); }

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
    if (r->learned_arena)
        cudaFree(r->learned_arena);
    if (r->multi_arena)
        cudaFree(r->multi_arena);
    for (void *h : r->multi_host)
        if (h)
            cudaFreeHost(h);
    if (r->multi_copied)
        cudaEventDestroy(r->multi_copied);
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

isti_status isti_renderer_device_status(isti_renderer *r, int32_t *device_status)
{
    if (!r || !device_status)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    *device_status = ISTI_OK;
    if (!r->has_frame)
        return ISTI_OK;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaDeviceSynchronize");
    e = cudaMemcpy(device_status, r->last.status, sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy");
    return ISTI_OK;
}

isti_status isti_renderer_set_arithmetic(isti_renderer *r, int32_t arith)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "renderer is NULL");
    if (arith != ISTI_ARITH_IEEE && arith != ISTI_ARITH_REFERENCE_GPU)
        return fail(ISTI_ERR_INVALID_ARG, "unknown arithmetic mode");
    if (arith == ISTI_ARITH_REFERENCE_GPU && isti_fm_params_size() != sizeof(isti::FrameParams))
        return fail(ISTI_ERR_UNSUPPORTED, "kernel parameter layouts of the two arithmetic modes differ");
    if (arith != r->arith)
        r->tuned.clear(); // launch timings belong to one set of kernels
    r->arith = arith;
    return ISTI_OK;
}

isti_status isti_renderer_test_withhold_tile(isti_renderer *r, int32_t x, int32_t y, uint32_t wait_limit)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "renderer is NULL");
    r->withhold_x = x;
    r->withhold_y = y;
    r->wait_limit = wait_limit;
    return ISTI_OK;
}

isti_status isti_renderer_test_stall_pair(isti_renderer *r, int32_t pair, uint32_t spin_limit)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "renderer is NULL");
    r->stall_pair = pair;
    r->stall_spin_limit = spin_limit;
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
        out->frames += r->event_frames[i / 4];
    }
    out->kernel_launches = r->timed_launches;
    r->events_used = 0;
    r->timed_launches = 0;
    return ISTI_OK;
}

isti_status isti_renderer_set_autotune(isti_renderer *r, int32_t on)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "renderer is NULL");
    r->autotune = on != 0;
    return ISTI_OK;
}

isti_status isti_renderer_set_reproj_launch(isti_renderer *r, int32_t regs, int32_t row_pairs, int32_t plain_tiles)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "null renderer");
    if ((regs != 0 && regs != isti::REPROJ_REGS_MANY_VIEWS && regs != isti::REPROJ_REGS && regs != isti::REPROJ_REGS_WIDE_WINDOW) ||
        row_pairs < 0 || row_pairs > 3 || (plain_tiles != 0 && plain_tiles != 1))
        return fail(ISTI_ERR_INVALID_ARG, "register cap must be 0, 40, 48 or 56, row pairs 0..3 and plain_tiles 0 or 1");
    r->pinned = isti::ReprojChoice{regs, row_pairs, plain_tiles};
    return ISTI_OK;
}

isti_status isti_renderer_tuning_count(const isti_renderer *r, int32_t *count)
{
    if (!r || !count)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    *count = (int32_t)r->tuned.size();
    return ISTI_OK;
}

isti_status isti_renderer_tuning(const isti_renderer *r, int32_t index, isti_tuning *out)
{
    if (!r || !out)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    if (index < 0 || (size_t)index >= r->tuned.size())
        return fail(ISTI_ERR_INVALID_ARG, "no tuned shape class with this index");
    *out = r->tuned[(size_t)index];
    return ISTI_OK;
}

isti_status isti_renderer_view_buffers(const isti_renderer *r, int32_t view, const uint64_t **splat, const float **cam_xy,
                                       const float **full_ff, uint32_t *width, uint32_t *height)
{
    if (!r || !r->has_frame)
        return fail(ISTI_ERR_INVALID_ARG, "no frame rendered yet");
    const int nv = r->last.n_views;
    if (view < 0 || view >= nv * r->last.n_frames)
        return fail(ISTI_ERR_INVALID_ARG, "view index out of range");
    const int k = view / nv;
    const isti::DevView &d = r->last.v[view % nv];
    const bool materialised = r->last.tw_mean == nullptr; // timewarp keeps no splat intermediates
    if (splat)
        *splat = materialised ? reinterpret_cast<const uint64_t *>(d.splat + k * r->last.key_stride) : nullptr;
    if (cam_xy)
        *cam_xy = materialised && d.cam_xy ? reinterpret_cast<const float *>(d.cam_xy + k * r->last.cam_stride) : nullptr;
    if (full_ff)
        *full_ff = materialised ? reinterpret_cast<const float *>(d.full_ff) : nullptr;
    if (width)
        *width = d.w;
    if (height)
        *height = d.h;
    return ISTI_OK;
}

isti_status isti_renderer_view_depth(const isti_renderer *r, int32_t view, const float **cam_depth, const uint8_t **visible)
{
    if (!r || !r->has_frame)
        return fail(ISTI_ERR_INVALID_ARG, "no frame rendered yet");
    const int nv = r->last.n_views;
    if (view < 0 || view >= nv * r->last.n_frames)
        return fail(ISTI_ERR_INVALID_ARG, "view index out of range");
    const int k = view / nv;
    const isti::DevView &d = r->last.v[view % nv];
    const bool materialised = r->last.tw_mean == nullptr;
    if (cam_depth)
        *cam_depth = materialised && d.cam_depth ? d.cam_depth + k * r->last.depth_stride : nullptr;
    if (visible)
        *visible = materialised ? d.vis : nullptr;
    return ISTI_OK;
}

} // extern "C"

// ============================ many keyframe pairs, one persistent launch ============================

namespace
{
template <int SW, int SI, bool MAV, int REGS>
cudaError_t launch_pairs_kernel(const isti::BatchParams &bp, size_t smem, unsigned threads_y, cudaStream_t stream)
{
    auto kernel = isti::batch_kernel<SW, SI, MAV, REGS>;
    static std::mutex mu;
    static size_t set_bytes[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (smem > 48 * 1024)
    {
        std::lock_guard<std::mutex> lock(mu);
        if (smem > set_bytes[dev & 63])
        {
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess)
                return e;
            set_bytes[dev & 63] = smem;
        }
    }
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)(32 * threads_y), smem);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(per_sm * sms));
    cfg.blockDim = dim3(32, threads_y);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative; // every CTA resident: the units' waits always end
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, bp);
}

cudaError_t launch_pairs_mode(int mode, int regs, const isti::BatchParams &bp, size_t smem, unsigned threads_y, cudaStream_t stream)
{
    switch (mode)
    {
    case ISTI_MODE_OURS:
    case ISTI_MODE_BACKWARD_UNIDIRECTIONAL:
        return regs == isti::REPROJ_REGS_MANY_VIEWS ? launch_pairs_kernel<1, 3, false, isti::REPROJ_REGS_MANY_VIEWS>(bp, smem, threads_y, stream)
                                                    : launch_pairs_kernel<1, 3, false, isti::REPROJ_REGS>(bp, smem, threads_y, stream);
    case ISTI_MODE_SPLATTING:
        return regs == isti::REPROJ_REGS_MANY_VIEWS ? launch_pairs_kernel<1, 0, false, isti::REPROJ_REGS_MANY_VIEWS>(bp, smem, threads_y, stream)
                                                    : launch_pairs_kernel<1, 0, false, isti::REPROJ_REGS>(bp, smem, threads_y, stream);
    case ISTI_MODE_BACKWARD_BIDIRECTIONAL:
        return launch_pairs_kernel<3, 5, true, isti::REPROJ_REGS_WIDE_WINDOW>(bp, smem, threads_y, stream);
    }
    return cudaErrorInvalidValue;
}

template <int SW>
bool pair_maps(const isti::FrameParams &p, isti::KeyMaps &km)
{
    return isti::make_key_maps<SW>(p, km);
}
} // namespace

extern "C" isti_status isti_renderer_set_pair_units(isti_renderer *r, int32_t splat_rows, int32_t init_unit_kib)
{
    if (!r)
        return fail(ISTI_ERR_INVALID_ARG, "null renderer");
    if (splat_rows < 0 || splat_rows > 256 || init_unit_kib < 0 || init_unit_kib > 4096 || (init_unit_kib && init_unit_kib < 16))
        return fail(ISTI_ERR_INVALID_ARG, "splat rows must be 0..256 and the init unit 0 or 16..4096 KiB");
    r->pair_splat_rows = splat_rows;
    r->pair_init_kib = init_unit_kib;
    return ISTI_OK;
}

extern "C" isti_status isti_render_pairs(isti_renderer *r, int32_t n_pairs, const isti_pair_frames *pairs, void *stream_ptr)
{
    if (!r || !pairs)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    if (n_pairs < 1 || n_pairs > ISTI_MAX_PAIRS)
        return fail(ISTI_ERR_INVALID_ARG, "n_pairs must be 1..ISTI_MAX_PAIRS");
    if (r->arith != ISTI_ARITH_IEEE)
        return fail(ISTI_ERR_UNSUPPORTED, "isti_render_pairs runs the IEEE kernels");
    const cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (cur != r->device)
        return fail(ISTI_ERR_INVALID_ARG, "renderer was created on another device");
    // validation and the arena layout: every pair's intermediates, then the parameter block
    std::vector<Layout> layouts(n_pairs);
    std::vector<std::vector<const isti_view *>> views(n_pairs);
    int mode = -1, nv = 0;
    size_t data_bytes = 0;
    for (int i = 0; i < n_pairs; i++)
    {
        const isti_pair_frames &pf = pairs[i];
        if (!pf.frame || !pf.out_rgba || !pf.infos)
            return fail(ISTI_ERR_INVALID_ARG, "NULL pair argument");
        const isti_view *vv[isti::MAX_VIEWS];
        int n_views = 0;
        isti_status st = validate(pf.n_frames, pf.out_rgba, pf.infos, pf.frame, vv, n_views);
        if (st != ISTI_OK)
            return st;
        if (i == 0)
        {
            mode = pf.infos[0].mode;
            nv = n_views;
        }
        if (pf.infos[0].mode != mode || n_views != nv)
            return fail(ISTI_ERR_INVALID_ARG, "all pairs of isti_render_pairs need the same mode and number of views");
        if (mode == ISTI_MODE_TIMEWARP)
            return fail(ISTI_ERR_UNSUPPORTED, "isti_render_pairs does not render timewarp frames");
        views[i].assign(vv, vv + n_views);
        layouts[i] = layout_of(vv, n_views, pf.n_frames);
        data_bytes += align_up(layouts[i].total, 256);
    }
    const size_t fp_bytes = align_up(sizeof(isti::FrameParams) * n_pairs, 256);
    const size_t map_bytes = align_up(sizeof(CUtensorMap) * isti::MAX_VIEWS * n_pairs, 256);
    const size_t pair_bytes = align_up(sizeof(isti::BatchPair) * n_pairs, 256);
    const size_t seg_bytes = align_up(sizeof(isti::BatchSeg) * 3 * n_pairs, 256);
    const size_t cnt_bytes = align_up(sizeof(uint32_t) * (2 + 2 * n_pairs), 256);
    const size_t block_bytes = fp_bytes + map_bytes + pair_bytes + seg_bytes + cnt_bytes;
    const size_t total = data_bytes + block_bytes;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(stream, &cs)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamIsCapturing");
    if (total > r->multi_bytes && cs != cudaStreamCaptureStatusNone)
        return fail(ISTI_ERR_INVALID_ARG, "isti_render_pairs: make one call of this size outside a stream capture first");
    if (total > r->multi_bytes)
    {
        if (r->multi_arena)
            cudaFree(r->multi_arena);
        r->multi_arena = nullptr;
        r->multi_bytes = 0;
        e = cudaMalloc(&r->multi_arena, total);
        if (e != cudaSuccess)
            return e == cudaErrorMemoryAllocation ? fail(ISTI_ERR_OOM, "cudaMalloc of the multi-pair arena failed") : cuda_fail(e, "cudaMalloc");
        r->multi_bytes = total;
    }
    if (!r->multi_copied && (e = cudaEventCreateWithFlags(&r->multi_copied, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(e, "cudaEventCreate");
    // Two pinned staging buffers: uncaptured calls reuse theirs once the previous uncaptured
    // call's copy is done; a captured call's copy reads its buffer whenever the graph runs, so
    // captured calls have their own, sized by the uncaptured calls (no allocation in a capture)
    // and overwritten only by the next captured call.
    if (cs == cudaStreamCaptureStatusNone)
    {
        if (r->multi_recorded && (e = cudaEventSynchronize(r->multi_copied)) != cudaSuccess)
            return cuda_fail(e, "waiting for the previous parameter copy");
        for (int i = 0; i < 2; i++)
            if (block_bytes > r->multi_host_bytes[i])
            {
                if (r->multi_host[i])
                    cudaFreeHost(r->multi_host[i]);
                r->multi_host[i] = nullptr;
                r->multi_host_bytes[i] = 0;
                if ((e = cudaHostAlloc(&r->multi_host[i], block_bytes, cudaHostAllocDefault)) != cudaSuccess)
                    return cuda_fail(e, "cudaHostAlloc of the parameter staging");
                r->multi_host_bytes[i] = block_bytes;
            }
    }
    else if (block_bytes > r->multi_host_bytes[1])
        return fail(ISTI_ERR_INVALID_ARG, "isti_render_pairs: make one call of this size outside a stream capture first");
    char *dbase = static_cast<char *>(r->multi_arena);
    char *dblock = dbase + data_bytes;
    char *h = static_cast<char *>(r->multi_host[cs == cudaStreamCaptureStatusNone ? 0 : 1]);
    std::memset(h, 0, block_bytes);
    auto *hfp = reinterpret_cast<isti::FrameParams *>(h);
    auto *hmaps = reinterpret_cast<CUtensorMap *>(h + fp_bytes);
    auto *hpairs = reinterpret_cast<isti::BatchPair *>(h + fp_bytes + map_bytes);
    auto *hsegs = reinterpret_cast<isti::BatchSeg *>(h + fp_bytes + map_bytes + pair_bytes);
    const auto *dfp = reinterpret_cast<const isti::FrameParams *>(dblock);
    const auto *dmaps = reinterpret_cast<const CUtensorMap *>(dblock + fp_bytes);
    auto *dcnt = reinterpret_cast<uint32_t *>(dblock + fp_bytes + map_bytes + pair_bytes + seg_bytes);
    int32_t *dstatus = reinterpret_cast<int32_t *>(dcnt + 1 + 2 * n_pairs);
    const uint32_t splat_rows = r->pair_splat_rows ? (uint32_t)r->pair_splat_rows : isti::BATCH_SPLAT_ROWS;
    const uint32_t init_keys = r->pair_init_kib ? (uint32_t)r->pair_init_kib * 64u : isti::BATCH_INIT_UNIT_KEYS; // 16-byte units
    const int sw = isti::mode_window(mode);
    // one register cap for every unit of the launch: by window size and view count (the
    // per-batch rule's occupancy test depends on a batch's frames, which differ from pair to pair)
    const int regs = sw != 1 ? isti::REPROJ_REGS_WIDE_WINDOW : (nv >= isti::REPROJ_MANY_VIEWS ? isti::REPROJ_REGS_MANY_VIEWS : isti::REPROJ_REGS);
    const unsigned nthreads = 32u * (unsigned)nv;
    size_t region = 0, off = 0;
    for (int i = 0; i < n_pairs; i++)
    {
        const isti_pair_frames &pf = pairs[i];
        isti::FrameParams &p = hfp[i];
        fill_params(p, pf.n_frames, pf.out_rgba, pf.infos, pf.frame, views[i].data(), nv, layouts[i], dbase + off, pf.chain_outputs != 0);
        off += align_up(layouts[i].total, 256);
        p.status = dstatus;
        p.row_pairs = isti::rule_row_pairs(nv, pf.n_frames);
        isti::KeyMaps km;
        p.use_tma = (sw == 1 ? pair_maps<1>(p, km) : pair_maps<3>(p, km)) ? 1 : 0;
        std::memcpy(hmaps + (size_t)i * isti::MAX_VIEWS, km.m, sizeof(CUtensorMap) * nv);
        const int nu = pf.n_frames * p.row_pairs;
        const size_t reg = (sw == 1 ? isti::reproj_tile_region<1>(nv, nu) : isti::reproj_tile_region<3>(nv, nu)) +
                           (size_t)nu * isti::ROWS * nv * 32 * sizeof(isti::DirRes);
        region = std::max(region, align_up(reg, 16));
        uint32_t max_w = 0, max_h = 0;
        for (int k = 0; k < nv; k++)
        {
            max_w = std::max(max_w, p.v[k].w);
            max_h = std::max(max_h, p.v[k].h);
        }
        isti::BatchPair &bpair = hpairs[i];
        bpair.fp = dfp + i;
        bpair.maps = dmaps + (size_t)i * isti::MAX_VIEWS;
        const size_t lut_need = (std::max(max_w, max_h) + nthreads - 1) / nthreads;
        bpair.init_units = (uint32_t)std::max<size_t>((p.key_units + init_keys - 1) / init_keys, lut_need);
        bpair.splat_gx = (max_w + 31) / 32;
        bpair.splat_gy = (max_h + splat_rows - 1) / splat_rows;
        bpair.splat_units = (uint32_t)nv * bpair.splat_gx * bpair.splat_gy;
        bpair.splat_need = bpair.splat_units + (i == r->stall_pair ? 1u : 0u); // the test hook: one unit more than there are
        bpair.reproj_gx = (p.out_w + 31) / 32;
        const uint32_t block_rows = (uint32_t)(isti::ROWS * p.row_pairs);
        bpair.reproj_units = bpair.reproj_gx * ((p.out_h + block_rows - 1) / block_rows);
    }
    // the queue: I0 S0 I1 S1 R0 I2 S2 R1 ... R(n-1)
    int ns = 0;
    uint32_t first = 0;
    auto seg = [&](int pair, int phase) {
        const isti::BatchPair &bpair = hpairs[pair];
        hsegs[ns++] = isti::BatchSeg{(uint32_t)pair, (uint32_t)phase, first};
        first += phase == 0 ? bpair.init_units : (phase == 1 ? bpair.splat_units : bpair.reproj_units);
    };
    for (int i = 0; i < n_pairs; i++)
    {
        seg(i, 0);
        seg(i, 1);
        if (i > 0)
            seg(i - 1, 2);
    }
    seg(n_pairs - 1, 2);
    isti::BatchParams bp{};
    bp.pairs = reinterpret_cast<const isti::BatchPair *>(dblock + fp_bytes + map_bytes);
    bp.segs = reinterpret_cast<const isti::BatchSeg *>(dblock + fp_bytes + map_bytes + pair_bytes);
    bp.n_segs = ns;
    bp.total = first;
    bp.ticket = dcnt;
    bp.done = dcnt + 1;
    bp.status = dstatus;
    bp.spin_limit = r->stall_pair >= 0 && r->stall_spin_limit ? r->stall_spin_limit : 1u << 24; // with 128 ns sleeps: about two seconds
    bp.region_bytes = (uint32_t)region;
    bp.param_bytes = (uint32_t)isti::params_prefix(nv);
    bp.splat_rows = splat_rows;
    const size_t smem = isti::batch_param_space(bp.param_bytes) + region + isti::BATCH_CTRL_BYTES;
    // counters to zero (in the staged block), then the block to the device, then the launch
    e = cudaMemcpyAsync(dblock, h, block_bytes, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
    {
        r->multi_recorded = cs == cudaStreamCaptureStatusNone;
        if (r->multi_recorded)
            e = cudaEventRecord(r->multi_copied, stream);
    }
    if (e == cudaSuccess)
        e = launch_pairs_mode(mode, regs, bp, smem, (unsigned)nv, stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "isti_render_pairs launch");
    r->last = hfp[0];
    r->has_frame = true;
    return ISTI_OK;
}

// ============================ learned initialisation ============================

namespace
{
constexpr int LEARNED_MAX_FRAMES = ISTI_MAX_BATCH_FRAMES;

int quarter_grid(uint32_t n) { return (int)(((n + 3) / 4 + 7) / 8 * 8); }
} // namespace

// Lays out the learned arena for a call and fills r->learned (everything but the stages).
isti_status learned_setup(isti_renderer *r, isti_flownet *net, int32_t n_frames, void *const *out_rgba, const isti_render_info *infos,
                          const isti_frame_data *frame, int32_t iterations, bool chain, __half **guess_out);

extern "C" isti_status isti_render_learned(isti_renderer *r, isti_flownet *net, int32_t n_frames, void *const *out_rgba,
                                           const isti_render_info *infos, const isti_frame_data *frame, int32_t iterations,
                                           int32_t chain_outputs, void *stream_ptr)
{
    __half *guess = nullptr;
    isti_status st = learned_setup(r, net, n_frames, out_rgba, infos, frame, iterations, chain_outputs != 0, &guess);
    if (st != ISTI_OK)
        return st;
    const cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    isti::LearnedParams &p = r->learned;
    const uint32_t w = infos[0].width, h = infos[0].height;
    cudaError_t e = cudaMemsetAsync(p.fallback_count, 0, 4, stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(p.fp.status, 0, 4, stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(p.cell_bits, 0, (size_t)n_frames * p.cells_y * p.cell_words * 4, stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemsetAsync");
    const dim3 b2(32, 8);
    isti::keyframe_kernel<<<dim3((w + 31) / 32, (h + 7) / 8, 2), b2, 0, stream>>>(p);
    if (net)
    {
        isti::input_kernel<<<dim3((p.wq + 31) / 32, (p.hq + 7) / 8, n_frames), b2, 0, stream>>>(p);
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return cuda_fail(e, "learned input launch");
        st = isti_flownet_forward(net, p.net_in, n_frames, p.hq, p.wq, nullptr, guess, stream);
        if (st != ISTI_OK)
            return st;
    }
    isti::learned_kernel<<<dim3(p.tiles_x, p.tiles_y), dim3(isti::LT_W, isti::LT_H), 0, stream>>>(p);
    // the fallback kernels walk the list of marked tiles (none: they return at once)
    const unsigned list_blocks = (unsigned)std::min(p.tiles_x * p.tiles_y * n_frames, 152 * 4);
    isti::fallback_init_kernel<<<list_blocks, dim3(isti::LT_W, isti::LT_H), 0, stream>>>(p);
    isti::fallback_splat_kernel<<<dim3((w + 31) / 32, (h + 7) / 8, 2), b2, 0, stream>>>(p);
    isti::fallback_reproj_kernel<<<list_blocks, dim3(isti::LT_W, isti::LT_H), 0, stream>>>(p);
    if (chain_outputs && n_frames > 1)
        isti::learned_chain_kernel<<<(unsigned)std::min<size_t>(((size_t)w * h + 255) / 256, 152 * 8), 256, 0, stream>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(e, "learned render launch");
    r->has_learned = true;
    return ISTI_OK;
}

extern "C" isti_status isti_learned_input(isti_renderer *r, int32_t n_frames, const isti_render_info *infos, const isti_frame_data *frame,
                                          void *net_input, void *stream_ptr)
{
    if (!net_input || ((uintptr_t)net_input & 15u))
        return fail(ISTI_ERR_INVALID_ARG, "net_input must be a 16-byte aligned device buffer");
    // the outputs are not touched by the input stages: the render info's frames only need a
    // placeholder address each
    void *dummy[isti::MAX_FRAMES];
    for (int k = 0; k < isti::MAX_FRAMES; k++)
        dummy[k] = net_input;
    __half *guess = nullptr;
    isti_status st = learned_setup(r, nullptr, n_frames, dummy, infos, frame, 1, false, &guess);
    if (st != ISTI_OK)
        return st;
    const cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    isti::LearnedParams p = r->learned;
    p.net_in = static_cast<__nv_bfloat16 *>(net_input);
    const uint32_t w = infos[0].width, h = infos[0].height;
    const dim3 b2(32, 8);
    isti::keyframe_kernel<<<dim3((w + 31) / 32, (h + 7) / 8, 2), b2, 0, stream>>>(p);
    isti::input_kernel<<<dim3((p.wq + 31) / 32, (p.hq + 7) / 8, n_frames), b2, 0, stream>>>(p);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "learned input launch");
}

extern "C" isti_status isti_learned_labels(isti_renderer *r, int32_t frame_index, float *labels, void *stream_ptr)
{
    if (!r || !labels || ((uintptr_t)labels & 15u))
        return fail(ISTI_ERR_INVALID_ARG, "NULL or unaligned argument");
    if (!r->has_frame || r->last.tw_mean != nullptr || r->last.n_aux != 0 || r->last.linear)
        return fail(ISTI_ERR_INVALID_ARG, "labels need a preceding plain render (main camera only, modes 0/2/3)");
    if (frame_index < 0 || frame_index >= r->last.n_frames)
        return fail(ISTI_ERR_INVALID_ARG, "frame index out of range");
    const int hq = quarter_grid(r->last.out_h), wq = quarter_grid(r->last.out_w);
    isti::label_kernel<<<dim3((wq + 31) / 32, (hq + 7) / 8), dim3(32, 8), 0, static_cast<cudaStream_t>(stream_ptr)>>>(r->last, frame_index, hq,
                                                                                                                         wq, labels);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "label launch");
}

extern "C" isti_status isti_learned_grid(uint32_t width, uint32_t height, int32_t *grid_w, int32_t *grid_h)
{
    if (!grid_w || !grid_h)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    *grid_w = quarter_grid(width);
    *grid_h = quarter_grid(height);
    return ISTI_OK;
}

isti_status learned_setup(isti_renderer *r, isti_flownet *net, int32_t n_frames, void *const *out_rgba, const isti_render_info *infos,
                          const isti_frame_data *frame, int32_t iterations, bool chain, __half **guess_out)
{
    if (!r || !out_rgba || !infos || !frame)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    const isti_view *views[isti::MAX_VIEWS];
    int n_views = 0;
    const isti_status st = validate(n_frames, out_rgba, infos, frame, views, n_views);
    if (st != ISTI_OK)
        return st;
    if (frame->num_aux != 0)
        return fail(ISTI_ERR_INVALID_ARG, "isti_render_learned renders the main camera only (num_aux must be 0)");
    if (infos[0].mode != ISTI_MODE_OURS && infos[0].mode != ISTI_MODE_BACKWARD_UNIDIRECTIONAL)
        return fail(ISTI_ERR_INVALID_ARG, "isti_render_learned implements modes 0 and 2 (3x3 window, 3 search iterations)");
    if (iterations < -1 || iterations > 16)
        return fail(ISTI_ERR_INVALID_ARG, "iterations must be -1..16");
    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (cur != r->device)
        return fail(ISTI_ERR_INVALID_ARG, "renderer was created on another device");
    const uint32_t w = infos[0].width, h = infos[0].height;
    const size_t px = (size_t)w * h;
    const int hq = quarter_grid(h), wq = quarter_grid(w);
    const int tiles_x = (int)((w + isti::LT_W - 1) / isti::LT_W), tiles_y = (int)((h + isti::LT_H - 1) / isti::LT_H);
    // [keys: frames x 2 views][full flow: 2 views][lut: 2 views][status] (fill_params' layout, no cam flow)
    // then [ws: 2 views][dws: 2 views][network input][network output][tile flags][fallback count]
    Layout l{};
    for (int k = 0; k < 2; k++)
    {
        l.key_frame_bytes += align_up(px * 8, 256);
        l.lut_bytes += align_up((size_t)(w + h) * 4, 256);
    }
    l.ff_bytes = 2 * align_up(px * 16, 256);
    l.key_bytes = l.key_frame_bytes * n_frames;
    l.total = l.key_bytes + l.ff_bytes + l.lut_bytes + STATUS_BYTES;
    const size_t ws_bytes = align_up(px * 16, 256);
    const size_t in_bytes = align_up((size_t)n_frames * hq * wq * 16 * 2, 256);
    const size_t guess_bytes = align_up((size_t)n_frames * hq * wq * 4 * 2, 256);
    const size_t flag_bytes = 2 * align_up((size_t)n_frames * tiles_x * tiles_y * 4, 256); // flags, then the marked-tile list
    const size_t valid_bytes = align_up((size_t)n_frames * px, 256);
    const int cells_y = (int)((h + isti::FB_CELL - 1) / isti::FB_CELL);
    const int cell_words = (int)(((w + isti::FB_CELL - 1) / isti::FB_CELL + 31) / 32);
    const size_t cell_bytes = align_up((size_t)n_frames * cells_y * cell_words * 4, 256);
    const size_t total = l.total + 4 * ws_bytes + in_bytes + guess_bytes + flag_bytes + 256 + valid_bytes + cell_bytes;
    if (total > r->learned_bytes)
    {
        if (r->learned_arena)
            cudaFree(r->learned_arena);
        r->learned_arena = nullptr;
        r->learned_bytes = 0;
        e = cudaMalloc(&r->learned_arena, total);
        if (e != cudaSuccess)
            return e == cudaErrorMemoryAllocation ? fail(ISTI_ERR_OOM, "cudaMalloc of the learned-path arena failed") : cuda_fail(e, "cudaMalloc");
        r->learned_bytes = total;
    }
    char *base = static_cast<char *>(r->learned_arena);
    isti::LearnedParams &p = r->learned;
    fill_params(p.fp, n_frames, out_rgba, infos, frame, views, n_views, l, base, chain); // no client-flow buffers:
                                                                                            // computed on the fly
    char *extra = base + l.total;
    for (int v = 0; v < 2; v++)
    {
        p.ws[v] = reinterpret_cast<float4 *>(extra + v * ws_bytes);
        p.dws[v] = reinterpret_cast<float4 *>(extra + (2 + v) * ws_bytes);
    }
    p.net_in = reinterpret_cast<__nv_bfloat16 *>(extra + 4 * ws_bytes);
    __half *guess = reinterpret_cast<__half *>(extra + 4 * ws_bytes + in_bytes);
    p.guess = net ? guess : nullptr;
    p.tile_flags = reinterpret_cast<uint32_t *>(extra + 4 * ws_bytes + in_bytes + guess_bytes);
    p.tile_list = reinterpret_cast<uint32_t *>(extra + 4 * ws_bytes + in_bytes + guess_bytes + flag_bytes / 2);
    p.fallback_count = reinterpret_cast<int32_t *>(extra + 4 * ws_bytes + in_bytes + guess_bytes + flag_bytes);
    p.valid = reinterpret_cast<uint8_t *>(extra + 4 * ws_bytes + in_bytes + guess_bytes + flag_bytes + 256);
    p.cell_bits = reinterpret_cast<uint32_t *>(extra + 4 * ws_bytes + in_bytes + guess_bytes + flag_bytes + 256 + valid_bytes);
    p.cells_y = cells_y;
    p.cell_words = cell_words;
    p.hq = hq;
    p.wq = wq;
    p.learned_iters = iterations;
    p.tiles_x = tiles_x;
    p.tiles_y = tiles_y;
    *guess_out = guess;
    return ISTI_OK;
}

extern "C" isti_status isti_renderer_learned_stats(isti_renderer *r, int32_t *fallback_tiles, int32_t *tiles)
{
    if (!r || !fallback_tiles || !tiles)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    *fallback_tiles = 0;
    *tiles = 0;
    if (!r->has_learned)
        return ISTI_OK;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(fallback_tiles, r->learned.fallback_count, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(e, "reading the fallback count");
    *tiles = r->learned.tiles_x * r->learned.tiles_y * r->learned.fp.n_frames;
    return ISTI_OK;
}

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
// Its last 256 bytes hold the device status word of the no-allocation calls, at a fixed
// place whatever the frame's layout, so isti_noalloc_device_status can read it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[ISTI_NOALLOC_SCRATCH_BYTES];
constexpr size_t NOALLOC_STATUS_OFFSET = (size_t)ISTI_NOALLOC_SCRATCH_BYTES - 256;
static_assert(NOALLOC_STATUS_OFFSET % 256 == 0, "status word must stay aligned");

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device.  In host code the
// array's name only denotes a host-side shadow, so the address is looked up with the
// device current.  It is looked up again on every call made outside a stream capture
// (a reset device or a recreated context may place the module elsewhere); a call
// inside a capture uses the address of the last uncaptured call on that device.
isti_status noalloc_scratch(int device, cudaStream_t stream, char **out)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return fail(ISTI_ERR_UNSUPPORTED, "device ordinal beyond the no-allocation scratch table");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &cs);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaStreamIsCapturing");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (cs == cudaStreamCaptureStatusNone)
    {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[device] = p;
    }
    else if (!g_noalloc_ptr[device])
        return fail(ISTI_ERR_INVALID_ARG, "the first isti_render_noalloc call on a device must not be captured");
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
    const Layout l = layout_for(info->mode, views, n_views, 1);
    if (l.total > NOALLOC_STATUS_OFFSET)
        return fail(ISTI_ERR_INVALID_ARG, "frame needs " + std::to_string(l.total) + " bytes of scratch; isti_render_noalloc holds at most " +
                                              std::to_string(NOALLOC_STATUS_OFFSET) + " of its " +
                                              std::to_string((size_t)ISTI_NOALLOC_SCRATCH_BYTES) + " (use isti_render for larger frames)");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    const cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    char *base = nullptr;
    st = noalloc_scratch(device, stream, &base);
    if (st != ISTI_OK)
        return st;
    isti::FrameParams p;
    fill_params(p, 1, outs, info, frame, views, n_views, l, base, false);
    p.status = reinterpret_cast<int32_t *>(base + NOALLOC_STATUS_OFFSET);
    // The array keeps the previous call's contents: the init kernel (the timewarp's mean
    // kernel in mode 4) resets the status word, the init kernel every key to the
    // reference's empty value (all bytes 0xfe) and the tables; the flow fields are fully
    // rewritten by the splat kernel before the reprojection reads them.
    e = info->mode == ISTI_MODE_TIMEWARP ? isti::launch_timewarp(p, base, stream, nullptr, nullptr)
                                         : isti::launch_batch(p, info->mode, stream, nullptr, nullptr, isti::ReprojChoice{});
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    return ISTI_OK;
}

extern "C" isti_status isti_noalloc_device_status(int32_t *device_status)
{
    if (!device_status)
        return fail(ISTI_ERR_INVALID_ARG, "NULL argument");
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaDeviceSynchronize");
    e = cudaMemcpyFromSymbol(device_status, g_noalloc_scratch, sizeof(int32_t), NOALLOC_STATUS_OFFSET, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(e, "reading the no-allocation status word");
    return ISTI_OK;
}

// RGB8 upload format -> RGBA8, declared in include/isti_dataset.h.
extern "C" isti_status isti_rgb8_to_rgba8(void *dst_rgba, const void *src_rgb, size_t n_pixels, void *stream_ptr)
{
    if (n_pixels == 0)
        return ISTI_OK;
    if (!dst_rgba || !src_rgb || ((uintptr_t)dst_rgba & 3u))
        return fail(ISTI_ERR_INVALID_ARG, "isti_rgb8_to_rgba8: NULL or unaligned buffer");
    const uintptr_t d = (uintptr_t)dst_rgba, s = (uintptr_t)src_rgb;
    if (d < s + 3 * n_pixels && s < d + 4 * n_pixels)
        return fail(ISTI_ERR_INVALID_ARG, "isti_rgb8_to_rgba8: buffers overlap");
    const bool vec = (d & 15u) == 0 && (s & 3u) == 0;
    const size_t work = vec ? n_pixels / 4 + 3 : n_pixels;
    const unsigned blocks = (unsigned)std::min<size_t>((work + 255) / 256, 152 * 16);
    cudaStream_t st = static_cast<cudaStream_t>(stream_ptr);
    uint32_t *dst = static_cast<uint32_t *>(dst_rgba);
    const uint8_t *src = static_cast<const uint8_t *>(src_rgb);
    if (vec)
        isti::rgb8_to_rgba8_kernel<true><<<blocks, 256, 0, st>>>(dst, src, n_pixels);
    else
        isti::rgb8_to_rgba8_kernel<false><<<blocks, 256, 0, st>>>(dst, src, n_pixels);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_rgb8_to_rgba8");
}

// Sparse shadow entries -> RGBA8 shadow images, declared in include/isti_dataset.h.
extern "C" isti_status isti_unpack_shadows(void *info_rgba, void *a_rgba, void *b_rgba, size_t n_pixels, const void *entries, size_t n_entries,
                                           const void *clear_entries, size_t n_clear, void *stream_ptr)
{
    if (n_pixels == 0)
        return ISTI_OK;
    if (!info_rgba || !a_rgba || !b_rgba || (n_entries && !entries))
        return fail(ISTI_ERR_INVALID_ARG, "isti_unpack_shadows: NULL buffer");
    if ((((uintptr_t)info_rgba | (uintptr_t)a_rgba | (uintptr_t)b_rgba | (uintptr_t)entries | (uintptr_t)clear_entries) & 15u) != 0)
        return fail(ISTI_ERR_INVALID_ARG, "isti_unpack_shadows: buffers must be 16-byte aligned");
    const size_t img = 4 * n_pixels;
    const uintptr_t imgs[3] = {(uintptr_t)info_rgba, (uintptr_t)a_rgba, (uintptr_t)b_rgba};
    const uintptr_t lists[2][2] = {{(uintptr_t)entries, (uintptr_t)entries + n_entries * ISTI_SHADOW_ENTRY_BYTES},
                                   {(uintptr_t)clear_entries, (uintptr_t)clear_entries + (clear_entries ? n_clear : 0) * ISTI_SHADOW_ENTRY_BYTES}};
    for (int i = 0; i < 3; i++)
    {
        for (int j = i + 1; j < 3; j++)
            if (imgs[i] < imgs[j] + img && imgs[j] < imgs[i] + img)
                return fail(ISTI_ERR_INVALID_ARG, "isti_unpack_shadows: images overlap");
        for (const auto &l : lists)
            if (l[1] > l[0] && imgs[i] < l[1] && l[0] < imgs[i] + img)
                return fail(ISTI_ERR_INVALID_ARG, "isti_unpack_shadows: an image overlaps the entries");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream_ptr);
    cudaError_t e = cudaSuccess;
    if (!clear_entries)
        for (int i = 0; i < 3 && e == cudaSuccess; i++)
            e = cudaMemsetAsync(reinterpret_cast<void *>(imgs[i]), 0, img, st);
    else if (n_clear)
    {
        const unsigned blocks = (unsigned)std::min<size_t>((n_clear + 255) / 256, 152 * 8);
        isti::clear_shadows_kernel<<<blocks, 256, 0, st>>>(static_cast<uint32_t *>(info_rgba), static_cast<uint32_t *>(a_rgba),
                                                           static_cast<uint32_t *>(b_rgba), n_pixels, static_cast<const uint4 *>(clear_entries),
                                                           n_clear);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && n_entries)
    {
        const unsigned blocks = (unsigned)std::min<size_t>((n_entries + 255) / 256, 152 * 8);
        isti::unpack_shadows_kernel<<<blocks, 256, 0, st>>>(static_cast<uint32_t *>(info_rgba), static_cast<uint32_t *>(a_rgba),
                                                            static_cast<uint32_t *>(b_rgba), n_pixels, static_cast<const uint4 *>(entries),
                                                            n_entries);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_unpack_shadows");
}

// convertDepthToZ_kernel (src/file_reader.cu:17-37), declared in include/isti_dataset.h.
extern "C" isti_status isti_depth_to_z(float *depth, int32_t width, int32_t height, void *stream_ptr)
{
    if (!depth || width <= 0 || height <= 0)
        return fail(ISTI_ERR_INVALID_ARG, "isti_depth_to_z: bad argument");
    const size_t n = (size_t)width * (size_t)height;
    const bool vec = ((uintptr_t)depth & 15) == 0;
    const size_t work = vec ? n / 4 + 3 : n;
    const unsigned blocks = (unsigned)std::min<size_t>((work + 255) / 256, 152 * 16);
    cudaStream_t s = static_cast<cudaStream_t>(stream_ptr);
    if (vec)
        isti::depth_to_z_kernel<true><<<blocks, 256, 0, s>>>(depth, n);
    else
        isti::depth_to_z_kernel<false><<<blocks, 256, 0, s>>>(depth, n);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_depth_to_z");
}
