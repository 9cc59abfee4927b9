// Keyframe loader of the reference's dataset format (include/isti_dataset.h).
//
// Reference: FrameFileReader (include/file_reader.h, src/file_reader.cu) and
// FrameData (include/data.h).  Each camera owns two device slots (the
// reference's fwd/bwd and curr/next MotionZBufferImage objects) that are
// swapped by pointer on every keyframe, as FrameData::swap does; a keyframe's
// files are decoded on host threads and copied into the slot in one pass.
#include "isti_dataset.h"
#include "isti_error.hpp"
#include "isti_io.h"
#include "isti_json.hpp"
#include "isti_mat4.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace fs = std::filesystem;
using isti::set_error;
using isti::host::mat4;

struct isti_camera_path
{
    isti_camera_info info{};
    std::vector<isti_camera_frame> frames;
};

namespace
{
// cam.json of one camera folder (FrameFileReader::initCamInfo, src/file_reader.cu:78-107).
isti_status parse_camera(const fs::path &dir, isti_camera_path &out)
{
    const fs::path file = dir / "cam.json";
    std::ifstream f(file, std::ios::binary);
    if (!f)
        return set_error(ISTI_ERR_INVALID_ARG, "Failed to open camera file: " + file.string());
    std::stringstream ss;
    ss << f.rdbuf();
    try
    {
        const isti::host::Json j = isti::host::Json::parse(ss.str());
        const isti::host::Json &frames = j.at("frames");
        if (frames.kind != isti::host::Json::Array)
            return set_error(ISTI_ERR_INVALID_ARG, "cam.json: \"frames\" is not an array (" + file.string() + ")");
        out.frames.clear();
        for (const isti::host::Json &fr : frames.items)
        {
            isti_camera_frame cf{};
            cf.idx = fr.at("idx").as_int();
            // glm::from_json (file_reader.cu:41-62): m[c][r] = "e<r><c>"
            for (int which = 0; which < 2; which++)
            {
                const isti::host::Json &m = fr.at(which == 0 ? "w2c" : "proj");
                float *dst = which == 0 ? cf.w2c : cf.proj;
                for (int c = 0; c < 4; c++)
                    for (int r = 0; r < 4; r++)
                        dst[c * 4 + r] = m.at("e" + std::to_string(r) + std::to_string(c)).as_float();
            }
            out.frames.push_back(cf);
        }
        if (out.frames.empty())
            return set_error(ISTI_ERR_INVALID_ARG, "Could not load any frames from camera file: " + file.string());
        const isti::host::Json &res = j.at("resolution");
        out.info.width = res.at("x").as_int();
        out.info.height = res.at("y").as_int();
        auto int_or = [&](const char *key, int dflt) {
            const isti::host::Json *v = j.find(key);
            return v ? v->as_int() : dflt;
        };
        auto bool_or = [&](const char *key, bool dflt) {
            const isti::host::Json *v = j.find(key);
            return v ? v->as_bool() : dflt;
        };
        out.info.client_fps = int_or("clientFps", 60);
        out.info.server_fps = int_or("serverFps", 10);
        out.info.shadow_fps = int_or("shadowFps", 60);
        out.info.priority = int(bool_or("objectMotion", true)) * 2 + int(bool_or("shadowGradients", true));
        out.info.n_frames = int32_t(out.frames.size());
    }
    catch (const std::exception &e)
    {
        return set_error(ISTI_ERR_INVALID_ARG, std::string(e.what()) + " (" + file.string() + ")");
    }
    if (out.info.width <= 0 || out.info.height <= 0 || out.info.width > 65535 || out.info.height > 65535)
        return set_error(ISTI_ERR_INVALID_ARG, "cam.json: resolution must be 1..65535 (" + file.string() + ")");
    return ISTI_OK;
}

std::string frame_name(int idx)
{
    std::ostringstream ss; // the reference's std::setw(4) << std::setfill('0')
    ss << std::setw(4) << std::setfill('0') << idx;
    return ss.str();
}

mat4 mat_of(const float *v)
{
    mat4 m;
    std::memcpy(m.m, v, sizeof(m.m));
    return m;
}

// One camera at one keyframe on the device (MotionZBufferImage, include/data.h:49-62).
struct Slot
{
    uint32_t w = 0, h = 0;
    void *color = nullptr, *z = nullptr, *motion = nullptr;
    void *shadow[3] = {nullptr, nullptr, nullptr}; // colour A, colour B, info
    bool motion_present = true;
    bool shadow_present[3] = {true, true, true};
    mat4 view{}, proj{}, vp{}, ivp{};
};

enum class FileKind { Color, Depth, Motion, Shadow };

struct Job
{
    Job(fs::path p, FileKind k, void *d, uint32_t w_, uint32_t h_) : path(std::move(p)), kind(k), dst(d), w(w_), h(h_) {}
    fs::path path;
    FileKind kind;
    void *dst;
    uint32_t w, h;
    uint8_t *png = nullptr;
    float *exr = nullptr;
    isti_status status = ISTI_OK;
    std::string err;
};

void decode(Job &j)
{
    int32_t w = 0, h = 0, ch = 0;
    if (j.kind == FileKind::Color || j.kind == FileKind::Shadow)
        j.status = isti_png_decode_file(j.path.string().c_str(), &w, &h, &j.png);
    else
    {
        j.status = isti_exr_decode_file(j.path.string().c_str(), &w, &h, &ch, &j.exr);
        if (j.status == ISTI_OK)
        {
            const int32_t want = j.kind == FileKind::Depth ? 1 : 4;
            if (ch != want)
            {
                j.status = ISTI_ERR_INVALID_ARG;
                j.err = std::string(j.kind == FileKind::Depth ? "depth" : "flow field") + " file must hold " +
                        (want == 1 ? "one channel: " : "R, G, B (and A) channels: ") + j.path.string();
                return;
            }
        }
    }
    if (j.status != ISTI_OK)
    {
        j.err = isti_last_error();
        return;
    }
    if (uint32_t(w) != j.w || uint32_t(h) != j.h)
    {
        j.status = ISTI_ERR_INVALID_ARG;
        j.err = "Image resolution has to be set in advance: " + j.path.string();
    }
}

} // namespace

struct isti_dataset
{
    fs::path input;
    isti_camera_path main;
    std::vector<isti_camera_path> aux;
    std::vector<fs::path> cam_dirs; // [main, aux...]
    std::vector<Slot> slots;        // two per camera
    std::vector<Slot *> curr, next; // per camera: fwd/curr and bwd/next
    int frame_index = 0;
    cudaStream_t stream = nullptr;
    std::vector<isti_view> aux_curr_views, aux_next_views;
    std::vector<int32_t> priorities;

    ~isti_dataset()
    {
        for (Slot &s : slots)
        {
            cudaFree(s.color);
            cudaFree(s.z);
            cudaFree(s.motion);
            for (void *p : s.shadow)
                cudaFree(p);
        }
    }

    const isti_camera_path &camera(size_t c) const { return c == 0 ? main : aux[c - 1]; }

    isti_status alloc_slot(Slot &s, uint32_t w, uint32_t h)
    {
        s.w = w;
        s.h = h;
        const size_t px = size_t(w) * h;
        cudaError_t e = cudaSuccess;
        auto get = [&](void **p, size_t bytes) {
            if (e == cudaSuccess)
                e = cudaMalloc(p, bytes);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(*p, 0, bytes, stream);
        };
        get(&s.color, px * 4);
        get(&s.z, px * 4);
        get(&s.motion, px * 16);
        for (void *&p : s.shadow)
            get(&p, px * 4);
        if (e != cudaSuccess)
            return set_error(e == cudaErrorMemoryAllocation ? ISTI_ERR_OOM : ISTI_ERR_CUDA,
                             std::string("isti_dataset: device buffers: ") + cudaGetErrorString(e));
        return ISTI_OK;
    }

    // Decodes `jobs` on host threads, then copies them to the device and converts depth to z.
    isti_status run_jobs(std::vector<Job> &jobs)
    {
        if (jobs.empty())
            return ISTI_OK;
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const size_t n_threads = std::min<size_t>(jobs.size(), std::min(hw, 16u));
        std::atomic<size_t> next_job{0};
        auto worker = [&]() {
            // the files are decoded side by side: one thread per file (restored for the caller's thread)
            isti::set_decode_threads(n_threads > 1 ? 1 : 0);
            for (size_t k; (k = next_job.fetch_add(1)) < jobs.size();)
                decode(jobs[k]);
            isti::set_decode_threads(0);
        };
        std::vector<std::thread> threads;
        for (size_t t = 1; t < n_threads; t++)
            threads.emplace_back(worker);
        worker();
        for (std::thread &t : threads)
            t.join();
        isti_status st = ISTI_OK;
        std::string err;
        for (Job &j : jobs)
        {
            if (j.status != ISTI_OK && st == ISTI_OK)
            {
                st = j.status;
                err = j.err;
            }
            if (st != ISTI_OK)
                continue;
            const size_t px = size_t(j.w) * j.h;
            const void *src = j.png ? static_cast<const void *>(j.png) : static_cast<const void *>(j.exr);
            const size_t bytes = j.kind == FileKind::Motion ? px * 16 : px * 4;
            cudaError_t e = cudaMemcpyAsync(j.dst, src, bytes, cudaMemcpyHostToDevice, stream);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(stream); // the host buffer is released below
            if (e != cudaSuccess)
            {
                st = ISTI_ERR_CUDA;
                err = std::string("isti_dataset: upload: ") + cudaGetErrorString(e);
                continue;
            }
            if (j.kind == FileKind::Depth)
            {
                const isti_status s = isti_depth_to_z(static_cast<float *>(j.dst), int32_t(j.w), int32_t(j.h), stream);
                if (s != ISTI_OK)
                {
                    st = s;
                    err = isti_last_error();
                }
            }
        }
        for (Job &j : jobs)
        {
            isti_image_free(j.png);
            isti_image_free(j.exr);
        }
        if (st != ISTI_OK)
            return set_error(st, err);
        const cudaError_t e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess)
            return set_error(ISTI_ERR_CUDA, std::string("isti_dataset: ") + cudaGetErrorString(e));
        return ISTI_OK;
    }

    // FrameFileReader::readColorDepthCam (file_reader.cu:138-157) for every
    // camera into its "next" slot.
    void color_depth_jobs(int frame_idx, std::vector<Job> &jobs)
    {
        for (size_t c = 0; c < cam_dirs.size(); c++)
        {
            const isti_camera_path &cam = camera(c);
            Slot &s = *next[c];
            const isti_camera_frame &fr = cam.frames[size_t(frame_idx)];
            s.view = mat_of(fr.w2c);
            s.proj = isti::host::normalize_proj(mat_of(fr.proj));
            s.vp = isti::host::mul(s.proj, s.view);
            s.ivp = isti::host::inverse(s.vp);
            const std::string name = frame_name(fr.idx);
            jobs.emplace_back(cam_dirs[c] / "color" / (name + ".png"), FileKind::Color, s.color, s.w, s.h);
            jobs.emplace_back(cam_dirs[c] / "depth" / (name + ".exr"), FileKind::Depth, s.z, s.w, s.h);
        }
    }

    isti_status read_next(int32_t *advanced)
    {
        for (size_t c = 0; c < curr.size(); c++) // FrameData::swap (include/data.h:110-116)
            std::swap(curr[c], next[c]);
        *advanced = 0;
        if (frame_index >= main.info.n_frames - 1)
            return ISTI_OK;
        for (const isti_camera_path &a : aux) // the reference indexes past the end here
            if (frame_index + 1 >= a.info.n_frames)
                return set_error(ISTI_ERR_INVALID_ARG, "isti_dataset: an aux camera has fewer frames than the main camera");
        std::vector<Job> jobs;
        color_depth_jobs(frame_index + 1, jobs);
        // readIfDirExists (file_reader.cu:180-188): the pair's flow fields and
        // shadow images, named after the earlier keyframe of the main camera
        const std::string name = frame_name(main.frames[size_t(frame_index)].idx);
        static const char *const SHADOW_DIRS[2][3] = {
            {"forwardShadowColorA", "forwardShadowColorB", "forwardShadowInfo"},
            {"backwardShadowColorA", "backwardShadowColorB", "backwardShadowInfo"}};
        for (size_t c = 0; c < cam_dirs.size(); c++)
        {
            for (int dir = 0; dir < 2; dir++)
            {
                Slot &s = dir == 0 ? *curr[c] : *next[c];
                const fs::path flow_dir = cam_dirs[c] / (dir == 0 ? "forwardFlowField" : "backwardFlowField");
                s.motion_present = fs::exists(flow_dir);
                if (s.motion_present)
                    jobs.emplace_back(flow_dir / (name + ".exr"), FileKind::Motion, s.motion, s.w, s.h);
                for (int k = 0; k < 3; k++)
                {
                    const fs::path d = cam_dirs[c] / SHADOW_DIRS[dir][k];
                    s.shadow_present[k] = fs::exists(d);
                    if (s.shadow_present[k])
                        jobs.emplace_back(d / (name + ".png"), FileKind::Shadow, s.shadow[k], s.w, s.h);
                }
            }
        }
        const isti_status st = run_jobs(jobs);
        if (st != ISTI_OK)
            return st;
        frame_index++;
        *advanced = 1;
        return ISTI_OK;
    }

    static isti_view view_of(const Slot &s)
    {
        isti_view v{};
        v.width = s.w;
        v.height = s.h;
        v.color = s.color;
        v.z = static_cast<const float *>(s.z);
        v.motion = s.motion_present ? s.motion : nullptr;
        v.motion_format = s.motion_present ? ISTI_MOTION_F32X4 : ISTI_MOTION_NONE;
        // the reference gates soft shadows on colour A (src/renderer.cu:277) and
        // then reads the info image; without an info image they are disabled here
        const bool shadows = s.shadow_present[0] && s.shadow_present[2];
        v.shadow_color_a = shadows ? s.shadow[0] : nullptr;
        v.shadow_color_b = shadows && s.shadow_present[1] ? s.shadow[1] : nullptr;
        v.shadow_info = shadows ? s.shadow[2] : nullptr;
        std::memcpy(v.viewproj, s.vp.m, sizeof(v.viewproj));
        std::memcpy(v.inv_viewproj, s.ivp.m, sizeof(v.inv_viewproj));
        return v;
    }
};

extern "C" {

isti_status isti_camera_path_open(const char *dir, isti_camera_path **out)
{
    if (!dir || !out)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_camera_path_open: null argument");
    auto *p = new (std::nothrow) isti_camera_path;
    if (!p)
        return set_error(ISTI_ERR_OOM, "isti_camera_path_open: out of host memory");
    const isti_status st = parse_camera(dir, *p);
    if (st != ISTI_OK)
    {
        delete p;
        return st;
    }
    *out = p;
    return ISTI_OK;
}

isti_status isti_camera_path_info(const isti_camera_path *p, isti_camera_info *info)
{
    if (!p || !info)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_camera_path_info: null argument");
    *info = p->info;
    return ISTI_OK;
}

isti_status isti_camera_path_frame(const isti_camera_path *p, int32_t i, isti_camera_frame *frame)
{
    if (!p || !frame)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_camera_path_frame: null argument");
    if (i < 0 || size_t(i) >= p->frames.size())
        return set_error(ISTI_ERR_INVALID_ARG, "isti_camera_path_frame: frame index out of range");
    *frame = p->frames[size_t(i)];
    return ISTI_OK;
}

void isti_camera_path_close(isti_camera_path *p) { delete p; }

isti_status isti_dataset_open(const char *input_dir, int32_t n_aux, const char *const *aux_dirs, void *stream,
                              isti_dataset **out)
{
    if (!input_dir || !out || n_aux < 0 || n_aux > ISTI_MAX_AUX_CAMS || (n_aux > 0 && !aux_dirs))
        return set_error(ISTI_ERR_INVALID_ARG, "isti_dataset_open: bad argument");
    auto *d = new (std::nothrow) isti_dataset;
    if (!d)
        return set_error(ISTI_ERR_OOM, "isti_dataset_open: out of host memory");
    d->input = input_dir;
    d->stream = static_cast<cudaStream_t>(stream);
    d->cam_dirs.push_back(d->input / "main");
    isti_status st = parse_camera(d->cam_dirs[0], d->main);
    for (int32_t i = 0; st == ISTI_OK && i < n_aux; i++)
    {
        if (!aux_dirs[i])
            st = set_error(ISTI_ERR_INVALID_ARG, "isti_dataset_open: null aux directory");
        else
        {
            d->cam_dirs.push_back(d->input / aux_dirs[i]);
            d->aux.emplace_back();
            st = parse_camera(d->cam_dirs.back(), d->aux.back());
        }
    }
    const size_t n_cams = d->cam_dirs.size();
    if (st == ISTI_OK)
    {
        d->slots.resize(2 * n_cams);
        for (size_t c = 0; c < n_cams && st == ISTI_OK; c++)
        {
            const isti_camera_info &ci = d->camera(c).info;
            for (int k = 0; k < 2 && st == ISTI_OK; k++)
                st = d->alloc_slot(d->slots[2 * c + size_t(k)], uint32_t(ci.width), uint32_t(ci.height));
            d->curr.push_back(&d->slots[2 * c]);
            d->next.push_back(&d->slots[2 * c + 1]);
        }
    }
    if (st == ISTI_OK)
    {
        std::vector<Job> jobs; // FrameFileReader::init -> readColorDepth(frame, 0)
        d->color_depth_jobs(0, jobs);
        st = d->run_jobs(jobs);
    }
    if (st != ISTI_OK)
    {
        delete d;
        return st;
    }
    for (size_t c = 1; c < n_cams; c++)
        d->priorities.push_back(d->aux[c - 1].info.priority);
    *out = d;
    return ISTI_OK;
}

isti_status isti_dataset_read_next(isti_dataset *d, int32_t *advanced)
{
    if (!d || !advanced)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_dataset_read_next: null argument");
    return d->read_next(advanced);
}

isti_status isti_dataset_frame(isti_dataset *d, isti_frame_data *frame)
{
    if (!d || !frame)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_dataset_frame: null argument");
    const size_t n_aux = d->aux.size();
    d->aux_curr_views.resize(n_aux);
    d->aux_next_views.resize(n_aux);
    for (size_t i = 0; i < n_aux; i++)
    {
        d->aux_curr_views[i] = isti_dataset::view_of(*d->curr[i + 1]);
        d->aux_next_views[i] = isti_dataset::view_of(*d->next[i + 1]);
    }
    *frame = isti_frame_data{};
    frame->fwd = isti_dataset::view_of(*d->curr[0]);
    frame->bwd = isti_dataset::view_of(*d->next[0]);
    frame->num_aux = int32_t(n_aux);
    frame->aux_curr = n_aux ? d->aux_curr_views.data() : nullptr;
    frame->aux_next = n_aux ? d->aux_next_views.data() : nullptr;
    frame->aux_priority = n_aux ? d->priorities.data() : nullptr;
    return ISTI_OK;
}

isti_status isti_dataset_camera(const isti_dataset *d, int32_t camera, isti_camera_info *info)
{
    if (!d || !info || camera < -1 || camera >= int32_t(d->aux.size()))
        return set_error(ISTI_ERR_INVALID_ARG, "isti_dataset_camera: bad argument");
    *info = camera < 0 ? d->main.info : d->aux[size_t(camera)].info;
    return ISTI_OK;
}

isti_status isti_dataset_matrices(const isti_dataset *d, int32_t slot, float view[16], float proj[16])
{
    if (!d || (slot != 0 && slot != 1))
        return set_error(ISTI_ERR_INVALID_ARG, "isti_dataset_matrices: bad argument");
    const Slot &s = slot == 0 ? *d->curr[0] : *d->next[0];
    if (view)
        std::memcpy(view, s.view.m, sizeof(s.view.m));
    if (proj)
        std::memcpy(proj, s.proj.m, sizeof(s.proj.m));
    return ISTI_OK;
}

int32_t isti_dataset_keyframe(const isti_dataset *d) { return d ? d->frame_index : -1; }

void isti_dataset_close(isti_dataset *d)
{
    if (d && d->stream)
        cudaStreamSynchronize(d->stream);
    delete d;
}

isti_status isti_normalize_proj(const float proj[16], float out[16])
{
    if (!proj || !out)
        return set_error(ISTI_ERR_INVALID_ARG, "isti_normalize_proj: null argument");
    const mat4 r = isti::host::normalize_proj(mat_of(proj));
    std::memcpy(out, r.m, sizeof(r.m));
    return ISTI_OK;
}

void isti_mat4_mul(const float a[16], const float b[16], float out[16])
{
    const mat4 r = isti::host::mul(mat_of(a), mat_of(b));
    std::memcpy(out, r.m, sizeof(r.m));
}

void isti_mat4_inverse(const float m[16], float out[16])
{
    const mat4 r = isti::host::inverse(mat_of(m));
    std::memcpy(out, r.m, sizeof(r.m));
}

void isti_mat4_interpolate(const float m1[16], const float m2[16], float t, float out[16])
{
    const mat4 r = isti::host::interpolate(mat_of(m1), mat_of(m2), t);
    std::memcpy(out, r.m, sizeof(r.m));
}

} // extern "C"
