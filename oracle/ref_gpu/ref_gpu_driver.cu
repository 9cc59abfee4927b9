// The reference's own src/renderer.cu, compiled for the GPU (sm_103a) with the
// reference's CUDA flags (CMakeLists.txt:36: -use_fast_math
// --expt-relaxed-constexpr --expt-extended-lambda, minus -keep), and run in the
// same process as the GB300 kernels.  TEST INFRASTRUCTURE ONLY: tests/ use it
// as the checker of the sm_103a path, bench.py as the timed reference GPU
// baseline.  Nothing in the product links or loads it.
//
// build_ref.py stages unmodified copies of src/renderer.cu and the headers it
// includes under oracle/_ref/gpu/ (never committed); this translation unit
// includes renderer.cu as it is.  What the reference links besides it is
// written here from the interfaces it declares:
//  * ImageBuffer<T, N> (include/util/image_buffer.h:9-48) on CUDA arrays with
//    the texture/surface setup of src/util/image_buffer.cu:54-58,227-264: point
//    filtering, unnormalised coordinates, border addressing, element reads;
//    uploads and downloads accept host or device pointers (cudaMemcpyDefault);
//    the file readers/writers are not needed and throw.
//  * glm: the subset in oracle/ref_host/glm (the reference's glm submodule is
//    empty), device-callable under nvcc.
//
// Entry points (host arrays in, host arrays out, like the CPU harness
// ref_host/ref_driver.cpp):
//  * isti_refgpu_render: one Renderer::render (src/renderer.cu:607-694) on a
//    fresh Renderer, then the output image, splat buffers and flow fields;
//  * isti_refgpu_time: one Renderer and FrameData kept alive, `warmup` + `repeats`
//    rounds of Renderer::render over the given client frames, each call
//    bracketed by CUDA events on the legacy default stream (the stream the
//    reference launches on); per-call milliseconds out.
#include <cuda_runtime.h>
#include <device_launch_parameters.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <memory>
#include <new>
#include <optional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <glm/glm.hpp>

// Renderer's splat buffers and flow fields (include/renderer.h:58-92) and
// ImageBuffer's array and texture handles (include/util/image_buffer.h:40-47) are
// private; the harness reads them back and releases them.
#define private public
#include "renderer.cu"
#undef private

#include "../isti_oracle.h"

// ---- ImageBuffer<T, N> on CUDA arrays ----

template <typename T>
__global__ void refgpu_sum_kernel(cudaTextureObject_t tex, uint2 res, T *acc)
{
    const unsigned x = threadIdx.x + blockIdx.x * blockDim.x, y = threadIdx.y + blockIdx.y * blockDim.y;
    if (x >= res.x || y >= res.y)
        return;
    atomicAdd(acc, tex2D<T>(tex, x, y));
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::resize(uint2 resolution)
{
    if (resolution.x == _resolution.x && resolution.y == _resolution.y)
        return;
    if (_resolution.x != 0 || _resolution.y != 0)
        throw std::runtime_error("Resizing of ImageBuffer currently not supported");
    _resolution = resolution;
    cudaChannelFormatDesc desc = cudaCreateChannelDesc<T>();
    if (cudaMallocArray(&_array, &desc, resolution.x, resolution.y, cudaArraySurfaceLoadStore) != cudaSuccess)
        throw std::runtime_error("cudaMallocArray failed");
    init();
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::init(cudaTextureAddressMode address_mode)
{
    _surface = createSurface();
    _texture = createTexture(cudaFilterModePoint, address_mode);
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::memsetBuffer(T val)
{
    std::vector<T> tmp((size_t)_resolution.x * _resolution.y, val);
    upload(tmp.data());
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::download(T *h_buffer)
{
    if (cudaMemcpy2DFromArray(h_buffer, _resolution.x * sizeof(T), _array, 0, 0, _resolution.x * sizeof(T), _resolution.y,
                              cudaMemcpyDefault) != cudaSuccess)
        throw std::runtime_error("cudaMemcpy2DFromArray failed");
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::upload(T *h_buffer)
{
    if (cudaMemcpy2DToArray(_array, 0, 0, h_buffer, _resolution.x * sizeof(T), _resolution.x * sizeof(T), _resolution.y,
                            cudaMemcpyDefault) != cudaSuccess)
        throw std::runtime_error("cudaMemcpy2DToArray failed");
}

template <typename T, int N_CHANNELS>
T ImageBuffer<T, N_CHANNELS>::average()
{
    if constexpr (!std::is_same_v<T, float>)
        return T();
    else
    {
        float *acc = nullptr;
        cudaMalloc(&acc, sizeof(float));
        cudaMemset(acc, 0, sizeof(float));
        dim3 block(16, 16), grid((_resolution.x + 15) / 16, (_resolution.y + 15) / 16);
        refgpu_sum_kernel<float><<<grid, block>>>(_texture, _resolution, acc);
        float h = 0.0f;
        cudaMemcpy(&h, acc, sizeof(float), cudaMemcpyDeviceToHost);
        cudaFree(acc);
        h /= (_resolution.x * _resolution.y);
        return h;
    }
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::readFromFile(std::filesystem::path)
{
    throw std::runtime_error("ImageBuffer::readFromFile is not part of the GPU oracle harness");
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::writeImageToFile(std::vector<T> &, int, int, int, std::filesystem::path)
{
    throw std::runtime_error("ImageBuffer::writeImageToFile is not part of the GPU oracle harness");
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::writeToFile(std::filesystem::path)
{
    throw std::runtime_error("ImageBuffer::writeToFile is not part of the GPU oracle harness");
}

template <typename T, int N_CHANNELS>
cudaTextureObject_t ImageBuffer<T, N_CHANNELS>::createTexture(cudaTextureFilterMode filter_mode, cudaTextureAddressMode address_mode)
{
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = _array;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof td);
    td.normalizedCoords = false;
    td.filterMode = filter_mode;
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = address_mode;
    td.readMode = cudaReadModeElementType;
    cudaTextureObject_t t = 0;
    if (cudaCreateTextureObject(&t, &rd, &td, nullptr) != cudaSuccess)
        throw std::runtime_error("cudaCreateTextureObject failed");
    return t;
}

template <typename T, int N_CHANNELS>
cudaSurfaceObject_t ImageBuffer<T, N_CHANNELS>::createSurface()
{
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = _array;
    cudaSurfaceObject_t s = 0;
    if (cudaCreateSurfaceObject(&s, &rd) != cudaSuccess)
        throw std::runtime_error("cudaCreateSurfaceObject failed");
    return s;
}

template struct ImageBuffer<uchar4, 4>;
template struct ImageBuffer<float, 1>;
template struct ImageBuffer<float4, 4>;

// ---- harness ----

namespace
{
// Every CUDA array and texture the harness creates is released after a call: the
// reference never frees its ImageBuffers, so they are tracked here.
struct Owned
{
    std::vector<cudaArray_t> arrays;
    std::vector<cudaTextureObject_t> textures;
    std::vector<cudaSurfaceObject_t> surfaces;
    std::vector<void *> device;
};

template <typename T, int N>
void track(Owned &o, ImageBuffer<T, N> &b)
{
    if (b._resolution.x == 0)
        return;
    o.arrays.push_back(b._array);
    o.textures.push_back(b._texture);
    o.surfaces.push_back(b._surface);
}

template <typename T, int N>
void track(Owned &o, std::optional<ImageBuffer<T, N>> &b)
{
    if (b.has_value())
        track(o, b.value());
}

void track_view(Owned &o, MotionZBufferImage &v)
{
    track(o, v.img);
    track(o, v.shadowColorA_img);
    track(o, v.shadowColorB_img);
    track(o, v.shadowInfo_img);
    track(o, v.z_buffer);
    track(o, v.object_motion);
}

void release(Owned &o)
{
    for (auto t : o.textures)
        cudaDestroyTextureObject(t);
    for (auto s : o.surfaces)
        cudaDestroySurfaceObject(s);
    for (auto a : o.arrays)
        cudaFreeArray(a);
    for (auto p : o.device)
        cudaFree(p);
    o = Owned{};
}

void track_renderer(Owned &o, Renderer &r)
{
    track(o, r.fwd2bwd_ff);
    track(o, r.fwd2cam_ff);
    track(o, r.fwd_momentum);
    track(o, r.bwd2fwd_ff);
    track(o, r.bwd2cam_ff);
    track(o, r.bwd_momentum);
    for (auto *vec : {&r.fwd2bwd_aux_ff, &r.fwd2cam_aux_ff, &r.bwd2fwd_aux_ff, &r.bwd2cam_aux_ff})
        for (auto &b : *vec)
            track(o, b);
    o.device.push_back(r.d_fwd_main_splatting_buffer);
    o.device.push_back(r.d_bwd_main_splatting_buffer);
    for (auto &s : r.d_aux_cam_splatting_buffers)
    {
        o.device.push_back(s.forward);
        o.device.push_back(s.backward);
    }
    o.device.push_back(r.d_fwd_aux_cam_info);
    o.device.push_back(r.d_bwd_aux_cam_info);
}

glm::mat4 to_mat(const float *m)
{
    glm::mat4 r;
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++)
            r[c][rr] = m[c * 4 + rr];
    return r;
}

void fill(MotionZBufferImage &img, const oracle_view &v)
{
    img.img.upload(reinterpret_cast<uchar4 *>(const_cast<uint8_t *>(v.color)));
    img.z_buffer.upload(const_cast<float *>(v.z));
    if (v.motion)
        img.object_motion.value().upload(reinterpret_cast<float4 *>(const_cast<float *>(v.motion)));
    auto opt_upload = [](std::optional<ImageBuffer<uchar4, 4>> &buf, const uint8_t *src) {
        if (src)
            buf.value().upload(reinterpret_cast<uchar4 *>(const_cast<uint8_t *>(src)));
    };
    opt_upload(img.shadowColorA_img, v.shadow_color_a);
    opt_upload(img.shadowColorB_img, v.shadow_color_b);
    opt_upload(img.shadowInfo_img, v.shadow_info);
    img.viewproj_mat = to_mat(v.viewproj);
    img.inv_viewproj_mat = to_mat(v.inv_viewproj);
}

// Absent optional images are dropped before resize, so no array is made for them.
void shape(MotionZBufferImage &img, const oracle_view &v)
{
    if (!v.motion)
        img.object_motion = std::nullopt;
    if (!v.shadow_color_a)
        img.shadowColorA_img = std::nullopt;
    if (!v.shadow_color_b)
        img.shadowColorB_img = std::nullopt;
    if (!v.shadow_info)
        img.shadowInfo_img = std::nullopt;
}

std::unique_ptr<FrameData> make_frame(const oracle_frame *frame)
{
    const int n_aux = frame->num_aux;
    std::unique_ptr<FrameData> fd(new FrameData((uint8_t)n_aux));
    std::vector<uint2> aux_res;
    std::vector<int> aux_prio;
    for (int i = 0; i < n_aux; i++)
    {
        aux_res.push_back(make_uint2(frame->aux_curr[i].width, frame->aux_curr[i].height));
        aux_prio.push_back(frame->aux_priority ? frame->aux_priority[i] : 0);
    }
    shape(*fd->fwd, frame->fwd);
    shape(*fd->bwd, frame->bwd);
    for (int i = 0; i < n_aux; i++)
    {
        shape(*fd->aux_cam_images[i].curr, frame->aux_curr[i]);
        shape(*fd->aux_cam_images[i].next, frame->aux_next[i]);
    }
    fd->resize(make_uint2(frame->fwd.width, frame->fwd.height), aux_res, aux_prio);
    fill(*fd->fwd, frame->fwd);
    fill(*fd->bwd, frame->bwd);
    for (int i = 0; i < n_aux; i++)
    {
        fill(*fd->aux_cam_images[i].curr, frame->aux_curr[i]);
        fill(*fd->aux_cam_images[i].next, frame->aux_next[i]);
    }
    return fd;
}

void track_frame(Owned &o, FrameData &fd)
{
    track_view(o, *fd.fwd);
    track_view(o, *fd.bwd);
    for (auto &a : fd.aux_cam_images)
    {
        track_view(o, *a.curr);
        track_view(o, *a.next);
    }
}

RenderInfo make_info(const oracle_render_info *info)
{
    return RenderInfo{make_uint2(info->width, info->height), info->alpha, to_mat(info->viewproj), to_mat(info->inv_viewproj),
                      {info->frames_per_anchor, info->shadow_frames_per_anchor, info->no_shadows != 0, (RenderMode)info->mode}};
}

void export_view(oracle_view_out &o, uint64_cu *splat, ImageBuffer<float4, 4> &cam_ff, ImageBuffer<float4, 4> &full_ff, uint2 dims)
{
    const size_t n = (size_t)dims.x * dims.y;
    if (o.splat && cudaMemcpy(o.splat, splat, n * sizeof(uint64_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        throw std::runtime_error("copying a splat buffer failed");
    if (o.cam_ff)
        cam_ff.download(reinterpret_cast<float4 *>(o.cam_ff));
    if (o.full_ff)
        full_ff.download(reinterpret_cast<float4 *>(o.full_ff));
}

// Renderer::_curr_resolution has no initialiser (include/renderer.h:86) and
// resizeBuffers only allocates the splat buffers when it differs from the render
// resolution (src/renderer.cu:575): construct in zeroed storage.
struct RendererHolder
{
    void *storage = nullptr;
    Renderer *r = nullptr;
    RendererHolder()
    {
        storage = std::calloc(1, sizeof(Renderer));
        if (!storage)
            throw std::bad_alloc();
        r = new (storage) Renderer();
    }
    ~RendererHolder()
    {
        r->~Renderer();
        std::free(storage);
    }
};
} // namespace

extern "C" int isti_refgpu_render(const oracle_frame *frame, const oracle_render_info *info, uint8_t *out_rgba, oracle_view_out *outs)
{
    int rc = 0;
    Owned owned;
    try
    {
        RendererHolder holder;
        Renderer &renderer = *holder.r;
        std::unique_ptr<FrameData> fd = make_frame(frame);
        track_frame(owned, *fd);
        ImageBuffer<uchar4, 4> out(make_uint2(info->width, info->height));
        track(owned, out);
        out.upload(reinterpret_cast<uchar4 *>(out_rgba));
        renderer.render(out, make_info(info), *fd);
        track_renderer(owned, renderer);
        if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess)
            throw std::runtime_error("reference render failed on the device");
        out.download(reinterpret_cast<uchar4 *>(out_rgba));
        if (outs && info->mode != TIMEWARP)
        {
            export_view(outs[0], renderer.d_fwd_main_splatting_buffer, renderer.fwd2cam_ff, renderer.fwd2bwd_ff, fd->fwd->dims);
            export_view(outs[1], renderer.d_bwd_main_splatting_buffer, renderer.bwd2cam_ff, renderer.bwd2fwd_ff, fd->bwd->dims);
            for (int i = 0; i < frame->num_aux; i++)
            {
                export_view(outs[2 + 2 * i], renderer.d_aux_cam_splatting_buffers[i].forward, renderer.fwd2cam_aux_ff[i],
                            renderer.fwd2bwd_aux_ff[i], fd->aux_cam_images[i].curr->dims);
                export_view(outs[3 + 2 * i], renderer.d_aux_cam_splatting_buffers[i].backward, renderer.bwd2cam_aux_ff[i],
                            renderer.bwd2fwd_aux_ff[i], fd->aux_cam_images[i].next->dims);
            }
        }
    }
    catch (const std::exception &ex)
    {
        std::fprintf(stderr, "isti_refgpu_render: %s\n", ex.what());
        rc = -1;
    }
    cudaDeviceSynchronize();
    release(owned);
    return rc;
}

extern "C" int isti_refgpu_time(const oracle_frame *frame, const oracle_render_info *infos, int n_infos, int warmup, int repeats,
                                float *ms_out)
{
    int rc = 0;
    Owned owned;
    std::vector<cudaEvent_t> ev;
    try
    {
        if (n_infos < 1 || repeats < 1)
            throw std::runtime_error("n_infos and repeats must be positive");
        RendererHolder holder;
        Renderer &renderer = *holder.r;
        std::unique_ptr<FrameData> fd = make_frame(frame);
        track_frame(owned, *fd);
        ImageBuffer<uchar4, 4> out(make_uint2(infos[0].width, infos[0].height));
        track(owned, out);
        out.memsetBuffer(make_uchar4(0, 0, 0, 255));
        std::vector<RenderInfo> ri;
        for (int i = 0; i < n_infos; i++)
            ri.push_back(make_info(&infos[i]));
        for (int w = 0; w < warmup; w++)
            for (int i = 0; i < n_infos; i++)
                renderer.render(out, ri[i], *fd);
        const int n = repeats * n_infos;
        ev.resize(2 * (size_t)n, nullptr);
        for (auto &e : ev)
            if (cudaEventCreate(&e) != cudaSuccess)
                throw std::runtime_error("cudaEventCreate failed");
        for (int k = 0; k < repeats; k++)
            for (int i = 0; i < n_infos; i++)
            {
                const int j = k * n_infos + i;
                cudaEventRecord(ev[2 * j], 0);
                renderer.render(out, ri[i], *fd);
                cudaEventRecord(ev[2 * j + 1], 0);
            }
        if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess)
            throw std::runtime_error("reference render failed on the device");
        for (int j = 0; j < n; j++)
            cudaEventElapsedTime(&ms_out[j], ev[2 * j], ev[2 * j + 1]);
        track_renderer(owned, renderer);
    }
    catch (const std::exception &ex)
    {
        std::fprintf(stderr, "isti_refgpu_time: %s\n", ex.what());
        rc = -1;
    }
    cudaDeviceSynchronize();
    for (auto e : ev)
        if (e)
            cudaEventDestroy(e);
    release(owned);
    return rc;
}
