// isti_renderer.hpp — the reference's C++ interface over the C ABI of libisti.
//
// Same names and shapes as the reference's headers, so that its frame loop
// (src/main.cu) compiles against this header with the include swapped:
//   RenderMode, AdditionalRenderInfo, RenderInfo, Renderer   <- include/renderer.h:9-93
//   FrameImage, ZBufferImage, MotionZBufferImage, AuxCamData,
//   FrameData                                                <- include/data.h:12-116
//   ImageBuffer<T, N>                                        <- include/util/image_buffer.h:9-48
// Differences: images are dense device arrays instead of cudaArrays behind
// texture objects (reads outside an image return zero in both); matrices are
// isti::Mat4 (column-major, m[column][row] like glm::mat4, and constructible
// from a glm::mat4); Renderer::render takes an optional stream and does not
// block the host.
// Errors as in the reference: a failing CUDA call or render is printed to
// stdout and execution continues (CUDA_CHECK_THROW,
// include/util/cuda_helper_host.h:19-29); Renderer::last_status() holds the
// isti_status of the last render.  What the reference throws (a resize to
// another size, an unreadable image file, a size mismatch) throws here too, as
// isti::Error, a std::runtime_error.
// Header-only; link libisti.so and the CUDA runtime.
#pragma once

#include "isti.h"
#include "isti_dataset.h"
#include "isti_io.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace isti
{
class Error : public std::runtime_error
{
public:
    Error(isti_status s, const std::string &msg) : std::runtime_error(msg), status(s) {}
    isti_status status;
};

inline void check(isti_status s)
{
    if (s != ISTI_OK)
        throw Error(s, isti_last_error());
}

// Prints a failed CUDA call and carries on, like the reference's CUDA_CHECK_THROW.
inline bool check_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return true;
    std::cout << "CUDA | " << what << " failed with error: " << cudaGetErrorString(e) << std::endl;
    return false;
}

// 4x4 float matrix, column-major: m[c][r] is row r of column c (glm::mat4's layout).
struct Mat4
{
    float m[4][4] = {};
    Mat4() = default;
    template <class M, class = decltype(std::declval<const M &>()[0][0])>
    Mat4(const M &src) // any m[c][r]-indexable matrix: glm::mat4, float[4][4]
    {
        for (int c = 0; c < 4; c++)
            for (int r = 0; r < 4; r++)
                m[c][r] = static_cast<float>(src[c][r]);
    }
    float *operator[](int c) { return m[c]; }
    const float *operator[](int c) const { return m[c]; }
    const float *data() const { return &m[0][0]; }
};

// RenderMode, include/renderer.h:9-16
enum RenderMode
{
    OURS = ISTI_MODE_OURS,
    BACKWARD_BIDIRECTIONAL = ISTI_MODE_BACKWARD_BIDIRECTIONAL,
    BACKWARD_UNIDIRECTIONAL = ISTI_MODE_BACKWARD_UNIDIRECTIONAL,
    SPLATTING = ISTI_MODE_SPLATTING,
    TIMEWARP = ISTI_MODE_TIMEWARP
};

// include/renderer.h:18-35
struct AdditionalRenderInfo
{
    int frames_per_anchor;
    int shadow_frames_per_anchor;
    bool no_shadows;
    RenderMode mode;
};

struct RenderInfo
{
    uint2 resolution;
    float alpha;
    Mat4 viewproj_mat;
    Mat4 inv_viewproj_mat;
    AdditionalRenderInfo additional_info;
};

// ImageBuffer<T, N_CHANNELS> (include/util/image_buffer.h): one device image.  A
// buffer is allocated once; resizing it to another size throws, as in the
// reference.  New allocations are zero-filled.
template <typename T, int N_CHANNELS>
class ImageBuffer
{
public:
    ImageBuffer() = default;
    explicit ImageBuffer(uint2 resolution) { resize(resolution); }
    ~ImageBuffer() { cudaFree(_ptr); }
    ImageBuffer(const ImageBuffer &) = delete;
    ImageBuffer &operator=(const ImageBuffer &) = delete;
    ImageBuffer(ImageBuffer &&o) noexcept : _resolution(o._resolution), _ptr(o._ptr)
    {
        o._ptr = nullptr;
        o._resolution = make_uint2(0u, 0u);
    }

    void resize(uint2 resolution)
    {
        if (resolution.x == _resolution.x && resolution.y == _resolution.y)
            return;
        if (_resolution.x != 0 || _resolution.y != 0)
            throw std::runtime_error("Resizing of ImageBuffer currently not supported");
        _resolution = resolution;
        if (check_cuda(cudaMalloc(&_ptr, bytes()), "cudaMalloc (ImageBuffer::resize)"))
            check_cuda(cudaMemset(_ptr, 0, bytes()), "cudaMemset (ImageBuffer::resize)");
    }

    void memsetBuffer(T val)
    {
        std::vector<T> tmp(size_t(_resolution.x) * _resolution.y, val);
        upload(tmp.data());
    }
    void download(T *h_buffer) const
    {
        check_cuda(cudaMemcpy(h_buffer, _ptr, bytes(), cudaMemcpyDeviceToHost), "cudaMemcpy (ImageBuffer::download)");
    }
    void upload(const T *h_buffer) { check_cuda(cudaMemcpy(_ptr, h_buffer, bytes(), cudaMemcpyHostToDevice), "cudaMemcpy (ImageBuffer::upload)"); }

    // PNG into uchar4 images, EXR into float (one channel) or float4 (RGBA) images
    // (ImageBuffer::readFromFile, src/util/image_buffer.cu:103-178)
    void readFromFile(const std::filesystem::path &filename)
    {
        int32_t w = 0, h = 0, ch = 0;
        if (filename.extension() == ".exr")
        {
            float *px = nullptr;
            const isti_status s = isti_exr_decode_file(filename.string().c_str(), &w, &h, &ch, &px);
            if (s != ISTI_OK)
                throw Error(s, "Error loading EXR file " + filename.string() + ": " + isti_last_error());
            std::unique_ptr<void, decltype(&isti_image_free)> guard(px, isti_image_free);
            if (ch * (int)sizeof(float) != (int)sizeof(T))
                throw std::runtime_error("EXR channel count does not match the image type: " + filename.string());
            check_size(w, h, filename);
            upload(reinterpret_cast<const T *>(px));
        }
        else
        {
            uint8_t *px = nullptr;
            const isti_status s = isti_png_decode_file(filename.string().c_str(), &w, &h, &px);
            if (s != ISTI_OK)
                throw Error(s, "Could not load image " + filename.string() + " (" + isti_last_error() + ")");
            std::unique_ptr<void, decltype(&isti_image_free)> guard(px, isti_image_free);
            if (sizeof(T) != 4)
                throw std::runtime_error("PNG files load into 4-byte RGBA images: " + filename.string());
            check_size(w, h, filename);
            upload(reinterpret_cast<const T *>(px));
        }
    }

    // .png for 8-bit images (3 or 4 channels), .exr for float images (1 or 4
    // channels, no compression) (ImageBuffer::writeImageToFile,
    // src/util/image_buffer.cu:180-213; .bmp and .jpg are not written here)
    static void writeImageToFile(const std::vector<T> &image, int w, int h, int channels,
                                 const std::filesystem::path &filename)
    {
        const std::string path = filename.string();
        if (filename.extension() == ".png")
        {
            if (channels * sizeof(uint8_t) != sizeof(T) && !(channels == 3 && sizeof(T) == 4))
                throw std::runtime_error("PNG files hold 8-bit RGB or RGBA images: " + path);
            if (channels == 3) // RGBA8 buffer written as RGB: drop alpha
            {
                std::vector<uint8_t> rgb(size_t(w) * h * 3);
                const uint8_t *src = reinterpret_cast<const uint8_t *>(image.data());
                for (size_t i = 0; i < size_t(w) * h; i++)
                    std::memcpy(&rgb[i * 3], src + i * 4, 3);
                check(isti_png_encode_file(path.c_str(), w, h, 3, rgb.data()));
            }
            else
                check(isti_png_encode_file(path.c_str(), w, h, 4, reinterpret_cast<const uint8_t *>(image.data())));
        }
        else if (filename.extension() == ".exr")
        {
            if (channels * sizeof(float) != sizeof(T) || (channels != 1 && channels != 4))
                throw std::runtime_error("EXR files are written from float or float4 images: " + path);
            check(isti_exr_encode_file(path.c_str(), w, h, channels, reinterpret_cast<const float *>(image.data()), 0));
        }
        else
            throw std::runtime_error("Image file extension not supported!");
    }

    void writeToFile(const std::filesystem::path &filename) const
    {
        std::vector<T> image(size_t(_resolution.x) * _resolution.y);
        download(image.data());
        writeImageToFile(image, int(_resolution.x), int(_resolution.y), N_CHANNELS, filename);
    }

    // Mean of a float image, T() for other types (ImageBuffer::average,
    // src/util/image_buffer.cu:74-101).  Summed in double on the host; the
    // reference's float atomics give an order-dependent last bit.
    T average() const
    {
        if constexpr (!std::is_same_v<T, float>)
            return T();
        else
        {
            std::vector<float> image(size_t(_resolution.x) * _resolution.y);
            download(image.data());
            double s = 0.0;
            for (float v : image)
                s += v;
            return image.empty() ? 0.0f : float(s / double(image.size()));
        }
    }

    uint2 resolution() const { return _resolution; }
    T *ptr() { return _ptr; }
    const T *ptr() const { return _ptr; }

private:
    static size_t bytes_for(uint2 r) { return size_t(r.x) * r.y * sizeof(T); }
    size_t bytes() const { return bytes_for(_resolution); }
    void check_size(int32_t w, int32_t h, const std::filesystem::path &f) const
    {
        if (uint32_t(w) != _resolution.x || uint32_t(h) != _resolution.y)
            throw std::runtime_error("Image resolution has to be set in advance: " + f.string());
    }
    uint2 _resolution = make_uint2(0u, 0u);
    T *_ptr = nullptr;
};

// include/data.h:12-62
struct FrameImage
{
    ImageBuffer<uchar4, 4> img;
    std::optional<ImageBuffer<uchar4, 4>> shadowColorA_img = std::make_optional<ImageBuffer<uchar4, 4>>();
    std::optional<ImageBuffer<uchar4, 4>> shadowColorB_img = std::make_optional<ImageBuffer<uchar4, 4>>();
    std::optional<ImageBuffer<uchar4, 4>> shadowInfo_img = std::make_optional<ImageBuffer<uchar4, 4>>();
    uint2 dims = make_uint2(0u, 0u);
    float t = 0.0f;
    Mat4 view_mat, proj_mat, viewproj_mat, inv_viewproj_mat;

    void resize(uint2 d)
    {
        if (shadowColorA_img.has_value())
            shadowColorA_img->resize(d);
        if (shadowColorB_img.has_value())
            shadowColorB_img->resize(d);
        if (shadowInfo_img.has_value())
            shadowInfo_img->resize(d);
        img.resize(d);
        dims = d;
    }
};

struct ZBufferImage : public FrameImage
{
    ImageBuffer<float, 1> z_buffer;
    void resize(uint2 d)
    {
        z_buffer.resize(d);
        FrameImage::resize(d);
    }
};

struct MotionZBufferImage : public ZBufferImage
{
    std::optional<ImageBuffer<float4, 4>> object_motion = std::make_optional<ImageBuffer<float4, 4>>();
    void resize(uint2 d)
    {
        if (object_motion.has_value())
        {
            object_motion->resize(d);
            object_motion->memsetBuffer(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        }
        ZBufferImage::resize(d);
    }
};

struct AuxCamData
{
    AuxCamData() : curr(std::make_unique<MotionZBufferImage>()), next(std::make_unique<MotionZBufferImage>()) {}
    void swap() { std::swap(curr, next); }
    std::unique_ptr<MotionZBufferImage> curr, next;
    int priority = 0;
};

struct FrameData
{
    explicit FrameData(uint8_t number_of_aux_cams)
        : fwd(std::make_unique<MotionZBufferImage>()), bwd(std::make_unique<MotionZBufferImage>()), aux_cam_images(number_of_aux_cams)
    {
    }
    std::unique_ptr<MotionZBufferImage> fwd;
    std::unique_ptr<MotionZBufferImage> bwd;
    std::vector<AuxCamData> aux_cam_images;
    std::vector<ZBufferImage> depth_imgs; // carried like the reference's; the renderer does not read it

    void resize(uint2 main_dims, const std::vector<uint2> &aux_res, const std::vector<int> &aux_priorities)
    {
        fwd->resize(main_dims);
        bwd->resize(main_dims);
        for (size_t i = 0; i < aux_cam_images.size(); i++)
        {
            aux_cam_images[i].curr->resize(aux_res[i]);
            aux_cam_images[i].next->resize(aux_res[i]);
            aux_cam_images[i].priority = aux_priorities[i];
        }
        for (ZBufferImage &d : depth_imgs)
            d.resize(main_dims);
    }
    void swap()
    {
        std::swap(fwd, bwd);
        for (AuxCamData &a : aux_cam_images)
            a.swap();
    }
};

// Renderer (include/renderer.h:52-93) on isti_render.
class Renderer
{
public:
    Renderer() { report(isti_renderer_create(&_r), "isti_renderer_create"); }
    ~Renderer() { isti_renderer_destroy(_r); }
    Renderer(const Renderer &) = delete;
    Renderer &operator=(const Renderer &) = delete;

    void render(ImageBuffer<uchar4, 4> &render_buffer, const RenderInfo render_info, const FrameData &frame_data,
                cudaStream_t stream = nullptr)
    {
        isti_render_info info{};
        info.width = render_info.resolution.x;
        info.height = render_info.resolution.y;
        info.alpha = render_info.alpha;
        std::memcpy(info.viewproj, render_info.viewproj_mat.data(), sizeof info.viewproj);
        std::memcpy(info.inv_viewproj, render_info.inv_viewproj_mat.data(), sizeof info.inv_viewproj);
        info.frames_per_anchor = render_info.additional_info.frames_per_anchor;
        info.shadow_frames_per_anchor = render_info.additional_info.shadow_frames_per_anchor;
        info.no_shadows = render_info.additional_info.no_shadows ? 1 : 0;
        info.mode = render_info.additional_info.mode;
        const size_t n_aux = frame_data.aux_cam_images.size();
        _curr.resize(n_aux);
        _next.resize(n_aux);
        _prio.resize(n_aux);
        for (size_t i = 0; i < n_aux; i++)
        {
            _curr[i] = view_of(*frame_data.aux_cam_images[i].curr);
            _next[i] = view_of(*frame_data.aux_cam_images[i].next);
            _prio[i] = frame_data.aux_cam_images[i].priority;
        }
        isti_frame_data fd{};
        fd.fwd = view_of(*frame_data.fwd);
        fd.bwd = view_of(*frame_data.bwd);
        fd.num_aux = int32_t(n_aux);
        fd.aux_curr = n_aux ? _curr.data() : nullptr;
        fd.aux_next = n_aux ? _next.data() : nullptr;
        fd.aux_priority = n_aux ? _prio.data() : nullptr;
        if (_r)
            report(isti_render(_r, render_buffer.ptr(), &info, &fd, stream), "Renderer::render");
        else
            report(ISTI_ERR_INVALID_ARG, "Renderer::render", "the renderer was not created");
    }

    // isti_status of the last render (or of the construction, before the first render)
    isti_status last_status() const { return _status; }
    isti_renderer *handle() { return _r; }

    // isti_renderer_set_autotune (no counterpart in the reference): the first uncaptured
    // render of each shape class times the reprojection's candidate launches; the output
    // does not depend on it.
    void setAutotune(bool on)
    {
        if (_r)
            report(isti_renderer_set_autotune(_r, on ? 1 : 0), "Renderer::setAutotune");
    }

    // isti_renderer_set_reproj_launch (no counterpart in the reference): pins the
    // reprojection launch (register cap, row pairs per block, plain-load key tiles; 0: the
    // rule's); the output does not depend on it.
    void setReprojLaunch(int regs, int row_pairs, bool plain_tiles)
    {
        if (_r)
            report(isti_renderer_set_reproj_launch(_r, regs, row_pairs, plain_tiles ? 1 : 0), "Renderer::setReprojLaunch");
    }

private:
    void report(isti_status s, const char *what, const char *msg = nullptr)
    {
        _status = s;
        if (s != ISTI_OK)
            std::cout << "isti | " << what << " failed with error: " << (msg ? msg : isti_last_error()) << std::endl;
    }
    template <class B>
    static const void *ptr_of(const std::optional<B> &b)
    {
        return b.has_value() && b->resolution().x != 0 ? static_cast<const void *>(b->ptr()) : nullptr;
    }
    static isti_view view_of(const MotionZBufferImage &im)
    {
        isti_view v{};
        v.width = im.dims.x;
        v.height = im.dims.y;
        v.color = im.img.ptr();
        v.z = im.z_buffer.ptr();
        v.motion = ptr_of(im.object_motion);
        v.motion_format = v.motion ? ISTI_MOTION_F32X4 : ISTI_MOTION_NONE;
        v.shadow_color_a = ptr_of(im.shadowColorA_img);
        v.shadow_color_b = ptr_of(im.shadowColorB_img);
        v.shadow_info = ptr_of(im.shadowInfo_img);
        if (!v.shadow_info) // soft shadows need the level field (src/renderer.cu:241-277)
            v.shadow_color_a = v.shadow_color_b = nullptr;
        std::memcpy(v.viewproj, im.viewproj_mat.data(), sizeof v.viewproj);
        std::memcpy(v.inv_viewproj, im.inv_viewproj_mat.data(), sizeof v.inv_viewproj);
        return v;
    }
    isti_renderer *_r = nullptr;
    isti_status _status = ISTI_OK;
    std::vector<isti_view> _curr, _next;
    std::vector<int32_t> _prio;
};

// Host side of isti_unpack_shadows (include/isti_dataset.h; no counterpart in the reference):
// the sparse entries of one view's shadow info, colour A and colour B images (host pixels,
// `ch_*` bytes per pixel, at least 3, R G B first).  One ISTI_SHADOW_ENTRY_BYTES entry per
// pixel whose info R, G or B is non-zero: index (uint32 little-endian), info RGB, A RGB,
// B RGB, 3 zero bytes.
inline std::vector<uint8_t> pack_shadow_entries(const uint8_t *info, int ch_info, const uint8_t *a, int ch_a, const uint8_t *b, int ch_b,
                                                uint32_t n_pixels)
{
    if (!info || !a || !b || ch_info < 3 || ch_a < 3 || ch_b < 3)
        throw Error(ISTI_ERR_INVALID_ARG, "pack_shadow_entries: three images of at least 3 channels");
    std::vector<uint8_t> out;
    for (uint32_t i = 0; i < n_pixels; i++)
    {
        const uint8_t *pi = info + (size_t)i * ch_info;
        if (!(pi[0] | pi[1] | pi[2]))
            continue;
        const uint8_t *pa = a + (size_t)i * ch_a, *pb = b + (size_t)i * ch_b;
        const uint8_t e[ISTI_SHADOW_ENTRY_BYTES] = {(uint8_t)i, (uint8_t)(i >> 8), (uint8_t)(i >> 16), (uint8_t)(i >> 24),
                                                    pi[0], pi[1], pi[2], pa[0], pa[1], pa[2], pb[0], pb[1], pb[2], 0, 0, 0};
        out.insert(out.end(), e, e + ISTI_SHADOW_ENTRY_BYTES);
    }
    return out;
}
} // namespace isti
