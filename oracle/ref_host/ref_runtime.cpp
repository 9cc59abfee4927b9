// Host emulation of the CUDA runtime calls and of ImageBuffer<T,N>
// (reference include/util/image_buffer.h:9-48) for the CPU build of the
// reference renderer.  Test infrastructure only.
//
// ImageBuffer semantics kept from src/util/image_buffer.cu:
//  * resize() allocates once and throws on a size change (:38-51);
//  * textures/surfaces address the same storage, border reads return zero;
//  * memsetBuffer() fills every texel with one value (:61-65);
//  * upload()/download() copy a dense host image (:68-78);
//  * average() sums the float image and divides by the pixel count (:80-100);
//    the device version uses a per-pixel float atomicAdd whose order is not
//    defined, here the order is row-major.
// File I/O is not emulated (disk formats are outside the oracle's scope).
#include "isti_refhost.h"

#include "util/image_buffer.h"

#include <cstdlib>
#include <mutex>

namespace isti_refhost
{
namespace
{
std::vector<Image> &registry()
{
    static std::vector<Image> r;
    return r;
}
std::vector<void *> &allocations()
{
    static std::vector<void *> a;
    return a;
}
void *tracked_alloc(size_t bytes)
{
    void *p = std::calloc(bytes ? bytes : 1, 1);
    if (!p)
        throw std::bad_alloc();
    allocations().push_back(p);
    return p;
}
} // namespace

const Image &image(unsigned long long handle)
{
    if (handle == 0 || handle > registry().size())
        throw std::runtime_error("invalid texture/surface handle");
    return registry()[handle - 1];
}

unsigned long long register_image(void *ptr, unsigned w, unsigned h, size_t elem)
{
    registry().push_back(Image{ptr, w, h, elem});
    return registry().size();
}

// Frees every emulated allocation and forgets all texture handles.
void reset_all()
{
    for (void *p : allocations())
        std::free(p);
    allocations().clear();
    registry().clear();
}
} // namespace isti_refhost

extern "C"
{
cudaError_t cudaMalloc(void **devPtr, size_t size)
{
    *devPtr = isti_refhost::tracked_alloc(size);
    return cudaSuccess;
}
cudaError_t cudaFree(void *) { return cudaSuccess; } // released by reset_all()
cudaError_t cudaMemset(void *devPtr, int value, size_t count)
{
    std::memset(devPtr, value, count);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void *dst, const void *src, size_t count, enum cudaMemcpyKind)
{
    if (count)
        std::memcpy(dst, src, count);
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t) { return "emulated"; }
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::resize(uint2 resolution)
{
    if (resolution.x == _resolution.x && resolution.y == _resolution.y)
        return;
    else if (_resolution.x != 0 || _resolution.y != 0)
        throw std::runtime_error("Resizing of ImageBuffer currently not supported");
    _resolution = resolution;
    _array = reinterpret_cast<cudaArray_t>(isti_refhost::tracked_alloc(sizeof(T) * resolution.x * resolution.y));
    init();
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::init(cudaTextureAddressMode)
{
    _surface = createSurface();
    _texture = createTexture(cudaFilterModePoint, cudaAddressModeBorder);
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::memsetBuffer(T val)
{
    T *p = reinterpret_cast<T *>(_array);
    for (size_t i = 0; i < (size_t)_resolution.x * _resolution.y; i++)
        p[i] = val;
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::download(T *h_buffer)
{
    std::memcpy(h_buffer, reinterpret_cast<T *>(_array), sizeof(T) * _resolution.x * _resolution.y);
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::upload(T *h_buffer)
{
    std::memcpy(reinterpret_cast<T *>(_array), h_buffer, sizeof(T) * _resolution.x * _resolution.y);
}

template <typename T, int N_CHANNELS>
T ImageBuffer<T, N_CHANNELS>::average()
{
    T tmp = T();
    if constexpr (!std::is_same_v<T, float>)
    {
        return tmp;
    }
    else
    {
        const float *p = reinterpret_cast<const float *>(_array);
        float acc = 0.0f;
        for (size_t i = 0; i < (size_t)_resolution.x * _resolution.y; i++)
            acc += p[i];
        acc /= (_resolution.x * _resolution.y);
        return (T)acc;
    }
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::readFromFile(std::filesystem::path)
{
    throw std::runtime_error("file input is not emulated");
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::writeImageToFile(std::vector<T> &, int, int, int, std::filesystem::path)
{
    throw std::runtime_error("file output is not emulated");
}

template <typename T, int N_CHANNELS>
void ImageBuffer<T, N_CHANNELS>::writeToFile(std::filesystem::path)
{
    throw std::runtime_error("file output is not emulated");
}

template <typename T, int N_CHANNELS>
cudaTextureObject_t ImageBuffer<T, N_CHANNELS>::createTexture(cudaTextureFilterMode, cudaTextureAddressMode)
{
    return isti_refhost::register_image(reinterpret_cast<void *>(_array), _resolution.x, _resolution.y, sizeof(T));
}

template <typename T, int N_CHANNELS>
cudaSurfaceObject_t ImageBuffer<T, N_CHANNELS>::createSurface()
{
    return isti_refhost::register_image(reinterpret_cast<void *>(_array), _resolution.x, _resolution.y, sizeof(T));
}

template struct ImageBuffer<uchar4, 4>;
template struct ImageBuffer<float, 1>;
template struct ImageBuffer<float4, 4>;
