// TEST INFRASTRUCTURE: the reference's own image libraries, compiled for the
// CPU (oracle/build_ref.py, only where the reference tree exists).
//
// src/util/image_buffer.cu:8-17 includes the vendored stb_image,
// stb_image_write and tinyexr headers (dependencies/) with these
// configuration macros; ImageBuffer::readFromFile (:103-178) then calls
// stbi_load(..., 4) and LoadEXR.  The functions below expose exactly those
// calls (plus tinyexr's writer, to produce EXR test files in every
// compression) so the decoders of libisti can be checked against them.
#define STB_IMAGE_IMPLEMENTATION
#define STB_IMAGE_WRITE_IMPLEMENTATION
#include <stb_image.h>
#include <stb_image_write.h>

#define TINYEXR_USE_MINIZ 0
#define TINYEXR_USE_STB_ZLIB 1
#define TINYEXR_USE_THREAD 1
#define TINYEXR_IMPLEMENTATION
#include <tinyexr.h>

#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

extern "C" {

// stbi_load(path, ..., 4): RGBA8, as ImageBuffer::readFromFile for PNG files
// fpng does not recognise (image_buffer.cu:144-149).
int ref_png_load(const char *path, int *w, int *h, unsigned char **rgba)
{
    int comp = 0;
    *rgba = stbi_load(path, w, h, &comp, 4);
    return *rgba ? 0 : -1;
}

const char *ref_png_failure(void) { return stbi_failure_reason(); }

// LoadEXR(path) (image_buffer.cu:112).  *channels = floats per pixel of the
// result: 1 when the default layer holds one channel, else 4.
int ref_exr_load(const char *path, int *w, int *h, int *channels, float **data, char *err_buf, int err_len)
{
    const char *err = nullptr;
    float *out = nullptr;
    const int ret = LoadEXR(&out, w, h, path, &err);
    if (ret != TINYEXR_SUCCESS)
    {
        if (err_buf && err_len > 0)
        {
            std::strncpy(err_buf, err ? err : "LoadEXR failed", size_t(err_len) - 1);
            err_buf[err_len - 1] = 0;
        }
        if (err)
            FreeEXRErrorMessage(err);
        return ret;
    }
    // channel count of the default layer, as LoadEXR decided it
    EXRVersion version;
    EXRHeader header;
    InitEXRHeader(&header);
    ParseEXRVersionFromFile(&version, path);
    ParseEXRHeaderFromFile(&header, &version, path, &err);
    int n = 0;
    for (int c = 0; c < header.num_channels; c++)
    {
        const std::string name(header.channels[c].name);
        const size_t pos = name.find_last_of('.');
        if (pos != std::string::npos && pos != 0)
            continue;
        n++;
    }
    FreeEXRHeader(&header);
    *channels = n == 1 ? 1 : 4;
    *data = out;
    return 0;
}

// SaveEXRImageToFile with explicit channel names, pixel types and
// compression.  `planar` holds n_channels planes of w*h floats in the order
// of `names` (comma-separated); pixel_type 1 = HALF, 2 = FLOAT.
int ref_exr_save(const char *path, int w, int h, int n_channels, const char *names, int pixel_type, int compression,
                 const float *planar)
{
    std::vector<std::string> nm;
    {
        std::string s(names), cur;
        for (char c : s)
        {
            if (c == ',')
            {
                nm.push_back(cur);
                cur.clear();
            }
            else
                cur += c;
        }
        nm.push_back(cur);
    }
    if (int(nm.size()) != n_channels)
        return -100;
    EXRHeader header;
    InitEXRHeader(&header);
    EXRImage image;
    InitEXRImage(&image);
    std::vector<float *> planes;
    for (int c = 0; c < n_channels; c++)
        planes.push_back(const_cast<float *>(planar) + size_t(c) * size_t(w) * size_t(h));
    image.images = reinterpret_cast<unsigned char **>(planes.data());
    image.width = w;
    image.height = h;
    image.num_channels = n_channels;
    header.num_channels = n_channels;
    header.compression_type = compression;
    header.channels = static_cast<EXRChannelInfo *>(std::calloc(size_t(n_channels), sizeof(EXRChannelInfo)));
    header.pixel_types = static_cast<int *>(std::malloc(sizeof(int) * size_t(n_channels)));
    header.requested_pixel_types = static_cast<int *>(std::malloc(sizeof(int) * size_t(n_channels)));
    for (int c = 0; c < n_channels; c++)
    {
        std::strncpy(header.channels[c].name, nm[size_t(c)].c_str(), 255);
        header.pixel_types[c] = TINYEXR_PIXELTYPE_FLOAT;
        header.requested_pixel_types[c] = pixel_type;
    }
    const char *err = nullptr;
    const int ret = SaveEXRImageToFile(&image, &header, path, &err);
    if (err)
        FreeEXRErrorMessage(err);
    std::free(header.channels);
    std::free(header.pixel_types);
    std::free(header.requested_pixel_types);
    return ret;
}

// stbi_write_png (8-bit, 1-4 channels).
int ref_png_save(const char *path, int w, int h, int comp, const unsigned char *data)
{
    return stbi_write_png(path, w, h, comp, data, w * comp) ? 0 : -1;
}

void ref_free(void *p) { std::free(p); }

} // extern "C"
