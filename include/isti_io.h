/*
 * isti_io — image files of the reference's dataset format, decoded on the host.
 *
 * The reference reads keyframe images with ImageBuffer::readFromFile
 * (src/util/image_buffer.cu:103-178): PNG through fpng or stb_image, always
 * expanded to 4 channels of 8 bits, and EXR through tinyexr's LoadEXR; it
 * writes client frames with ImageBuffer::writeToFile (:180-200, PNG through
 * fpng).  These entry points replace those third-party calls with codecs
 * written for this library:
 *
 *   isti_png_decode_file  <- fpng_decode_file(..., 4) / stbi_load(..., 4)
 *                            (image_buffer.cu:144-165): RGBA8 result with
 *                            stb_image's conversions (grey -> RGB, missing
 *                            alpha = 255, tRNS colour key and palette alpha,
 *                            16-bit samples keep their high byte, 1/2/4-bit
 *                            grey scaled to 0..255, Adam7 interlace).
 *   isti_exr_decode_file  <- LoadEXR (image_buffer.cu:112): a file with one
 *                            channel gives one float per pixel; otherwise R, G
 *                            and B must be among its first four channels and
 *                            the result is RGBA float (A = 1 when absent).
 *                            HALF samples are widened exactly; scan-line files
 *                            with NONE, RLE, ZIPS, ZIP or PIZ compression.
 *   isti_png_encode_file  <- fpng_encode_image_to_file (image_buffer.cu:185).
 *
 * Differences from the reference's libraries: tiled, multi-part, deep and
 * PXR24/B44/DWA-compressed EXR files return ISTI_ERR_UNSUPPORTED, and the
 * zlib checksum of PNG and EXR data is verified (stb_image skips it).
 * Decoded buffers are allocated with malloc; release them with
 * isti_image_free.  Errors set isti_last_error().
 */
#ifndef ISTI_IO_H
#define ISTI_IO_H

#include "isti.h"

#ifdef __cplusplus
extern "C" {
#endif

isti_status isti_png_decode_file(const char *path, int32_t *width, int32_t *height, uint8_t **rgba);
isti_status isti_png_decode_memory(const uint8_t *data, size_t size, int32_t *width, int32_t *height,
                                   uint8_t **rgba);

/* channels is 3 (RGB) or 4 (RGBA), 8 bits per sample, rows top to bottom. */
isti_status isti_png_encode_file(const char *path, int32_t width, int32_t height, int32_t channels,
                                 const uint8_t *pixels);
isti_status isti_png_encode_memory(int32_t width, int32_t height, int32_t channels, const uint8_t *pixels,
                                   uint8_t **png, size_t *png_size);

/* *channels receives 1 or 4 (the float values per pixel in *data). */
isti_status isti_exr_decode_file(const char *path, int32_t *width, int32_t *height, int32_t *channels,
                                 float **data);
isti_status isti_exr_decode_memory(const uint8_t *bytes, size_t size, int32_t *width, int32_t *height,
                                   int32_t *channels, float **data);

/* Scan-line EXR of FLOAT samples, the counterpart of ImageBuffer::writeToFile
 * for float buffers (image_buffer.cu:195-200, SaveEXR): channels 1 (written
 * as "Y") or 4 (RGBA, written as A, B, G, R); compression 0 = NONE, 3 = ZIP. */
isti_status isti_exr_encode_file(const char *path, int32_t width, int32_t height, int32_t channels, const float *data,
                                 int32_t compression);

/* zlib (RFC 1950) stream -> bytes; the building block of both decoders. */
isti_status isti_zlib_decompress(const uint8_t *src, size_t src_size, uint8_t **out, size_t *out_size);

void isti_image_free(void *p);

#ifdef __cplusplus
}
#endif

#endif /* ISTI_IO_H */
