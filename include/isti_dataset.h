/*
 * isti_dataset — the reference's on-disk keyframe format, loaded into device
 * buffers that isti_render consumes directly.
 *
 * Replaces FrameFileReader (include/file_reader.h:9-67, src/file_reader.cu)
 * and the FrameData double buffer it fills (include/data.h:79-116):
 *
 *   isti_camera_path_open   <- FrameFileReader::initCamInfo (file_reader.cu:78-107):
 *                              <dir>/cam.json with "frames" [{idx, w2c, proj}],
 *                              "resolution" {x, y}, clientFps (60), serverFps (10),
 *                              shadowFps (60), objectMotion (true),
 *                              shadowGradients (true); matrices as e<row><col>.
 *   isti_dataset_open       <- FrameFileReader::init (:109-136): main camera in
 *                              <input>/main, aux camera i in <input>/<aux_dirs[i]>;
 *                              keyframe 0 is loaded into the "bwd" slot.
 *   isti_dataset_read_next  <- FrameFileReader::readNextFrame (:167-217): swaps
 *                              fwd/bwd (and aux curr/next), then, unless the
 *                              sequence is exhausted, loads the next keyframe's
 *                              colour + depth into bwd / aux next and the flow
 *                              fields and shadow images of the pair from the
 *                              "forward..." and "backward..." folders; a folder
 *                              that does not exist makes that buffer absent.
 *   isti_dataset_frame      <- the FrameData handed to Renderer::render
 *                              (src/main.cu:177): device views of the pair.
 *   isti_depth_to_z         <- convertDepthToZ_kernel (file_reader.cu:17-37) with
 *                              the reader's settings (reversed z, [0,1] depth,
 *                              right-handed): z = 2 (1 - d) - 1.
 *   isti_normalize_proj     <- FrameFileReader::normalizeProjMat (:218-229).
 *
 * File layout per camera folder: color/NNNN.png (RGBA8), depth/NNNN.exr
 * (one float channel), forwardFlowField/ and backwardFlowField/NNNN.exr
 * (RGBA float: NDC motion), forwardShadowColorA|B|Info/ and
 * backwardShadowColorA|B|Info/NNNN.png, NNNN = the frame's idx, 4 digits.
 *
 * Differences from the reference: buffers that the reference allocates but
 * leaves unwritten until the first read_next (the "fwd" slot and the shadow
 * images) start as zeros; every image must have the camera's resolution, depth
 * files must hold one channel and flow files four (the reference reads out of
 * bounds otherwise); loading is synchronous and returns errors instead of
 * throwing.  Files are decoded on several host threads.
 */
#ifndef ISTI_DATASET_H
#define ISTI_DATASET_H

#include "isti.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct isti_camera_path isti_camera_path;
typedef struct isti_dataset isti_dataset;

/* CameraInfo (include/file_reader.h:18-26) */
typedef struct isti_camera_info
{
    int32_t width, height;
    int32_t client_fps, server_fps, shadow_fps;
    int32_t priority; /* objectMotion * 2 + shadowGradients */
    int32_t n_frames;
} isti_camera_info;

/* FrameInfo (include/file_reader.h:11-16); matrices column-major as read */
typedef struct isti_camera_frame
{
    int32_t idx;
    float w2c[16];
    float proj[16];
} isti_camera_frame;

isti_status isti_camera_path_open(const char *dir, isti_camera_path **out);
isti_status isti_camera_path_info(const isti_camera_path *p, isti_camera_info *info);
isti_status isti_camera_path_frame(const isti_camera_path *p, int32_t i, isti_camera_frame *frame);
void isti_camera_path_close(isti_camera_path *p);

/* Loads keyframe 0 (synchronously; `stream` orders the device work). */
isti_status isti_dataset_open(const char *input_dir, int32_t n_aux, const char *const *aux_dirs, void *stream,
                              isti_dataset **out);
/* *advanced = 1 when a new keyframe was loaded, 0 when the sequence is exhausted
 * (the slots are swapped either way, as in the reference). */
isti_status isti_dataset_read_next(isti_dataset *d, int32_t *advanced);
/* Device views of the current pair; pointers stay valid until the next
 * read_next or close. */
isti_status isti_dataset_frame(isti_dataset *d, isti_frame_data *frame);
/* camera = -1 for the main camera, else the aux index */
isti_status isti_dataset_camera(const isti_dataset *d, int32_t camera, isti_camera_info *info);
/* Keyframe matrices of the main camera in slot 0 (fwd) or 1 (bwd): the view
 * (w2c) and the normalised projection; zeros for a slot never loaded. */
isti_status isti_dataset_matrices(const isti_dataset *d, int32_t slot, float view[16], float proj[16]);
/* Index of the keyframe in the bwd slot (0 after open). */
int32_t isti_dataset_keyframe(const isti_dataset *d);
void isti_dataset_close(isti_dataset *d);

isti_status isti_depth_to_z(float *depth, int32_t width, int32_t height, void *stream);
isti_status isti_normalize_proj(const float proj[16], float out[16]);

/* Packed RGB8 (3 bytes per pixel, device) -> the RGBA8 image the renderer reads
 * (device, 4-byte aligned), alpha 255 (stb_image's fill for images without
 * alpha).  No counterpart in the reference, which uploads RGBA: the renderer
 * never reads the alpha bytes of shadow colour A/B and shadow info images, so a
 * caller bound by the host link can upload those as RGB (3/4 of the bytes) and
 * expand them on the device.  dst and src must not overlap. */
isti_status isti_rgb8_to_rgba8(void *dst_rgba, const void *src_rgb, size_t n_pixels, void *stream);

/* Sparse shadow images (no counterpart in the reference, whose loader reads dense PNGs).
 * The renderer reads a view's shadow info, colour A and colour B images only at pixels whose
 * shadow-info field (R, G, B) is non-zero, and reads no alpha byte of them (src/renderer.cu
 * :217-295).  A caller bound by the host link can therefore send just those pixels: each
 * entry is 16 bytes -- the pixel index (uint32, little-endian), info R G B, colour A R G B,
 * colour B R G B, 3 bytes of padding (ISTI_SHADOW_ENTRY_BYTES).  isti_unpack_shadows writes
 * the three RGBA8 images of n_pixels (device, 16-byte aligned, not overlapping the entries)
 * on `stream`: zero everywhere, then each listed pixel's colours with alpha 255.  Entries
 * whose index is not below n_pixels are skipped.  Rendering with the unpacked images gives
 * the same frames as with the dense ones.
 *
 * clear_entries: NULL, or the entries of the previous unpack into the same three images
 * (which are then zero everywhere else): only their pixels are cleared instead of the whole
 * images, which saves 12 bytes of device writes per pixel. */
#define ISTI_SHADOW_ENTRY_BYTES 16
isti_status isti_unpack_shadows(void *info_rgba, void *a_rgba, void *b_rgba, size_t n_pixels, const void *entries, size_t n_entries,
                                const void *clear_entries, size_t n_clear, void *stream);

/* Host matrix helpers of the frame loop (src/main.cu:26-28,161,176), the glm
 * operations the reference applies: out = a * b, out = inverse(m), and
 * glm::interpolate(m1, m2, t). */
void isti_mat4_mul(const float a[16], const float b[16], float out[16]);
void isti_mat4_inverse(const float m[16], float out[16]);
void isti_mat4_interpolate(const float m1[16], const float m2[16], float t, float out[16]);

#ifdef __cplusplus
}
#endif

#endif /* ISTI_DATASET_H */
