/*
 * isti_metrics — image quality of interpolated frames on the GPU.
 *
 * Replaces the per-image metrics of the reference's offline evaluation
 * (scripts/eval.py:66-132), which loads both PNGs as RGB float in [0, 1]
 * (alpha dropped, eval.py:55-57) and computes
 *   PSNR = -10 log10(MSE)                         (eval.py:68, F.mse_loss)
 *   SSIM = mean of the SSIM map, 11x11 Gaussian window, sigma 1.5, zero
 *          padding, C1 = 0.01^2, C2 = 0.03^2, per channel (scripts/loss_utils.py:17-57)
 * for each frame against its ground truth, and LDR-FLIP (scripts/flip_loss.py,
 * isti_flip_rgba8 below).
 *
 * One fused kernel reads both RGBA8 images once: per 32x16 tile it stages the
 * tile and its 5-pixel halo in shared memory, filters the five SSIM moments
 * separably and accumulates the squared error exactly in integers; a second
 * one-block kernel adds the per-tile partial sums in a fixed order, so the
 * result is deterministic.  Both run on `stream`; the result is written to
 * device memory and nothing blocks the host.
 *
 * Numerics: the squared error is summed exactly (integers), MSE = sum /
 * (3 * width * height * 255^2) in double; SSIM per pixel in float32 like the
 * reference, summed in double.  Agreement with eval.py is within 1e-5 (SSIM)
 * and 1e-4 dB (PSNR); the reference's own torch results depend on its
 * convolution algorithm at the 1e-7 level.
 */
#ifndef ISTI_METRICS_H
#define ISTI_METRICS_H

#include "isti.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct isti_quality
{
    double mse;  /* mean squared error of RGB in [0, 1] */
    double psnr; /* dB; +inf for identical images */
    double ssim;
} isti_quality;

/* Device scratch the metric kernels need for an image of this size. */
size_t isti_quality_scratch_bytes(int32_t width, int32_t height);

/* a, b: device RGBA8 images of width*height pixels (4-byte aligned, dense
 * rows); scratch: isti_quality_scratch_bytes(width, height) device bytes;
 * out: device pointer to one isti_quality. */
isti_status isti_quality_rgba8(const void *a, const void *b, int32_t width, int32_t height, void *scratch,
                               isti_quality *out, void *stream);

/* LDR-FLIP (scripts/flip_loss.py, LDRFLIPLoss; eval.py's flip_fn(render,
 * ground_truth)): `test` is the rendered frame, `reference` the ground truth,
 * both device RGBA8 (alpha ignored).  pixels_per_degree = the observer's
 * pixels per degree of visual angle (eval.py: 0.7 m wide 4K screen at 0.7 m,
 * 3840 * pi / 180 = 67.02); the filters must fit in ISTI_FLIP_MAX_RADIUS
 * pixels (pixels_per_degree <= 118).  One tile kernel stages both images as
 * YCxCz with a replicate-padded halo, applies the contrast-sensitivity filters
 * and the edge / point detectors separably (the reference's 2-D kernels
 * factor exactly), and reduces in a fixed order.  *out_mean (device double)
 * receives the mean FLIP; out_map (device float, width*height) the per-pixel
 * values, or NULL. */
#define ISTI_FLIP_MAX_RADIUS 16
size_t isti_flip_scratch_bytes(int32_t width, int32_t height);
isti_status isti_flip_rgba8(const void *test, const void *reference, int32_t width, int32_t height, float pixels_per_degree,
                            void *scratch, double *out_mean, float *out_map, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ISTI_METRICS_H */
