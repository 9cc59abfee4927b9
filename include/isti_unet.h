/*
 * isti_unet — the learned flow initialiser (no counterpart in the reference, whose
 * renderer starts every flow-field search from splatting, src/renderer.cu:148-202).
 *
 * A 4-level U-Net (channels 32-64-96-128) on quarter-resolution keyframe data
 * predicts, for every output pixel, the source pixel offset of the converged search
 * in both keyframes; the learned render path (isti_render_learned, include/isti.h)
 * starts its search there.  Convolutions are implicit GEMMs on the tcgen05 tensor
 * core (bf16 operands staged by TMA, f32 accumulators in TMEM), for inference and for
 * both training gradients.
 *
 * Conventions: activations are NHWC bf16 in device memory, channels a multiple of 16,
 * width and height of the network input multiples of 8.  Weights are f32 masters laid
 * out [cout][tap][cin] with tap = 3 * (dy + 1) + (dx + 1) for 3x3 kernels (zero
 * padding of 1) and tap = 0 for 1x1.  All calls enqueue on `stream` and do not block;
 * `status` (device int32, may be NULL where noted) receives ISTI_ERR_TIMEOUT when a
 * bounded wait inside a kernel gave up.
 */
#ifndef ISTI_UNET_H
#define ISTI_UNET_H

#include <stddef.h>
#include <stdint.h>

#include "isti.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- operators ---- */

/* Bytes of the packed bf16 operand image of a cout x taps x cin weight tensor. */
size_t isti_unet_packed_bytes(int32_t taps, int32_t cin, int32_t cout);

/* Packs f32 weights [cout][taps][cin] for isti_unet_conv; transpose != 0 packs the
 * data-gradient convolution (inputs = the forward's cout channels, taps mirrored). */
isti_status isti_unet_pack(int32_t taps, const float *w, int32_t cin, int32_t cout, int32_t transpose, void *wpack, void *stream);

/* out[n,h,w,cout] = conv(x[n,h,w,cin], W) (+ bias[cout]) with optional ReLU, then,
 * when mask is given, multiplied by (mask[n,h,w,cout] > 0).  taps: 9 (3x3) or 1 (1x1);
 * cin, cout multiples of 16, cout <= 256. */
isti_status isti_unet_conv(int32_t taps, const void *x, int32_t n, int32_t h, int32_t w, int32_t cin, const void *wpack,
                           const float *bias, const void *mask, int32_t relu, void *out, int32_t cout, int32_t *status, void *stream);

/* dW[cout][taps][cin] (+)= sum over pixels of dy[p][co] * x[p + offset(tap)][ci]
 * (accumulate != 0 adds to dw).  scratch: isti_unet_wgrad_scratch_bytes bytes. */
size_t isti_unet_wgrad_scratch_bytes(int32_t taps, int32_t n, int32_t h, int32_t w, int32_t cin, int32_t cout);
isti_status isti_unet_wgrad(int32_t taps, const void *dy, const void *x, int32_t n, int32_t h, int32_t w, int32_t cin, int32_t cout,
                            float *dw, int32_t accumulate, void *scratch, size_t scratch_bytes, int32_t *status, void *stream);

/* ---- the network ----
 *
 * Architecture (h, w: the quarter-resolution input size, multiples of 8):
 *   e1 = relu(conv3x3 16->32)(x)        q1 = avgpool2(e1)
 *   e2 = relu(conv3x3 32->64)(q1)       q2 = avgpool2(e2)
 *   e3 = relu(conv3x3 64->96)(q2)       q3 = avgpool2(e3)
 *   e4 = relu(conv3x3 96->128)(q3)
 *   d3 = relu(conv3x3 96->96)(up2(conv1x1 128->96 (e4)) + e3)
 *   d2 = relu(conv3x3 64->64)(up2(conv1x1 96->64 (d3)) + e2)
 *   d1 = relu(conv3x3 32->32)(up2(conv1x1 64->32 (d2)) + e1)
 *   flow = conv1x1 32->4 (d1)           (f32, or f16 pairs: the FP16x2 flow per keyframe)
 * Layer i (0..9: e1, e2, e3, e4, p3, d3, p2, d2, p1, d1; 10: the head) is described by
 * isti_flownet_layer.  Parameters live in one f32 array: for each layer its weights
 * [cout][taps][cin] then its biases (offsets: isti_flownet_param_offsets); gradients
 * and Adam moments are laid out alike.
 *
 * Training: isti_flownet_backward runs the forward pass and the loss
 *   sum over labelled outputs of huber(flow - label) / (n * h * w)
 * (label: n x h x w x 4 f32, NaN = not labelled; huber delta 1), and writes every
 * parameter gradient (tensor-core data and weight gradients, fixed-order reductions);
 * isti_flownet_adam applies one Adam step (beta 0.9 / 0.999, eps 1e-8) and repacks the
 * bf16 operand images. */
typedef struct isti_flownet isti_flownet;

int32_t isti_flownet_input_channels(void);  /* 16 */
int32_t isti_flownet_output_channels(void); /* 4 */
int32_t isti_flownet_num_layers(void);      /* 11 */
isti_status isti_flownet_layer(int32_t index, int32_t *taps, int32_t *cin, int32_t *cout, int32_t *relu);

/* He-normal weights (seeded), zero biases. */
isti_status isti_flownet_create(isti_flownet **out, uint64_t seed);
isti_status isti_flownet_destroy(isti_flownet *net);

/* Device pointers to the f32 parameter and gradient arrays and their length.  After
 * writing parameters directly, call isti_flownet_sync_params. */
isti_status isti_flownet_tensors(isti_flownet *net, float **params, float **grads, size_t *count);
isti_status isti_flownet_param_offsets(const isti_flownet *net, int32_t layer, size_t *w_off, size_t *b_off);
isti_status isti_flownet_sync_params(isti_flownet *net, void *stream);

/* x: n x h x w x 16 bf16.  flow (n x h x w x 4 f32) and/or flow_f16 (n x h x w x 4 f16)
 * may be NULL. */
isti_status isti_flownet_forward(isti_flownet *net, const void *x, int32_t n, int32_t h, int32_t w, float *flow, void *flow_f16,
                                 void *stream);
isti_status isti_flownet_backward(isti_flownet *net, const void *x, const float *label, int32_t n, int32_t h, int32_t w, void *stream);
isti_status isti_flownet_adam(isti_flownet *net, float lr, void *stream);
/* Device address of the f32 loss of the last backward call. */
isti_status isti_flownet_loss(isti_flownet *net, float **loss_device);
/* Waits for the device; ISTI_OK or ISTI_ERR_TIMEOUT (a bounded wait in a kernel gave up). */
isti_status isti_flownet_device_status(isti_flownet *net, int32_t *status);

/* ---- the learned render path ----
 *
 * Renders n_frames client frames of one keyframe pair (main camera only, modes 0 and
 * 2) like isti_render_batch (chain_outputs with the same meaning), with the search
 * started from the network's guess instead of splatting:
 *  1. per keyframe pair: the client-independent part of the splat kernel (world
 *     positions and their motion, keyframe-to-keyframe flow);
 *  2. per frame: the network input at quarter resolution (inverse depth, object
 *     motion and client-camera flow of both keyframes, t), the network forward pass
 *     (the FP16x2 source offset per keyframe), then per output pixel `iterations`
 *     search steps (the reference's plain count is 3; 1 = a quarter of it rounded
 *     up) from the guessed source pixel, with the client-camera flow computed on the
 *     fly, and the error, direction choice and colour of the plain path;
 *  3. per 32 x 8 tile: when a pixel is left without a converged direction (its
 *     residual above EPS_1 in both keyframes) and its sources are not on the far
 *     plane, the tile is rendered by the plain method instead -- its keys from every
 *     source pixel that splats into it, window initialisation and 3 iterations --
 *     with the plain path's results.
 * net == NULL starts every search at the output pixel itself (no initialiser).
 * iterations == -1 sends every tile to the plain method (the result then equals
 * isti_render_batch's bit for bit: a check of the fallback).
 * No host synchronisation; isti_renderer_learned_stats waits and reports how many
 * tiles of the last call went to the plain method. */
isti_status isti_render_learned(isti_renderer *r, isti_flownet *net, int32_t n_frames, void *const *out_rgba,
                                const isti_render_info *infos, const isti_frame_data *frame, int32_t iterations, int32_t chain_outputs,
                                void *stream);
isti_status isti_renderer_learned_stats(isti_renderer *r, int32_t *fallback_tiles, int32_t *tiles);

#ifdef __cplusplus
}
#endif
#endif
