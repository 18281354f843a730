/*
 * recon_initnet.h -- learned initialisation for the tracker: a small
 * convolutional network that predicts the frame-to-frame motion twist from the
 * coarse (80x60) intensity and depth of the previous and the current frame.
 *
 * There is no counterpart in the reference: its tracker always starts a frame
 * from the previous frame's pose (PhotoTracker::track, phototracker.cpp:596-689).
 * Here the prediction replaces that start pose unless its coarse-level
 * photometric residual is higher (the plain start pose is the fallback), and
 * the tracker then runs the schedule given to recon_batch_set_init_net.
 *
 * Network: 6 convolutions 3x3 / stride 2 / pad 1 with ReLU (channels 4 -> 16
 * -> 32 -> 64 -> 64 -> 128 -> 128; 60x80 -> 30x40 -> 15x20 -> 8x10 -> 4x5 ->
 * 2x3 -> 1x2), global average pooling and a linear layer to 6 outputs.
 * Convolution inputs and weights are BF16 and accumulate in FP32 on the tensor
 * cores; activations are stored in BF16; gradients, biases and the optimizer
 * state are FP32.  Input layout: [n][60][80][4] BF16 (previous gray, previous
 * depth, current gray, current depth), gray in [0,1], depth in metres / 4.
 * Output: 6 numbers per sample, the twist divided by the per-component scale
 * stored with the parameters (rotation in radians, translation in metres;
 * the SE(3) convention of the tracker's pose update).
 *
 * Parameter layout (one flat FP32 array): for layer l = 1..6, W_l[cout][kpad]
 * with k = (ky*3 + kx) * cin + c (kpad = 9 cin rounded up to 16, padding zero)
 * then b_l[cout]; then W_fc[6][128], b_fc[6]; then scale[6].
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RECON_NET_W 80
#define RECON_NET_H 60
#define RECON_NET_IN_CH 4
#define RECON_NET_OUT 6

typedef struct recon_initnet recon_initnet;

int64_t recon_initnet_param_count(void);

/* A network with room for batches of up to max_batch samples; parameters zero.
 * All its work runs on `stream` (NULL: the legacy default stream). */
int recon_initnet_create(int32_t max_batch, void *stream, recon_initnet **out);
int recon_initnet_destroy(recon_initnet *net);
/* FP32 parameters (host or device, recon_initnet_param_count() floats). */
int recon_initnet_set_params(recon_initnet *net, const float *params, int32_t on_device);
int recon_initnet_get_params(recon_initnet *net, float *params_host);

/* Forward pass: in_bf16 [n][60][80][4] (device, BF16 bits), out [n][6] FP32 (device). */
int recon_initnet_forward(recon_initnet *net, const uint16_t *in_bf16, int32_t n, float *out);

/* Forward + backward of the loss mean_n sum_j (out[n][j] - target[n][j])^2 / 6:
 * the gradient of every parameter (the scale entries get 0) into grad (device,
 * param_count floats) and the loss into *loss_dev (device).  No update. */
int recon_initnet_gradient(recon_initnet *net, const uint16_t *in_bf16, const float *target, int32_t n,
                           float *grad, float *loss_dev);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the same loss. */
int recon_initnet_train_step(recon_initnet *net, const uint16_t *in_bf16, const float *target, int32_t n,
                             float lr, float *loss_dev);

/* Coarse network image of a frame: [60][80][2] BF16 (gray in [0,1], depth in
 * metres / 4, 0 where the depth is 0) from uint8 gray and uint16 depth (mm) of
 * a width x height frame (multiples of 80 x 60); each output pixel averages
 * its (width/80) x (height/60) block, depth over the valid pixels.  Device
 * pointers, n frames, frame k at gray + k * width * height. */
int recon_initnet_coarse(const uint8_t *gray, const uint16_t *depth, int32_t n, int32_t width, int32_t height,
                         uint16_t *out_bf16, void *stream);
/* Network inputs [n][60][80][4] from coarse images: prev[k], cur[k] (device). */
int recon_initnet_pair(const uint16_t *prev_coarse, const uint16_t *cur_coarse, int32_t n, uint16_t *in_bf16,
                       void *stream);

#ifdef __cplusplus
}
#endif
