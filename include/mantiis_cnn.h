/*
 * C ABI of the warm-start network kernels (libmantiis_cnn.so).  No counterpart
 * in the reference: the learned warm start is an addition of this build.  A
 * convolutional encoder-decoder predicts steady fields from a pore image; the
 * lattice Boltzmann solver then starts from that prediction and iterates to
 * its own convergence criterion, so every reported answer is the solver's.
 *
 * Layouts: activations are FP32 NCHW (batch, channel, row, column); 3x3
 * convolution weights are [Cout][Cin][3][3], kept in FP32 for the optimiser
 * and in BF16 (uint16_t bit patterns) for the convolutions, which accumulate
 * in FP32.  All pointers are device pointers; every call enqueues on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and returns 0 or a negative
 * CUDA error code.
 */
#ifndef MANTIIS_CNN_H
#define MANTIIS_CNN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y = conv3x3(x, w) + b, zero padding, stride 1; relu != 0 applies max(0, .) */
int cnn_conv3x3_forward(const float *x, const uint16_t *w, const float *b, float *y, int n, int cin, int cout, int h,
                        int wd, int relu, void *stream);
/* dx = the gradient of conv3x3 with respect to its input, from dy (cout channels) */
int cnn_conv3x3_backward_data(const float *dy, const uint16_t *w, float *dx, int n, int cin, int cout, int h, int wd,
                              void *stream);
/* The same convolutions as implicit GEMMs on the tensor cores (tcgen05): the FP32
 * activations are split into two BF16 parts, each multiplied by the BF16 weights with FP32
 * accumulation in tensor memory, so the results agree with the two calls above to FP32
 * rounding.  cnn_tc_error() returns (and clears) the error word those kernels set when a
 * wait for their MMAs ran out (0 = none). */
int cnn_conv3x3_forward_tc(const float *x, const uint16_t *w, const float *b, float *y, int n, int cin, int cout,
                           int h, int wd, int relu, void *stream);
int cnn_conv3x3_backward_data_tc(const float *dy, const uint16_t *w, float *dx, int n, int cin, int cout, int h, int wd,
                                 void *stream);
/* the weight gradient the same way (both operands split, three MMAs per step, the
 * pixels split over CTAs whose partial sums are added to dw atomically) */
int cnn_conv3x3_backward_weight_tc(const float *x, const float *dy, float *dw, float *db, int n, int cin, int cout,
                                   int h, int wd, void *stream);
int cnn_tc_error(void);
/* dw += sum over batch and pixels of dy * shifted x; db += sum of dy (db may be NULL) */
int cnn_conv3x3_backward_weight(const float *x, const float *dy, float *dw, float *db, int n, int cin, int cout, int h,
                                int wd, void *stream);
/* dy *= (y > 0), y the ReLU output */
int cnn_relu_backward(float *dy, const float *y, int64_t count, void *stream);
/* 2x2 mean pooling (h, wd even) and its adjoint */
int cnn_avgpool2_forward(const float *x, float *y, int nc, int h, int wd, void *stream);
int cnn_avgpool2_backward(const float *dy, float *dx, int nc, int h, int wd, void *stream);
/* nearest 2x upsampling of an (h, wd) map and its adjoint (sum of the 2x2 block) */
int cnn_upsample2_forward(const float *x, float *y, int nc, int h, int wd, void *stream);
int cnn_upsample2_backward(const float *dy, float *dx, int nc, int h, int wd, void *stream);
/* y += x */
int cnn_add(float *y, const float *x, int64_t count, void *stream);
/* masked mean squared error over n images of c channels: loss[0] += sum mask (p - t)^2 / norm,
 * dp = 2 mask (p - t) / norm; mask is one (h, wd) map per image */
int cnn_mse(const float *p, const float *t, const float *mask, float *dp, float *loss, int n, int c, int h, int wd,
            float norm, void *stream);
/* Adam step on FP32 parameters, then their BF16 copy (w16 may be NULL) */
int cnn_adam(float *w, const float *g, float *m, float *v, uint16_t *w16, int64_t count, float lr, float beta1,
             float beta2, float eps, int step, void *stream);
/* FP32 -> BF16 (round to nearest even) */
int cnn_to_bf16(const float *x, uint16_t *y, int64_t count, void *stream);

#ifdef __cplusplus
}
#endif
#endif
