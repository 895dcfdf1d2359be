/*
 * bf_unet.h -- device kernels of the learned variant (no counterpart in the
 * reference): a small 3D convolutional U-Net that restores full-aperture DAS
 * volumes from volumes beamformed with every 4th receive channel, trained on the
 * GPU with these kernels. Part of libogl_beamformer_lib.so.
 *
 * Tensors are device pointers in channels-first layout [C][D][H][W] (x fastest),
 * dims = {W, H, D}. Element types: BF_UNET_F32 (float) or BF_UNET_BF16 (bfloat16
 * bits in uint16). Activations are stored in BF16, gradients and master weights
 * in FP32; every product is accumulated in FP32. Convolutions are 3 x 3 x 3,
 * stride 1, zero padding 1 ("same"); weights are [Cout][Cin][27] with tap index
 * (kz * 3 + ky) * 3 + kx. All functions enqueue on `stream` (a cudaStream_t) and
 * return 1, or 0 for invalid arguments or a launch error.
 */
#ifndef BF_UNET_H
#define BF_UNET_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BF_UNET_F32  0
#define BF_UNET_BF16 1

/* out[co] = relu?(bias[co] + sum_ci w[co][ci] * in[ci]) + residual[co] (residual
 * optional, same type as out, may alias nothing else). BF16 inputs run as an
 * implicit GEMM on the tensor cores (tcgen05, FP32 accumulation); FP32 inputs on
 * the direct kernel (FP32 products). Tensor-core calls share staging buffers
 * (weights, channels-last input): do not run two on different streams at once. */
uint32_t bf_unet_conv3d(const void *in, int32_t in_type, int32_t cin, const uint16_t *w, const float *bias,
                        const void *residual, void *out, int32_t out_type, int32_t cout, const int32_t dims[3],
                        int32_t relu, void *stream);

/* Nonzero when a tensor-core convolution's bounded wait ran out since the last
 * call (its CTA stopped early); synchronises `stream` first and clears the flag. */
uint32_t bf_unet_tc_errors(void *stream);

/* grad_in[ci] = sum_co w[co][ci] (flipped) * grad_out[co]; w_scratch holds
 * cin * cout * 27 bf16 (the transposed, flipped weights). grad_out is rounded to
 * BF16 and the sum runs on the tensor cores with FP32 accumulation (the direct
 * kernel with FP32 products where the tensor-core form does not apply). */
uint32_t bf_unet_conv3d_grad_input(const float *grad_out, int32_t cout, const uint16_t *w, float *grad_in, int32_t cin,
                                   const int32_t dims[3], uint16_t *w_scratch, void *stream);

/* grad_w[co][ci][k] += sum_v grad_out[co][v] in[ci][v + k - 1];
 * grad_b[co] += sum_v grad_out[co][v] (grad_b may be null). */
uint32_t bf_unet_conv3d_grad_weight(const float *grad_out, int32_t cout, const void *in, int32_t in_type, int32_t cin,
                                    const int32_t dims[3], float *grad_w, float *grad_b, void *stream);

/* grad[i] *= (act[i] > 0): the ReLU derivative from the stored activation */
uint32_t bf_unet_relu_grad(float *grad, const uint16_t *act, int64_t n, void *stream);

/* 2 x 2 x 2 mean pooling (dims of the input, each even) and its gradient
 * (accumulate != 0 adds the gradient into grad_in) */
uint32_t bf_unet_avgpool2(const void *in, int32_t in_type, void *out, int32_t out_type, int32_t c,
                          const int32_t dims_in[3], void *stream);
uint32_t bf_unet_avgpool2_grad(const float *grad_out, float *grad_in, int32_t c, const int32_t dims_in[3],
                               int32_t accumulate, void *stream);

/* nearest 2 x upsampling (dims of the output, each even) and its gradient */
uint32_t bf_unet_upsample2(const void *in, int32_t in_type, void *out, int32_t out_type, int32_t c,
                           const int32_t dims_out[3], void *stream);
uint32_t bf_unet_upsample2_grad(const float *grad_out, float *grad_in, int32_t c, const int32_t dims_out[3],
                                void *stream);

/* mean squared error of y against t (n values): *loss (f32, accumulated with
 * atomics; zero it first), grad = 2 (y - t) / n */
uint32_t bf_unet_mse(const float *y, const float *t, float *grad, float *loss, int64_t n, void *stream);

/* one Adam step on master weights w (FP32) with moments m, v; writes the BF16
 * copy w16 used by the convolutions */
uint32_t bf_unet_adam(float *w, const float *grad, float *m, float *v, uint16_t *w16, int64_t n, float lr,
                      float beta1, float beta2, float eps, int32_t step, void *stream);

/* exponential moving average of the master weights: ema = decay ema + (1 - decay) w;
 * writes the BF16 copy ema16 when it is not null */
uint32_t bf_unet_ema(float *ema, const float *w, uint16_t *ema16, int64_t n, float decay, void *stream);

/* type conversion (n values) */
uint32_t bf_unet_convert(const void *x, int32_t x_type, void *y, int32_t y_type, int64_t n, float scale, void *stream);

/* Seeded RF of point scatterers for training data: decoded traces
 * x[t][r][n] (f32, zeroed first) of a HERCULES acquisition with a plane-wave
 * transmit at 0 degrees; per scatterer a Gaussian-windowed two-cycle sine at the
 * two-way time of flight. pos = xyz in transducer coordinates [m] (n_scat x 3),
 * amp = amplitudes. */
uint32_t bf_synth_traces(const float *pos, const float *amp, int32_t n_scat, float *x, int32_t samples,
                         int32_t channels, int32_t transmits, float pitch_x, float pitch_y, float fs, float fc,
                         float c, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* BF_UNET_H */
