/* lbm_nn.h -- C ABI of the warm-start network kernels (liblbm_gb300.so).
 *
 * No counterpart in the reference: these train and run the 3D U-Net that maps
 * (solid mask, distance to solid) to a steady (v, rho - 1) field, used to
 * initialise the populations at equilibrium (lbm_init with rho, v).
 *
 * All pointers are device pointers; tensors are channels last (N, D, H, W, C).
 * Activations and conv weights are BF16, accumulation FP32.  Conv weights are
 * laid out [cout][27][cin] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)).  Every call
 * enqueues on `stream` (NULL = default stream) and returns 0 or LBM_E*.
 */
#ifndef LBM_NN_H
#define LBM_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 3x3x3 convolution, zero padding, implicit GEMM on the tcgen05 tensor cores
 * (accumulator in tensor memory, 128 voxels per accumulator).  Narrow layers
 * read a shared-memory halo, the others TMA im2col loads; LBM_NN_HALO=0 and
 * LBM_NN_TMA=0 in the environment (read once per process) select the next
 * kernel down, the last one staging operands with the CTA's threads.  mode 0:
 * out = relu(conv(in, w) + bias); mode 1: out = conv(in, w) * (mask > 0)
 * (mask NULL: no mask) -- the backward-data pass with flip-transposed weights.
 * Any voxel count; cin a multiple of 16 up to 128; cout in {16, 32, 48, 64, 96}. */
int lbm_nn_conv3d(const void* in, const void* w, const float* bias, const void* mask, void* out, int32_t n, int32_t d,
                  int32_t h, int32_t wd, int32_t cin, int32_t cout, int32_t mode, void* stream);
/* Same convolution with the activation choice: mode 0 and 1 as above; mode 2:
 * pre = conv(in, w) + bias, out = gelu(pre) (exact erf form; pre must be given,
 * same shape as out); mode 3: out = conv(in, w) * gelu'(mask) (mask = the
 * pre-activation of the layer being back-propagated into; NULL: no factor). */
int lbm_nn_conv3d_act(const void* in, const void* w, const float* bias, const void* mask, void* out, void* pre,
                      int32_t n, int32_t d, int32_t h, int32_t wd, int32_t cin, int32_t cout, int32_t mode,
                      void* stream);
/* *timed_out = 1 when a tensor-core convolution gave up waiting on its
 * pipeline since the last call (its output is then invalid); clears the flag. */
int lbm_nn_tc_status(int32_t* timed_out);
/* Self-test of that path: one CTA allocates tensor memory, waits (bounded,
 * about 1e6 cycles) on an mbarrier phase that nothing completes, sets the flag,
 * frees its tensor memory and returns; the context stays usable. */
int lbm_nn_tc_timeout_selftest(void* stream);
/* wt[ci][tap][co] = w[co][26 - tap][ci]: weights of the backward-data conv. */
int lbm_nn_flip_transpose(const void* w, void* wt, int32_t cin, int32_t cout, void* stream);
/* Weight gradient dw[co][tap][ci] (FP32) and bias gradient db[co] (may be NULL)
 * of the conv with input `in` and output gradient `g`, on the tcgen05 tensor
 * cores with both operands read MN-major from TMA boxes (LBM_NN_TMA=0: staged
 * by the CTA's threads); per-chunk FP32 partials summed in a fixed order; cin a multiple of
 * 16 up to 128, cout a multiple of 8 up to 64; scratch of
 * lbm_nn_wgrad_scratch_floats() floats. */
int64_t lbm_nn_wgrad_scratch_floats(int32_t n, int32_t d, int32_t h, int32_t w, int32_t cin, int32_t cout);
int lbm_nn_conv3d_wgrad(const void* in, const void* g, float* dw, float* db, float* scratch, int64_t scratch_floats,
                        int32_t n, int32_t d, int32_t h, int32_t w, int32_t cin, int32_t cout, void* stream);
/* 2x2x2 max pool (argmax kept for the backward pass) and its gradient:
 * gin = (accumulate ? gin : 0) + scatter(gout), then gin *= (mask > 0) when mask
 * is given (dims are the full-resolution ones). */
int lbm_nn_pool2(const void* in, void* out, uint8_t* arg, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                 void* stream);
int lbm_nn_pool2_bwd(const void* gout, const uint8_t* arg, void* gin, const void* mask, int32_t n, int32_t d,
                     int32_t h, int32_t w, int32_t c, int32_t accumulate, void* stream);
/* 2x nearest upsample (dims are the low-resolution ones) and its gradient,
 * multiplied by (mask > 0) when mask (low resolution) is given. */
int lbm_nn_upsample2(const void* in, void* out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void* stream);
int lbm_nn_upsample2_bwd(const void* gout, void* gin, const void* mask, int32_t n, int32_t d, int32_t h, int32_t w,
                         int32_t c, void* stream);
/* Channel concat [a | b] and the gradient split: ga = g[:, :ca];
 * gb = (accumulate_b ? gb : 0) + g[:, ca:], then gb *= (mask_b > 0) if mask_b. */
int lbm_nn_concat(const void* a, int32_t ca, const void* b, int32_t cb, void* out, int64_t nvox, void* stream);
int lbm_nn_split(const void* g, int32_t ca, int32_t cb, void* ga, void* gb, const void* mask_b, int32_t accumulate_b,
                 int64_t nvox, void* stream);
/* 1x1 output head y = x w^T + b (FP32 out; cin <= 64, cout <= 8), and its
 * backward: gx = (x > 0) * gy w; dw_db = [dw (cout*cin) | db (cout)];
 * scratch of 256 * (cout*cin + cout) floats. */
int lbm_nn_head(const void* x, const float* w, const float* b, float* y, int64_t nvox, int32_t cin, int32_t cout,
                void* stream);
int lbm_nn_head_bwd(const float* gy, const float* w, const void* x, void* gx, float* dw_db, float* scratch,
                    int64_t nvox, int32_t cin, int32_t cout, void* stream);
/* The head's backward for either activation of its input x: act 0 (ReLU) as
 * lbm_nn_head_bwd; act 1 (GELU) gx = gelu'(pre) * gy w with pre the
 * pre-activation of x. */
int lbm_nn_head_bwd_act(const float* gy, const float* w, const void* x, const void* pre, void* gx, float* dw_db,
                        float* scratch, int64_t nvox, int32_t cin, int32_t cout, int32_t act, void* stream);
/* g *= act'(d) in place over count BF16 elements: act 0 (ReLU) with d the
 * activation or pre-activation (factor d > 0), act 1 (GELU) with d the
 * pre-activation. */
int lbm_nn_act_bwd(void* g, const void* d, int64_t count, int32_t act, void* stream);
/* Masked MSE: loss = inv_count * sum over mask voxels of (y - t)^2, gy = its
 * gradient; scratch of 256 floats. */
int lbm_nn_mse(const float* y, const float* t, const uint8_t* mask, float* gy, float* loss, float* scratch,
               int64_t nvox, int32_t c, float inv_count, void* stream);
/* Adam step on FP32 master weights p (step counts from 1); p16 (BF16 copy) may be NULL. */
int lbm_nn_adam(float* p, const float* g, float* m, float* v, void* p16, int64_t n, float lr, float b1, float b2,
                float eps, int32_t step, float weight_decay, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LBM_NN_H */
