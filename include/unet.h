/*
 * unet.h -- C ABI of the learned-warm-start network kernels in
 * libstencil_gb300.so (no counterpart in the reference).
 *
 * The network is a 4-level fully-convolutional U-Net (3x3 convolutions, 32
 * base channels) that maps a 2-D Laplace problem's Dirichlet border to an
 * initial field for the Jacobi solve.  Activations are BF16 in NHWC layout
 * (channels innermost); convolution weights are BF16 [cout][3][3][cin] with
 * FP32 master copies; every convolution accumulates in FP32 on the tensor
 * cores (implicit GEMM).  All entry points are asynchronous on `stream`,
 * allocate nothing, and return STENCIL_OK or a negative STENCIL_E* status
 * (include/stencil_dispatch.h).
 */
#ifndef UNET_H
#define UNET_H

#include "stencil_dispatch.h"

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define UNET_API __attribute__((visibility("default")))
#else
#define UNET_API
#endif

/* A BF16 NHWC activation view: pixel (n, y, x) channel c lives at
 * ptr[((n*h + y)*w + x)*c_stride + c_off + c].  c_stride, c_off and c are
 * multiples of 8 (16-byte vectors); concatenation is a wider c_stride. */
typedef struct unet_act {
    void *ptr;
    int n, h, w;
    int c_stride, c_off, c;
    int reserved;
} unet_act;

/* y = act(conv3x3(x, w) + b), zero padding 1.  w: BF16 [y->c][3][3][x->c];
 * b: FP32 [y->c] or NULL; relu: 0/1.  x->c multiple of 32, y->c of 32. */
UNET_API int unet_conv3x3_fwd(const unet_act *x, const void *w, const float *b,
                              const unet_act *y, int relu, stencil_stream_t stream);
/* The same with the taps `dilation` cells apart (zero padding = dilation):
 * y[p] = act(b + sum_tap w[tap] x[p + dilation * (ky-1, kx-1)]). */
UNET_API int unet_conv3x3_fwd_dil(const unet_act *x, const void *w, const float *b,
                                  const unet_act *y, int relu, int dilation, stencil_stream_t stream);
/* The same convolution on a chosen engine: 1 = tcgen05 (5th-generation tensor
 * cores, FP32 accumulator in tensor memory), 2 = warp-level mma.sync, 0 = the
 * library's default.  Both engines take the same views and weights and agree
 * up to the FP32 summation order before the BF16 rounding. */
UNET_API int unet_conv3x3_fwd_engine(const unet_act *x, const void *w, const float *b,
                                     const unet_act *y, int relu, int dilation, int engine,
                                     stencil_stream_t stream);
/* wt[ci][ky][kx][co] = w[co][2-ky][2-kx][ci]: the weights of the data-gradient
 * convolution, so that dx = unet_conv3x3_fwd(dy, wt, NULL, dx, 0). */
UNET_API int unet_flip_weights(const void *w, void *wt, int cout, int cin,
                               stencil_stream_t stream);
/* dw[co][ky][kx][ci] += sum_p dy[p][co] * x[p + (ky-1, kx-1)][ci] (FP32, atomics);
 * db[co] += sum_p dy[p][co] if db != NULL. */
UNET_API int unet_conv3x3_wgrad(const unet_act *x, const unet_act *dy, float *dw, float *db,
                                stencil_stream_t stream);
/* Weight gradient of the dilated convolution (taps dilation * (ky-1, kx-1));
 * its data gradient is unet_conv3x3_fwd_dil with the flipped weights and the
 * same dilation. */
UNET_API int unet_conv3x3_wgrad_dil(const unet_act *x, const unet_act *dy, float *dw, float *db,
                                    int dilation, stencil_stream_t stream);
/* Bytes of device workspace the tcgen05 weight gradient needs for these
 * views: channel-major copies of x (three, shifted by -dilation, 0 and
 * +dilation columns) and of dy: (3 x->c + dy->c) * n * h * w * 2. */
UNET_API int unet_wgrad_workspace_bytes(const unet_act *x, const unet_act *dy, size_t *bytes);
/* The weight gradient on a chosen engine: 1 = tcgen05 (TMEM accumulator,
 * TMA-fed operands; needs w % 32 == 0 and a 256-byte aligned workspace of
 * unet_wgrad_workspace_bytes), 2 = mma.sync, 0 = tcgen05 where it applies.
 * Same accumulation contract as unet_conv3x3_wgrad_dil (FP32 atomics). */
UNET_API int unet_conv3x3_wgrad_engine(const unet_act *x, const unet_act *dy, float *dw, float *db,
                                       int dilation, int engine, void *workspace,
                                       size_t workspace_bytes, stencil_stream_t stream);
/* g *= (y > 0), element-wise over the view. */
UNET_API int unet_relu_bwd(const unet_act *g, const unet_act *y, stencil_stream_t stream);
/* 2x2 max pooling (h, w even) and its gradient (to the first maximal input). */
UNET_API int unet_maxpool2_fwd(const unet_act *x, const unet_act *y, stencil_stream_t stream);
UNET_API int unet_maxpool2_bwd(const unet_act *x, const unet_act *y, const unet_act *dy,
                               const unet_act *dx, stencil_stream_t stream);
/* Nearest-neighbour x2 upsampling and its gradient (sum of the 2x2 block). */
UNET_API int unet_upsample2_fwd(const unet_act *x, const unet_act *y, stencil_stream_t stream);
UNET_API int unet_upsample2_bwd(const unet_act *dy, const unet_act *dx, stencil_stream_t stream);
/* a += b (BF16 views of the same shape). */
UNET_API int unet_add(const unet_act *a, const unet_act *b, stencil_stream_t stream);
/* Output head: y[p] = sum_c x[p][c] * w[c] + b[0] (FP32 out, one channel). */
UNET_API int unet_head_fwd(const unet_act *x, const float *w, const float *b, float *y,
                           stencil_stream_t stream);
/* Head gradient: dx[p][c] = dy[p] * w[c]; dw[c] += sum_p dy[p] x[p][c]; db += sum dy. */
UNET_API int unet_head_bwd(const unet_act *x, const float *w, const float *dy,
                           const unet_act *dx, float *dw, float *db, stencil_stream_t stream);
/* Input features of n 2-D problems (fields fp32 [n][h][w], border band of
 * width 1 holds the Dirichlet values): channel 0 = the border field (zero
 * interior), 1 = the border mask, 2 = the transfinite (Coons) interpolation of
 * the border, channels 3.. of the view = 0.  coons (optional, fp32 [n][h][w])
 * receives channel 2. */
UNET_API int unet_features(const float *fields, int n, int h, int w, const unet_act *x,
                           float *coons, stencil_stream_t stream);
/* Masked MSE over interior cells: pred = coons + out; loss_sum (fp32, device)
 * += sum (pred - target)^2; dout = 2 (pred - target) * scale.  Border cells
 * get zero gradient. */
UNET_API int unet_mse(const float *out, const float *coons, const float *target, int n, int h,
                      int w, float scale, float *loss_sum, float *dout, stencil_stream_t stream);
/* Adam step on FP32 master parameters; also writes a BF16 copy if p_bf16 != NULL. */
UNET_API int unet_adam(float *p, const float *g, float *m, float *v, void *p_bf16, long long count,
                       float lr, float beta1, float beta2, float eps, int step,
                       stencil_stream_t stream);
/* Field assembly: u = coons + out on interior cells, the given border on the
 * band (fields is read for the border). */
UNET_API int unet_assemble(const float *fields, const float *coons, const float *out, int n, int h,
                           int w, float *u, stencil_stream_t stream);
/* Transfinite (Coons) interpolation of each field's border band (width 1)
 * on its interior, the border copied: fields and u fp32 [n][h][w]. */
UNET_API int unet_coons_fill(const float *fields, int n, int h, int w, float *u,
                             stencil_stream_t stream);
/* Coarse problems for the network: coarse fp32 [n][h][w] takes, on its border
 * band, the value of fields (fp32 [n][H][W]) at the nearest fine position
 * round(k (H-1)/(h-1)) (ties up) per axis, and zero inside. */
UNET_API int unet_resample_border(const float *fields, int n, int H, int W, int h, int w,
                                  float *coarse, stencil_stream_t stream);
/* Fine initial fields from coarse predictions: u fp32 [n][H][W] is the
 * bilinear interpolation of coarse (fp32 [n][h][w]) with corner cells
 * aligned (fine index I at coarse position I (w-1)/(W-1)) on the interior,
 * and equals fields (fp32 [n][H][W]) on the border band. */
UNET_API int unet_upsample_bilinear(const float *coarse, int n, int h, int w, const float *fields,
                                    int H, int W, float *u, stencil_stream_t stream);
/* FP32 -> BF16 copy (count elements). */
UNET_API int unet_to_bf16(const float *src, void *dst, long long count, stencil_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* UNET_H */
