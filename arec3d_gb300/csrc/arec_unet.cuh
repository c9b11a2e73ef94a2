// Learned warm start: a BF16 4-level U-Net (32 base channels, FP32
// accumulation) trained and evaluated with this library's own kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "arec_internal.cuh"

namespace arecgb {

int conv3x3_bf16(const void *X, const void *Wt, const float *bias, void *Y, int N, int H, int Wd,
                 int Cin, int Cout, int relu, int layout, int *err, cudaStream_t st,
                 int ystride = 0);

namespace unet {

void conv_in(const float *x, const float *w, const float *b, __nv_bfloat16 *y, int N, int H, int W,
             int C, cudaStream_t st);
void conv_in_wgrad(const float *x, const __nv_bfloat16 *dpre, float *gw, float *gb, int N, int H,
                   int W, int C, cudaStream_t st);
void conv_out(const __nv_bfloat16 *h, const float *w, const float *b, const float *x0, float *y,
              size_t P, int C, cudaStream_t st);
void conv_out_bwd(const __nv_bfloat16 *h, const float *w, const float *dy, __nv_bfloat16 *dh,
                  float *gw, float *gb, size_t P, int C, cudaStream_t st);
void maxpool(const __nv_bfloat16 *x, __nv_bfloat16 *y, uint8_t *arg, int N, int H, int W, int C,
             cudaStream_t st, int xs = 0);
void maxpool_bwd(const __nv_bfloat16 *dy, const uint8_t *arg, float *dx_acc, int N, int H, int W,
                 int C, cudaStream_t st);
void upsample(const __nv_bfloat16 *x, __nv_bfloat16 *y, int N, int H, int W, int C, int Cy,
              cudaStream_t st);
void upsample_bwd(const __nv_bfloat16 *dy, __nv_bfloat16 *dx, int N, int H, int W, int C, int Cy,
                  cudaStream_t st);
void chan_copy(const __nv_bfloat16 *x, __nv_bfloat16 *y, size_t P, int C, int Cy, int off,
               cudaStream_t st);
void chan_add(const __nv_bfloat16 *src, float *dst, size_t P, int C, int Cs, int off,
              cudaStream_t st);
void f32_to_bf16(const float *a, __nv_bfloat16 *b, size_t n, cudaStream_t st);
void relu_bwd(const __nv_bfloat16 *y, const __nv_bfloat16 *dy, __nv_bfloat16 *dpre, size_t n,
              cudaStream_t st);
// dpre[p][c] = dy[p*dys + dyo + c] * (y[p*yys + yo + c] > 0), c < C
void relu_bwd_s(const __nv_bfloat16 *y, int yys, int yo, const __nv_bfloat16 *dy, int dys, int dyo,
                __nv_bfloat16 *dpre, size_t P, int C, cudaStream_t st);
void conv_wgrad(const __nv_bfloat16 *x, const __nv_bfloat16 *dpre, float *gw, float *gb, int N,
                int H, int W, int Cin, int Cout, cudaStream_t st);
void flip_weights(const float *w, __nv_bfloat16 *wt, int Cin, int Cout, cudaStream_t st);
void mse(const float *out, const float *target, float *dout, double *partial, size_t n, float scale,
         int nblocks, cudaStream_t st);
// Multi-scale loss (sum over levels s = 0..levels of ratio^s x the mean square
// of the error averaged over 2^s x 2^s blocks) and its gradient; pyr holds the
// pooled levels (N H W / 3 floats suffice).
void multiscale_loss(const float *out, const float *target, float *pyr, float *dout,
                     double *partial, int N, int H, int W, int levels, float ratio, float scale,
                     int nblocks, cudaStream_t st);
void adamw(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
           float eps, float wd, float bc1, float bc2, cudaStream_t st);
void cyl_to_img(const float *vol, const RowInfo *rows, float *img, int nx, int npad, int ys,
                int y0, int B, float scale, cudaStream_t st);
void img_to_cyl(const float *img, const RowInfo *rows, float *vol, int nx, int npad, int ys,
                int y0, int B, float scale, cudaStream_t st);
void sumsq_partial(const float *a, size_t n, double *part, int nblocks, cudaStream_t st);

}  // namespace unet
}  // namespace arecgb
