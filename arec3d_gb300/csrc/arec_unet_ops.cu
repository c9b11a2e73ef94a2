// Element-wise and reduction kernels of the learned warm start (U-Net), all
// NHWC with bf16 activations and fp32 weights/gradients.  The GEMM-shaped 3x3
// convolutions run on the tensor cores (arec_unet_conv.cu); everything here is
// memory-bound or small.
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

#include "arec_internal.cuh"
#include "arec_unet.cuh"

namespace arecgb {
namespace unet {

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ __nv_bfloat16 tobf(float v) { return __float2bfloat16(v); }

static int blocks_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

#define GRID_STRIDE(i, n) \
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

// ---- first layer: 1 -> C channels, 3x3, bias, ReLU (CUDA cores: 9 MACs per output) ---------
// One thread per pixel and all C channels: the 9 inputs are read once, the
// outputs leave as 16-byte vectors; per output the FMAs run in tap order from
// the bias (taps outside the image skipped).
template <int C>
__global__ void __launch_bounds__(256)
    k_conv_in(const float *__restrict__ x, const float *__restrict__ w,
              const float *__restrict__ b, __nv_bfloat16 *__restrict__ y, int N, int H, int W) {
    __shared__ float sw[C * 9], sb[C];
    for (int i = threadIdx.x; i < C * 9; i += blockDim.x) sw[i] = w[i];
    for (int i = threadIdx.x; i < C; i += blockDim.x) sb[i] = b[i];
    __syncthreads();
    const size_t P = (size_t)N * H * W;
    GRID_STRIDE(p, P) {
        const int wx = (int)(p % W);
        const size_t nh = p / W;
        const int h = (int)(nh % H);
        const size_t row0 = nh - h;  // first row of this image
        float v[9];
        bool in[9];
#pragma unroll
        for (int t = 0; t < 9; t++) {
            const int hh = h + t / 3 - 1, ww = wx + t % 3 - 1;
            in[t] = hh >= 0 && hh < H && ww >= 0 && ww < W;
            v[t] = in[t] ? x[(row0 + hh) * W + ww] : 0.f;
        }
        uint4 *yp = reinterpret_cast<uint4 *>(y + p * C);
#pragma unroll
        for (int q = 0; q < C / 8; q++) {
            __align__(16) __nv_bfloat16 o[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int c = q * 8 + j;
                float s = sb[c];
#pragma unroll
                for (int t = 0; t < 9; t++)
                    if (in[t]) s = fmaf(sw[c * 9 + t], v[t], s);
                o[j] = tobf(fmaxf(s, 0.f));
            }
            yp[q] = *reinterpret_cast<const uint4 *>(o);
        }
    }
}

// weight/bias gradient of the first layer: gw[c][t] += sum_p dpre[p][c] * x[p+t]
__global__ void k_conv_in_wgrad(const float *__restrict__ x, const __nv_bfloat16 *__restrict__ dpre,
                                float *__restrict__ gw, float *__restrict__ gb, int N, int H, int W,
                                int C) {
    // one block per output channel c; threads over pixels, block reduction
    const int c = blockIdx.x;
    float acc[10];
#pragma unroll
    for (int t = 0; t < 10; t++) acc[t] = 0.f;
    const size_t P = (size_t)N * H * W;
    for (size_t p = (size_t)blockIdx.y * blockDim.x + threadIdx.x; p < P;
         p += (size_t)gridDim.y * blockDim.x) {
        const float d = bf(dpre[p * C + c]);
        if (d == 0.f) continue;
        const int n = (int)(p / ((size_t)H * W)), h = (int)((p / W) % H), wx = (int)(p % W);
#pragma unroll
        for (int t = 0; t < 9; t++) {
            const int hh = h + t / 3 - 1, ww = wx + t % 3 - 1;
            if (hh >= 0 && hh < H && ww >= 0 && ww < W)
                acc[t] = fmaf(d, x[((size_t)n * H + hh) * W + ww], acc[t]);
        }
        acc[9] += d;
    }
    __shared__ float red[10][256];
#pragma unroll
    for (int t = 0; t < 10; t++) red[t][threadIdx.x] = acc[t];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
#pragma unroll
            for (int t = 0; t < 10; t++) red[t][threadIdx.x] += red[t][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 9) atomicAdd(&gw[c * 9 + threadIdx.x], red[threadIdx.x][0]);
    if (threadIdx.x == 9) atomicAdd(&gb[c], red[9][0]);
}

// ---- last layer: 1x1, C -> 1, plus the residual input --------------------------------------
template <int C>
__global__ void __launch_bounds__(256)
    k_conv_out(const __nv_bfloat16 *__restrict__ h, const float *__restrict__ w,
               const float *__restrict__ b, const float *__restrict__ x0,
               float *__restrict__ y, size_t P) {
    __shared__ float sw[C];
    for (int i = threadIdx.x; i < C; i += blockDim.x) sw[i] = w[i];
    __syncthreads();
    GRID_STRIDE(p, P) {
        float s = b[0] + x0[p];
        const uint4 *hp = reinterpret_cast<const uint4 *>(h + p * C);
#pragma unroll
        for (int q = 0; q < C / 8; q++) {
            const uint4 hv = hp[q];
            const __nv_bfloat16 *hb = reinterpret_cast<const __nv_bfloat16 *>(&hv);
#pragma unroll
            for (int j = 0; j < 8; j++) s = fmaf(sw[q * 8 + j], bf(hb[j]), s);
        }
        y[p] = s;
    }
}

// dh[p][c] = w[c]*dy[p]; gw[c] += sum dy*h; gb += sum dy  (C = kOutC channels)
constexpr int kOutC = 32;
__global__ void __launch_bounds__(128)
    k_conv_out_bwd(const __nv_bfloat16 *__restrict__ h, const float *__restrict__ w,
                   const float *__restrict__ dy, __nv_bfloat16 *__restrict__ dh,
                   float *__restrict__ gw, float *__restrict__ gb, size_t P) {
    __shared__ float sred[kOutC + 1][128];
    float acc[kOutC + 1];
#pragma unroll
    for (int c = 0; c <= kOutC; c++) acc[c] = 0.f;
    GRID_STRIDE(p, P) {
        const float d = dy[p];
        const uint4 *hp = reinterpret_cast<const uint4 *>(h + p * kOutC);
        uint4 *dp = reinterpret_cast<uint4 *>(dh + p * kOutC);
#pragma unroll
        for (int q = 0; q < kOutC / 8; q++) {
            const uint4 hv = hp[q];
            const __nv_bfloat16 *hb = reinterpret_cast<const __nv_bfloat16 *>(&hv);
            __align__(16) __nv_bfloat16 o[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                o[j] = tobf(w[q * 8 + j] * d);
                acc[q * 8 + j] = fmaf(d, bf(hb[j]), acc[q * 8 + j]);
            }
            dp[q] = *reinterpret_cast<const uint4 *>(o);
        }
        acc[kOutC] += d;
    }
#pragma unroll
    for (int c = 0; c <= kOutC; c++) sred[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int c = 0; c <= kOutC; c++) sred[c][threadIdx.x] += sred[c][threadIdx.x + o];
        __syncthreads();
    }
    if ((int)threadIdx.x < kOutC) atomicAdd(&gw[threadIdx.x], sred[threadIdx.x][0]);
    if ((int)threadIdx.x == kOutC) atomicAdd(gb, sred[kOutC][0]);
}

// ---- pooling / upsampling / concat -----------------------------------------------------------
// 2x2 max pooling with the arg max (0..3, first of equals) per output; one
// thread per output pixel and 8 channels (16-byte vectors; C % 8 == 0).
__global__ void k_maxpool(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y,
                          uint8_t *__restrict__ arg, int N, int H, int W, int C, int xs) {
    const int Ho = H / 2, Wo = W / 2, C8 = C / 8;
    const size_t n_out = (size_t)N * Ho * Wo * C8;
    GRID_STRIDE(i, n_out) {
        const int g = (int)(i % C8);
        const size_t po = i / C8;
        const int wo = (int)(po % Wo);
        const size_t nho = po / Wo;  // n * Ho + ho
        const size_t top = (2 * nho) * W + 2 * wo;  // (n * H + 2 ho) * W + 2 wo
        float best[8];
        uint8_t bi[8];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const size_t pix = top + (size_t)(t >> 1) * W + (t & 1);
            const uint4 xv = *reinterpret_cast<const uint4 *>(x + pix * xs + g * 8);
            const __nv_bfloat16 *xb = reinterpret_cast<const __nv_bfloat16 *>(&xv);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float v = bf(xb[j]);
                if (t == 0 || v > best[j]) {
                    best[j] = v;
                    bi[j] = (uint8_t)t;
                }
            }
        }
        __align__(16) __nv_bfloat16 o[8];
#pragma unroll
        for (int j = 0; j < 8; j++) o[j] = tobf(best[j]);
        *reinterpret_cast<uint4 *>(y + po * C + g * 8) = *reinterpret_cast<const uint4 *>(o);
        if (arg) {
            uint2 a;
            a.x = bi[0] | (bi[1] << 8) | (bi[2] << 16) | ((uint32_t)bi[3] << 24);
            a.y = bi[4] | (bi[5] << 8) | (bi[6] << 16) | ((uint32_t)bi[7] << 24);
            *reinterpret_cast<uint2 *>(arg + po * C + g * 8) = a;
        }
    }
}

__global__ void k_maxpool_bwd(const __nv_bfloat16 *__restrict__ dy, const uint8_t *__restrict__ arg,
                              float *__restrict__ dx_acc, int N, int H, int W, int C) {
    // dx_acc (fp32, zeroed by the caller) += routed gradient
    const int Ho = H / 2, Wo = W / 2;
    const size_t n_out = (size_t)N * Ho * Wo * C;
    GRID_STRIDE(i, n_out) {
        const int c = (int)(i % C);
        const size_t po = i / C;
        const int n = (int)(po / ((size_t)Ho * Wo)), ho = (int)((po / Wo) % Ho), wo = (int)(po % Wo);
        const int t = arg[i];
        const int h = 2 * ho + (t >> 1), w = 2 * wo + (t & 1);
        dx_acc[(((size_t)n * H + h) * W + w) * C + c] += bf(dy[i]);
    }
}

// nearest 2x upsampling of x [N][H][W][C] into channels [0, C) of y [N][2H][2W][Cy]
// One thread per input pixel and 8 channels: one 16-byte load, four stores
// (C, Cy multiples of 8).
__global__ void k_upsample(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y,
                           int N, int H, int W, int C, int Cy) {
    const int C8 = C / 8;
    const size_t n_in = (size_t)N * H * W * C8;
    GRID_STRIDE(i, n_in) {
        const int g = (int)(i % C8);
        const size_t p = i / C8;
        const int w = (int)(p % W);
        const size_t nh = p / W;  // n * H + h
        const uint4 v = *reinterpret_cast<const uint4 *>(x + p * C + g * 8);
        const size_t o0 = ((2 * nh) * (2 * W) + 2 * w) * Cy + g * 8;  // row 2h, column 2w
        *reinterpret_cast<uint4 *>(y + o0) = v;
        *reinterpret_cast<uint4 *>(y + o0 + Cy) = v;
        *reinterpret_cast<uint4 *>(y + o0 + (size_t)2 * W * Cy) = v;
        *reinterpret_cast<uint4 *>(y + o0 + (size_t)2 * W * Cy + Cy) = v;
    }
}

// dx[n][h][w][c] = sum over the 2x2 children of dy (channels [0, C) of a Cy-channel tensor)
__global__ void k_upsample_bwd(const __nv_bfloat16 *__restrict__ dy, __nv_bfloat16 *__restrict__ dx,
                               int N, int H, int W, int C, int Cy) {
    const size_t n_in = (size_t)N * H * W * C;
    GRID_STRIDE(i, n_in) {
        const int c = (int)(i % C);
        const size_t p = i / C;
        const int n = (int)(p / ((size_t)H * W)), h = (int)((p / W) % H), w = (int)(p % W);
        float s = 0.f;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int hh = 2 * h + (t >> 1), ww = 2 * w + (t & 1);
            s += bf(dy[(((size_t)n * 2 * H + hh) * 2 * W + ww) * Cy + c]);
        }
        dx[i] = tobf(s);
    }
}

// copy x [P][C] into channels [off, off+C) of y [P][Cy]
__global__ void k_chan_copy(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y,
                            size_t P, int C, int Cy, int off) {
    const int C8 = C / 8;  // 16-byte vectors (C, Cy, off multiples of 8)
    GRID_STRIDE(i, P * C8) {
        const size_t p = i / C8;
        const int g = (int)(i % C8);
        *reinterpret_cast<uint4 *>(y + p * Cy + off + g * 8) =
            *reinterpret_cast<const uint4 *>(x + p * C + g * 8);
    }
}

// dst[P][C] (fp32 accumulator) += channels [off, off+C) of src [P][Cs]
__global__ void k_chan_add(const __nv_bfloat16 *__restrict__ src, float *__restrict__ dst, size_t P,
                           int C, int Cs, int off) {
    GRID_STRIDE(i, P * C) { dst[i] += bf(src[(i / C) * Cs + off + (i % C)]); }
}

__global__ void k_f32_to_bf16(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, size_t n) {
    GRID_STRIDE(i, n) { b[i] = tobf(a[i]); }
}

// dpre = dy * (y > 0) (ReLU backward on the post-activation output)
__global__ void k_relu_bwd(const __nv_bfloat16 *__restrict__ y, const __nv_bfloat16 *__restrict__ dy,
                           __nv_bfloat16 *__restrict__ dpre, size_t n) {
    GRID_STRIDE(i, n) { dpre[i] = bf(y[i]) > 0.f ? dy[i] : tobf(0.f); }
}

__global__ void k_relu_bwd_s(const __nv_bfloat16 *__restrict__ y, int yys, int yo,
                             const __nv_bfloat16 *__restrict__ dy, int dys, int dyo,
                             __nv_bfloat16 *__restrict__ dpre, size_t P, int C) {
    GRID_STRIDE(i, P * C) {
        const size_t p = i / C;
        const int c = (int)(i % C);
        dpre[i] = bf(y[p * yys + yo + c]) > 0.f ? dy[p * dys + dyo + c] : tobf(0.f);
    }
}

// Weight gradient of a 3x3 conv on CUDA cores:
//   gw[co][t][ci] += sum_p dpre[p][co] * x[p+t][ci],  gb[co] += sum_p dpre[p][co]
// Block: 32 co x 32 ci for one tap, a slice of the pixels (grid.z); 256 threads,
// each 2 co x 2 ci; pixels staged through shared memory 64 at a time.
__global__ void __launch_bounds__(256)
    k_conv_wgrad(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ dpre,
                 float *__restrict__ gw, float *__restrict__ gb, int N, int H, int W, int Cin,
                 int Cout) {
    const int t = blockIdx.y % 9, cob = (blockIdx.y / 9) * 32, cib = blockIdx.x * 32;
    __shared__ float sd[64][33], sx[64][33];
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;  // co pair ty, ci pair tx
    float a00 = 0, a01 = 0, a10 = 0, a11 = 0, bsum0 = 0, bsum1 = 0;
    const size_t P = (size_t)N * H * W;
    const size_t per = (P + gridDim.z - 1) / gridDim.z;
    const size_t p_begin = per * blockIdx.z, p_end = min(P, p_begin + per);
    const int dy = t / 3 - 1, dx = t % 3 - 1;
    for (size_t pc = p_begin; pc < p_end; pc += 64) {
        for (int e = threadIdx.x; e < 64 * 32; e += 256) {
            const int pp = e / 32, c = e % 32;
            const size_t p = pc + pp;
            float dv = 0.f, xv = 0.f;
            if (p < p_end) {
                dv = bf(dpre[p * Cout + cob + c]);
                const int n = (int)(p / ((size_t)H * W)), h = (int)((p / W) % H), w = (int)(p % W);
                const int hh = h + dy, ww = w + dx;
                if (hh >= 0 && hh < H && ww >= 0 && ww < W)
                    xv = bf(x[(((size_t)n * H + hh) * W + ww) * Cin + cib + c]);
            }
            sd[pp][c] = dv;
            sx[pp][c] = xv;
        }
        __syncthreads();
#pragma unroll 8
        for (int pp = 0; pp < 64; pp++) {
            const float d0 = sd[pp][2 * ty], d1 = sd[pp][2 * ty + 1];
            const float x0 = sx[pp][2 * tx], x1 = sx[pp][2 * tx + 1];
            a00 = fmaf(d0, x0, a00);
            a01 = fmaf(d0, x1, a01);
            a10 = fmaf(d1, x0, a10);
            a11 = fmaf(d1, x1, a11);
            if (t == 4 && blockIdx.x == 0 && tx == 0) {
                bsum0 += d0;
                bsum1 += d1;
            }
        }
        __syncthreads();
    }
    const int co0 = cob + 2 * ty, ci0 = cib + 2 * tx;
    atomicAdd(&gw[((size_t)co0 * 9 + t) * Cin + ci0], a00);
    atomicAdd(&gw[((size_t)co0 * 9 + t) * Cin + ci0 + 1], a01);
    atomicAdd(&gw[((size_t)(co0 + 1) * 9 + t) * Cin + ci0], a10);
    atomicAdd(&gw[((size_t)(co0 + 1) * 9 + t) * Cin + ci0 + 1], a11);
    if (t == 4 && blockIdx.x == 0 && tx == 0) {
        atomicAdd(&gb[co0], bsum0);
        atomicAdd(&gb[co0 + 1], bsum1);
    }
}

// Data-gradient weights: wt[ci][t][co] = w[co][8 - t][ci] (flip and transpose), bf16.
__global__ void k_flip_weights(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wt, int Cin,
                               int Cout) {
    GRID_STRIDE(i, (size_t)Cout * 9 * Cin) {
        const int ci = (int)(i % Cin);
        const int t = (int)((i / Cin) % 9);
        const int co = (int)(i / ((size_t)Cin * 9));
        wt[((size_t)ci * 9 + (8 - t)) * Cout + co] = tobf(w[i]);
    }
}

// Loss: mean squared error over n values; writes d(loss)/d(out) and the sum of
// squared errors (one partial per block).
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ target,
                      float *__restrict__ dout, double *__restrict__ partial, size_t n, float scale) {
    __shared__ double red[256];
    double s = 0.0;
    GRID_STRIDE(i, n) {
        const float d = out[i] - target[i];
        dout[i] = scale * 2.f * d;
        s += (double)d * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Multi-scale loss: level s of the error pyramid is the error out - target
// averaged over 2^s x 2^s blocks (level 0 the error itself).  Pooling by 2 of
// level s-1 into level s; level 1 is pooled straight from out - target.
__global__ void k_err_pool(const float *__restrict__ a, const float *__restrict__ b,
                           float *__restrict__ y, int N, int H, int W) {
    const int Ho = H / 2, Wo = W / 2;
    GRID_STRIDE(p, (size_t)N * Ho * Wo) {
        const int xo = (int)(p % Wo), yo = (int)((p / Wo) % Ho), n = (int)(p / ((size_t)Wo * Ho));
        const size_t i0 = ((size_t)n * H + 2 * yo) * W + 2 * xo;
        float s = a[i0] + a[i0 + 1] + a[i0 + W] + a[i0 + W + 1];
        if (b) s -= b[i0] + b[i0 + 1] + b[i0 + W] + b[i0 + W + 1];
        y[p] = 0.25f * s;
    }
}

// dout = scale * 2 * sum_s alpha_s * level_s(block of p), alpha_s = ratio^s;
// the loss sum_s alpha_s * mean(level_s^2) is accumulated per pixel as
// sum_s alpha_s * level_s(block of p)^2 (the caller divides by the pixels).
__global__ void k_multiscale_grad(const float *__restrict__ out, const float *__restrict__ target,
                                  const float *__restrict__ pyr, float *__restrict__ dout,
                                  double *__restrict__ partial, int N, int H, int W, int levels,
                                  float ratio, float scale) {
    __shared__ double red[256];
    double acc = 0.0;
    GRID_STRIDE(p, (size_t)N * H * W) {
        const int x = (int)(p % W), yy = (int)((p / W) % H), n = (int)(p / ((size_t)W * H));
        const float e = out[p] - target[p];
        float g = e, a = 1.0f;
        double l = (double)e * e;
        const float *lev = pyr;
        int h = H, w = W;
        for (int s = 1; s <= levels; s++) {
            h >>= 1;
            w >>= 1;
            a *= ratio;
            const float v = lev[((size_t)n * h + (yy >> s)) * w + (x >> s)];
            g += a * v;
            // summed over the cell's 4^s pixels and divided by P: the cell mean
            l += (double)a * v * v;
            lev += (size_t)N * h * w;
        }
        dout[p] = scale * 2.f * g;
        acc += l;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// AdamW on fp32 master weights; refreshes the bf16 copy.
__global__ void k_adamw(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                        float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                        float wd, float bc1, float bc2) {
    GRID_STRIDE(i, n) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / bc1, vh = vi / bc2;
        w[i] = w[i] - lr * (mh / (sqrtf(vh) + eps) + wd * w[i]);
    }
}

// Cylinder volume [nrays][ys] (slices y0..y0+B) <-> image stack [B][np][np]
// (iz rows, ix columns, np >= nx padded with zeros), scaled by `scale`; zeros
// outside the disk (the device form of ImageCyl2CB / ImageCB2Cyl,
// AREC3D/AREC3D/arecImage.cpp:88-232).
__global__ void k_cyl_to_img(const float *__restrict__ vol, const RowInfo *__restrict__ rows,
                             float *__restrict__ img, int nx, int npad, int ys, int y0, int B,
                             float scale) {
    GRID_STRIDE(i, (size_t)B * npad * npad) {
        const int ix = (int)(i % npad), iz = (int)((i / npad) % npad);
        const int b = (int)(i / ((size_t)npad * npad));
        float v = 0.f;
        if (iz < nx) {
            const RowInfo r = rows[iz];
            if (ix >= r.lo && ix <= r.hi)
                v = scale * vol[(size_t)(r.start + ix - r.lo) * ys + y0 + b];
        }
        img[i] = v;
    }
}

__global__ void k_img_to_cyl(const float *__restrict__ img, const RowInfo *__restrict__ rows,
                             float *__restrict__ vol, int nx, int npad, int ys, int y0, int B,
                             float scale) {
    GRID_STRIDE(i, (size_t)B * npad * npad) {
        const int ix = (int)(i % npad), iz = (int)((i / npad) % npad);
        const int b = (int)(i / ((size_t)npad * npad));
        if (iz < nx) {
            const RowInfo r = rows[iz];
            if (ix >= r.lo && ix <= r.hi)
                vol[(size_t)(r.start + ix - r.lo) * ys + y0 + b] = scale * img[i];
        }
    }
}

// Sum of squares of n floats, one FP64 partial per block (summed on the host).
__global__ void k_sumsq_partial(const float *__restrict__ a, size_t n, double *__restrict__ part) {
    __shared__ double red[256];
    double s = 0.0;
    GRID_STRIDE(i, n) s += (double)a[i] * a[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// ---- host launchers -----------------------------------------------------------------------
void conv_in(const float *x, const float *w, const float *b, __nv_bfloat16 *y, int N, int H, int W,
             int C, cudaStream_t st) {
    if (C != 32) return;  // the network's first layer (32 channels)
    k_conv_in<32><<<blocks_for((size_t)N * H * W), 256, 0, st>>>(x, w, b, y, N, H, W);
}
void conv_in_wgrad(const float *x, const __nv_bfloat16 *dpre, float *gw, float *gb, int N, int H,
                   int W, int C, cudaStream_t st) {
    const size_t P = (size_t)N * H * W;
    int gy = (int)std::min<size_t>(64, (P + 255) / 256);
    k_conv_in_wgrad<<<dim3(C, gy), 256, 0, st>>>(x, dpre, gw, gb, N, H, W, C);
}
void conv_out(const __nv_bfloat16 *h, const float *w, const float *b, const float *x0, float *y,
              size_t P, int C, cudaStream_t st) {
    if (C != kOutC) return;
    k_conv_out<kOutC><<<blocks_for(P), 256, 0, st>>>(h, w, b, x0, y, P);
}
void conv_out_bwd(const __nv_bfloat16 *h, const float *w, const float *dy, __nv_bfloat16 *dh,
                  float *gw, float *gb, size_t P, int C, cudaStream_t st) {
    (void)C;  // kOutC
    int blocks = (int)std::min<size_t>(1024, (P + 127) / 128);
    k_conv_out_bwd<<<blocks, 128, 0, st>>>(h, w, dy, dh, gw, gb, P);
}
// x: [N][H][W] pixels of xs channels (xs = 0: C), the first C of them pooled
void maxpool(const __nv_bfloat16 *x, __nv_bfloat16 *y, uint8_t *arg, int N, int H, int W, int C,
             cudaStream_t st, int xs) {
    k_maxpool<<<blocks_for((size_t)N * H * W * C / 32), 256, 0, st>>>(x, y, arg, N, H, W, C,
                                                                      xs > 0 ? xs : C);
}
void maxpool_bwd(const __nv_bfloat16 *dy, const uint8_t *arg, float *dx_acc, int N, int H, int W,
                 int C, cudaStream_t st) {
    k_maxpool_bwd<<<blocks_for((size_t)N * H * W * C / 4), 256, 0, st>>>(dy, arg, dx_acc, N, H, W, C);
}
void upsample(const __nv_bfloat16 *x, __nv_bfloat16 *y, int N, int H, int W, int C, int Cy,
              cudaStream_t st) {
    k_upsample<<<blocks_for((size_t)N * H * W * C / 8), 256, 0, st>>>(x, y, N, H, W, C, Cy);
}
void upsample_bwd(const __nv_bfloat16 *dy, __nv_bfloat16 *dx, int N, int H, int W, int C, int Cy,
                  cudaStream_t st) {
    k_upsample_bwd<<<blocks_for((size_t)N * H * W * C), 256, 0, st>>>(dy, dx, N, H, W, C, Cy);
}
void chan_copy(const __nv_bfloat16 *x, __nv_bfloat16 *y, size_t P, int C, int Cy, int off,
               cudaStream_t st) {
    k_chan_copy<<<blocks_for(P * C / 8), 256, 0, st>>>(x, y, P, C, Cy, off);
}
void chan_add(const __nv_bfloat16 *src, float *dst, size_t P, int C, int Cs, int off,
              cudaStream_t st) {
    k_chan_add<<<blocks_for(P * C), 256, 0, st>>>(src, dst, P, C, Cs, off);
}
void f32_to_bf16(const float *a, __nv_bfloat16 *b, size_t n, cudaStream_t st) {
    k_f32_to_bf16<<<blocks_for(n), 256, 0, st>>>(a, b, n);
}
void relu_bwd(const __nv_bfloat16 *y, const __nv_bfloat16 *dy, __nv_bfloat16 *dpre, size_t n,
              cudaStream_t st) {
    k_relu_bwd<<<blocks_for(n), 256, 0, st>>>(y, dy, dpre, n);
}
void relu_bwd_s(const __nv_bfloat16 *y, int yys, int yo, const __nv_bfloat16 *dy, int dys, int dyo,
                __nv_bfloat16 *dpre, size_t P, int C, cudaStream_t st) {
    k_relu_bwd_s<<<blocks_for(P * C), 256, 0, st>>>(y, yys, yo, dy, dys, dyo, dpre, P, C);
}
void conv_wgrad(const __nv_bfloat16 *x, const __nv_bfloat16 *dpre, float *gw, float *gb, int N,
                int H, int W, int Cin, int Cout, cudaStream_t st) {
    const size_t P = (size_t)N * H * W;
    const int tiles = (Cin / 32) * (Cout / 32) * 9;
    int gz = (int)std::max<size_t>(1, std::min<size_t>((P + 4095) / 4096, (size_t)(152 * 8 / tiles + 1)));
    k_conv_wgrad<<<dim3(Cin / 32, 9 * (Cout / 32), gz), 256, 0, st>>>(x, dpre, gw, gb, N, H, W, Cin, Cout);
}
void flip_weights(const float *w, __nv_bfloat16 *wt, int Cin, int Cout, cudaStream_t st) {
    k_flip_weights<<<blocks_for((size_t)Cout * 9 * Cin), 256, 0, st>>>(w, wt, Cin, Cout);
}
void mse(const float *out, const float *target, float *dout, double *partial, size_t n, float scale,
         int nblocks, cudaStream_t st) {
    k_mse<<<nblocks, 256, 0, st>>>(out, target, dout, partial, n, scale);
}
void multiscale_loss(const float *out, const float *target, float *pyr, float *dout,
                     double *partial, int N, int H, int W, int levels, float ratio, float scale,
                     int nblocks, cudaStream_t st) {
    float *lev = pyr;
    const float *prev = nullptr;
    int h = H, w = W;
    for (int s = 1; s <= levels; s++) {
        const size_t n = (size_t)N * (h / 2) * (w / 2);
        if (s == 1)
            k_err_pool<<<blocks_for(n), 256, 0, st>>>(out, target, lev, N, h, w);
        else
            k_err_pool<<<blocks_for(n), 256, 0, st>>>(prev, nullptr, lev, N, h, w);
        prev = lev;
        lev += n;
        h /= 2;
        w /= 2;
    }
    k_multiscale_grad<<<nblocks, 256, 0, st>>>(out, target, pyr, dout, partial, N, H, W, levels,
                                               ratio, scale);
}
void adamw(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
           float eps, float wd, float bc1, float bc2, cudaStream_t st) {
    k_adamw<<<blocks_for(n), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, eps, wd, bc1, bc2);
}
void cyl_to_img(const float *vol, const RowInfo *rows, float *img, int nx, int npad, int ys,
                int y0, int B, float scale, cudaStream_t st) {
    k_cyl_to_img<<<blocks_for((size_t)B * npad * npad), 256, 0, st>>>(vol, rows, img, nx, npad, ys,
                                                                      y0, B, scale);
}
void img_to_cyl(const float *img, const RowInfo *rows, float *vol, int nx, int npad, int ys,
                int y0, int B, float scale, cudaStream_t st) {
    k_img_to_cyl<<<blocks_for((size_t)B * npad * npad), 256, 0, st>>>(img, rows, vol, nx, npad, ys,
                                                                      y0, B, scale);
}
void sumsq_partial(const float *a, size_t n, double *part, int nblocks, cudaStream_t st) {
    k_sumsq_partial<<<nblocks, 256, 0, st>>>(a, n, part);
}

}  // namespace unet
}  // namespace arecgb
