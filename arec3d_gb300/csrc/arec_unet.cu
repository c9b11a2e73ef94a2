// Learned warm start: a BF16 4-level U-Net (32 base channels, FP32
// accumulation and master weights) mapping an early reconstruction of a slice
// (few-iteration SIRT) to an initial guess for CGLS.  The reference has no
// counterpart; plain CGLS continuing from the guess is unchanged and still
// decides the result.
//
// Architecture (NHWC, bf16 activations, every 3x3 conv with bias + ReLU):
//   level 0 (H x W):    c1a 1->32 (CUDA cores), c1b 32->32               = e1
//   level 1 (H/2):      pool, c2a 32->64, c2b 64->64                     = e2
//   level 2 (H/4):      pool, c3a 64->128, c3b 128->128                  = e3
//   level 3 (H/8):      pool, c4a 128->256, c4b 256->256                 = e4
//   decoder level 2:    up(e4), u3 256->128 | e3 -> d3a 256->128, d3b 128->128 = g3
//   decoder level 1:    up(g3), u2 128->64  | e2 -> d2a 128->64,  d2b 64->64   = g2
//   decoder level 0:    up(g2), u1 64->32   | e1 -> d1a 64->32,   d1b 32->32   = g1
//   output:             1x1 32->1 + the input (residual)
// "up" is nearest 2x upsampling, "|" channel concatenation ([up-conv, skip]):
// c1b, c2b and c3b write e1, e2, e3 straight into the trailing channels of
// the concatenation buffers cat1, cat2, cat3, where the pooling and the
// decoder read them (no copy).
// The 3x3 convolutions of 32+ input channels, forward and data-gradient, run on
// the tensor cores (tcgen05, arec_unet_conv.cu); weight gradients, pooling,
// upsampling, the first and last layers run on CUDA cores (arec_unet_ops.cu).
//
// Parameters: one flat FP32 vector, per layer W then b, W in [Cout][9][Cin]
// (c1a: [32][9]; output: [32]); a bf16 mirror with the same offsets feeds the
// forward convolutions, a flipped/transposed bf16 copy the data gradients.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "arec_internal.cuh"
#include "arec_unet.cuh"

namespace arecgb {
namespace unet {

enum Layer { C1A, C1B, C2A, C2B, C3A, C3B, C4A, C4B, U3, D3A, D3B, U2, D2A, D2B, U1, D1A, D1B, OUT, NL };
static const int kCin[NL] = {1, 32, 32, 64, 64, 128, 128, 256, 256, 256, 128, 128, 128, 64, 64, 64, 32, 32};
static const int kCout[NL] = {32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 128, 64, 64, 64, 32, 32, 32, 1};

struct Net {
    int H = 0, W = 0, maxN = 0, train = 0;
    size_t woff[NL], boff[NL], nparams = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wbf = nullptr, *wflip = nullptr;
    int step = 0;
    bool mirrors_fresh = false;
    // training loss: loss_levels = 0 is the mean square error; > 0 adds the
    // error pooled over 2^s x 2^s blocks for s = 1..loss_levels, weighted
    // loss_ratio^s (low frequencies count more, as in the normal-equation
    // residual the solver's stopping test measures)
    int loss_levels = 0;
    float loss_ratio = 1.f;
    float *pyr = nullptr;

    // activations (P0 = maxN*H*W pixels, P1 = P0/4, ...)
    __nv_bfloat16 *a1, *q1, *a2, *q2, *a3, *q3, *a4, *e4;
    __nv_bfloat16 *up3, *cat3, *f3, *g3, *up2, *cat2, *f2, *g2, *up1, *cat1, *f1, *g1;
    uint8_t *arg1, *arg2, *arg3;
    const float *in = nullptr;  // input of the last forward
    int lastN = 0;
    // training scratch
    __nv_bfloat16 *gX = nullptr, *gY = nullptr, *gpre = nullptr;
    float *de1 = nullptr, *de2 = nullptr, *de3 = nullptr, *out = nullptr, *dout = nullptr;
    double *partials = nullptr, *h_partials = nullptr;
    int *err = nullptr;
    std::vector<void *> blocks;  // everything cudaMalloc'd
};

static constexpr int kLossBlocks = 512;

template <typename T>
static int alloc(Net *n, T **p, size_t count) {
    void *q = nullptr;
    ARECGB_CUDA(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    n->blocks.push_back(q);
    *p = reinterpret_cast<T *>(q);
    return 0;
}

static void destroy(Net *n) {
    if (!n) return;
    for (void *p : n->blocks) cudaFree(p);
    if (n->h_partials) cudaFreeHost(n->h_partials);
    delete n;
}

// Deterministic initial weights: He-normal for the ReLU layers, zero biases,
// zero output layer (the untrained network is the identity map).
static uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double gauss(uint64_t &s) {
    const double u1 = ((splitmix(s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
    const double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
}

static int refresh_mirrors(Net *n, cudaStream_t st) {
    f32_to_bf16(n->params, n->wbf, n->nparams, st);
    if (n->train)
        for (int l = C1B; l <= D1B; l++)
            flip_weights(n->params + n->woff[l], n->wflip + n->woff[l], kCin[l], kCout[l], st);
    ARECGB_CUDA(cudaGetLastError());
    n->mirrors_fresh = true;
    return 0;
}

static int create(Net **out, int H, int W, int maxN, int train, uint64_t seed) {
    if (H < 8 || W < 8 || H % 8 || W % 8 || maxN < 1) {
        set_error("unet_create: H and W must be positive multiples of 8, batch >= 1");
        return ARECGB_ERR_ARG;
    }
    Net *n = new Net();
    n->H = H;
    n->W = W;
    n->maxN = maxN;
    n->train = train;
    size_t off = 0;
    for (int l = 0; l < NL; l++) {
        const size_t nw = l == OUT ? (size_t)kCin[l] : (size_t)kCout[l] * 9 * kCin[l];
        n->woff[l] = off;
        off += nw;
        n->boff[l] = off;
        off += (size_t)((kCout[l] + 7) / 8 * 8);  // keep every offset a multiple of 8
    }
    n->nparams = off;
    const size_t P0 = (size_t)maxN * H * W, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
    int rc = 0;
#define A(ptr, count) \
    if (!rc) rc = alloc(n, &n->ptr, (count));
    A(params, off) A(wbf, off)
    A(a1, P0 * 32) A(q1, P1 * 32) A(a2, P1 * 64) A(q2, P2 * 64)
    A(a3, P2 * 128) A(q3, P3 * 128) A(a4, P3 * 256) A(e4, P3 * 256)
    A(up3, P2 * 256) A(cat3, P2 * 256) A(f3, P2 * 128) A(g3, P2 * 128)
    A(up2, P1 * 128) A(cat2, P1 * 128) A(f2, P1 * 64) A(g2, P1 * 64)
    A(up1, P0 * 64) A(cat1, P0 * 64) A(f1, P0 * 32) A(g1, P0 * 32)
    A(arg1, P1 * 32) A(arg2, P2 * 64) A(arg3, P3 * 128) A(err, 1)
    if (train) {
        A(grads, off) A(m, off) A(v, off) A(wflip, off)
        A(gX, P0 * 64) A(gY, P0 * 64) A(gpre, P0 * 32)
        A(de1, P0 * 32) A(de2, P1 * 64) A(de3, P2 * 128) A(out, P0) A(dout, P0)
        A(partials, kLossBlocks) A(pyr, P0 / 3 + 64)
    }
#undef A
    if (!rc && train) {
        cudaError_t e = cudaMallocHost(&n->h_partials, sizeof(double) * kLossBlocks);
        if (e != cudaSuccess) {
            set_error(std::string("unet_create: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    if (rc) {
        destroy(n);
        return rc;
    }
    std::vector<float> h(off, 0.f);
    uint64_t s = seed;
    for (int l = 0; l < OUT; l++) {
        const double sd = std::sqrt(2.0 / (9.0 * kCin[l]));
        const size_t nw = (size_t)kCout[l] * 9 * kCin[l];
        for (size_t i = 0; i < nw; i++) h[n->woff[l] + i] = (float)(sd * gauss(s));
    }
    cudaError_t e = cudaMemcpy(n->params, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && train) {
        e = cudaMemset(n->m, 0, sizeof(float) * off);
        if (e == cudaSuccess) e = cudaMemset(n->v, 0, sizeof(float) * off);
    }
    if (e == cudaSuccess) e = cudaMemset(n->err, 0, sizeof(int));
    if (e != cudaSuccess) {
        set_error(std::string("unet_create: ") + cudaGetErrorString(e));
        destroy(n);
        return cuda_status(e);
    }
    if ((rc = refresh_mirrors(n, 0))) {
        destroy(n);
        return rc;
    }
    *out = n;
    return 0;
}

// 3x3 conv + bias + ReLU with this net's bf16 weights; `ystride` > Cout writes
// into the leading channels of a wider (concatenated) tensor.
static int conv(Net *n, int l, const __nv_bfloat16 *x, __nv_bfloat16 *y, int N, int h, int w,
                cudaStream_t st, int ystride = 0) {
    return conv3x3_bf16(x, n->wbf + n->woff[l], n->params + n->boff[l], y, N, h, w, kCin[l],
                        kCout[l], 1, 0, n->err, st, ystride);
}

static int forward(Net *n, const float *x, float *y, int N, cudaStream_t st) {
    const int H = n->H, W = n->W;
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
    const size_t P0 = (size_t)N * H * W, P1 = P0 / 4, P2 = P0 / 16;
    int rc = 0;
    if (!n->mirrors_fresh && (rc = refresh_mirrors(n, st))) return rc;
    conv_in(x, n->params + n->woff[C1A], n->params + n->boff[C1A], n->a1, N, H, W, 32, st);
    // e1 = cat1[:, 32:64), e2 = cat2[:, 64:128), e3 = cat3[:, 128:256)
    if ((rc = conv(n, C1B, n->a1, n->cat1 + 32, N, H, W, st, 64))) return rc;
    maxpool(n->cat1 + 32, n->q1, n->arg1, N, H, W, 32, st, 64);
    if ((rc = conv(n, C2A, n->q1, n->a2, N, H1, W1, st))) return rc;
    if ((rc = conv(n, C2B, n->a2, n->cat2 + 64, N, H1, W1, st, 128))) return rc;
    maxpool(n->cat2 + 64, n->q2, n->arg2, N, H1, W1, 64, st, 128);
    if ((rc = conv(n, C3A, n->q2, n->a3, N, H2, W2, st))) return rc;
    if ((rc = conv(n, C3B, n->a3, n->cat3 + 128, N, H2, W2, st, 256))) return rc;
    maxpool(n->cat3 + 128, n->q3, n->arg3, N, H2, W2, 128, st, 256);
    if ((rc = conv(n, C4A, n->q3, n->a4, N, H3, W3, st))) return rc;
    if ((rc = conv(n, C4B, n->a4, n->e4, N, H3, W3, st))) return rc;
    // decoder level 2
    upsample(n->e4, n->up3, N, H3, W3, 256, 256, st);
    if ((rc = conv(n, U3, n->up3, n->cat3, N, H2, W2, st, 256))) return rc;
    if ((rc = conv(n, D3A, n->cat3, n->f3, N, H2, W2, st))) return rc;
    if ((rc = conv(n, D3B, n->f3, n->g3, N, H2, W2, st))) return rc;
    // decoder level 1
    upsample(n->g3, n->up2, N, H2, W2, 128, 128, st);
    if ((rc = conv(n, U2, n->up2, n->cat2, N, H1, W1, st, 128))) return rc;
    if ((rc = conv(n, D2A, n->cat2, n->f2, N, H1, W1, st))) return rc;
    if ((rc = conv(n, D2B, n->f2, n->g2, N, H1, W1, st))) return rc;
    // decoder level 0
    upsample(n->g2, n->up1, N, H1, W1, 64, 64, st);
    if ((rc = conv(n, U1, n->up1, n->cat1, N, H, W, st, 64))) return rc;
    if ((rc = conv(n, D1A, n->cat1, n->f1, N, H, W, st))) return rc;
    if ((rc = conv(n, D1B, n->f1, n->g1, N, H, W, st))) return rc;
    conv_out(n->g1, n->params + n->woff[OUT], n->params + n->boff[OUT], x, y, P0, 32, st);
    count_launches(24);  // conv_in, 16 tensor-core convolutions, 3 pool, 3 upsample, out
    ARECGB_CUDA(cudaGetLastError());
    n->in = x;
    n->lastN = N;
    return 0;
}

// Backward of one 3x3 conv + ReLU layer: dy (gradient w.r.t. its post-ReLU
// output y, both read with row stride ys) -> weight/bias gradients and, if dx,
// the gradient w.r.t. its input x.
static int conv_bwd(Net *n, int l, const __nv_bfloat16 *x, const __nv_bfloat16 *y, int ys,
                    const __nv_bfloat16 *dy, int dys, __nv_bfloat16 *dx, int N, int h, int w,
                    cudaStream_t st) {
    const size_t P = (size_t)N * h * w;
    const int ci = kCin[l], co = kCout[l];
    relu_bwd_s(y, ys, 0, dy, dys, 0, n->gpre, P, co, st);
    conv_wgrad(x, n->gpre, n->grads + n->woff[l], n->grads + n->boff[l], N, h, w, ci, co, st);
    if (dx)
        return conv3x3_bf16(n->gpre, n->wflip + n->woff[l], nullptr, dx, N, h, w, co, ci, 0, 0,
                            n->err, st, ci);
    return 0;
}

// Gradients (accumulated into n->grads) of the loss whose gradient w.r.t. the
// last forward's output is dout.
static int backward(Net *n, const float *dout, cudaStream_t st) {
    const int N = n->lastN, H = n->H, W = n->W;
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
    const size_t P0 = (size_t)N * H * W, P1 = P0 / 4, P2 = P0 / 16;
    __nv_bfloat16 *gX = n->gX, *gY = n->gY;
    int rc = 0;
    conv_out_bwd(n->g1, n->params + n->woff[OUT], dout, gY, n->grads + n->woff[OUT],
                 n->grads + n->boff[OUT], P0, 32, st);
    // decoder level 0
    if ((rc = conv_bwd(n, D1B, n->f1, n->g1, 32, gY, 32, gX, N, H, W, st))) return rc;
    if ((rc = conv_bwd(n, D1A, n->cat1, n->f1, 32, gX, 32, gY, N, H, W, st))) return rc;
    ARECGB_CUDA(cudaMemsetAsync(n->de1, 0, sizeof(float) * P0 * 32, st));
    chan_add(gY, n->de1, P0, 32, 64, 32, st);
    if ((rc = conv_bwd(n, U1, n->up1, n->cat1, 64, gY, 64, gX, N, H, W, st))) return rc;
    upsample_bwd(gX, gY, N, H1, W1, 64, 64, st);
    // decoder level 1
    if ((rc = conv_bwd(n, D2B, n->f2, n->g2, 64, gY, 64, gX, N, H1, W1, st))) return rc;
    if ((rc = conv_bwd(n, D2A, n->cat2, n->f2, 64, gX, 64, gY, N, H1, W1, st))) return rc;
    ARECGB_CUDA(cudaMemsetAsync(n->de2, 0, sizeof(float) * P1 * 64, st));
    chan_add(gY, n->de2, P1, 64, 128, 64, st);
    if ((rc = conv_bwd(n, U2, n->up2, n->cat2, 128, gY, 128, gX, N, H1, W1, st))) return rc;
    upsample_bwd(gX, gY, N, H2, W2, 128, 128, st);
    // decoder level 2
    if ((rc = conv_bwd(n, D3B, n->f3, n->g3, 128, gY, 128, gX, N, H2, W2, st))) return rc;
    if ((rc = conv_bwd(n, D3A, n->cat3, n->f3, 128, gX, 128, gY, N, H2, W2, st))) return rc;
    ARECGB_CUDA(cudaMemsetAsync(n->de3, 0, sizeof(float) * P2 * 128, st));
    chan_add(gY, n->de3, P2, 128, 256, 128, st);
    if ((rc = conv_bwd(n, U3, n->up3, n->cat3, 256, gY, 256, gX, N, H2, W2, st))) return rc;
    upsample_bwd(gX, gY, N, H3, W3, 256, 256, st);
    // encoder level 3
    if ((rc = conv_bwd(n, C4B, n->a4, n->e4, 256, gY, 256, gX, N, H3, W3, st))) return rc;
    if ((rc = conv_bwd(n, C4A, n->q3, n->a4, 256, gX, 256, gY, N, H3, W3, st))) return rc;
    maxpool_bwd(gY, n->arg3, n->de3, N, H2, W2, 128, st);
    f32_to_bf16(n->de3, gX, P2 * 128, st);
    // encoder level 2
    if ((rc = conv_bwd(n, C3B, n->a3, n->cat3 + 128, 256, gX, 128, gY, N, H2, W2, st))) return rc;
    if ((rc = conv_bwd(n, C3A, n->q2, n->a3, 128, gY, 128, gX, N, H2, W2, st))) return rc;
    maxpool_bwd(gX, n->arg2, n->de2, N, H1, W1, 64, st);
    f32_to_bf16(n->de2, gY, P1 * 64, st);
    // encoder level 1
    if ((rc = conv_bwd(n, C2B, n->a2, n->cat2 + 64, 128, gY, 64, gX, N, H1, W1, st))) return rc;
    if ((rc = conv_bwd(n, C2A, n->q1, n->a2, 64, gX, 64, gY, N, H1, W1, st))) return rc;
    maxpool_bwd(gY, n->arg1, n->de1, N, H, W, 32, st);
    f32_to_bf16(n->de1, gX, P0 * 32, st);
    // encoder level 0
    if ((rc = conv_bwd(n, C1B, n->a1, n->cat1 + 32, 64, gX, 32, gY, N, H, W, st))) return rc;
    relu_bwd(n->a1, gY, n->gpre, P0 * 32, st);
    conv_in_wgrad(n->in, n->gpre, n->grads + n->woff[C1A], n->grads + n->boff[C1A], N, H, W, 32,
                  st);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

static int check_err(Net *n, cudaStream_t st, const char *what) {
    int h = 0;
    ARECGB_CUDA(cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    ARECGB_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error(std::string(what) + ": a tensor-core wait timed out (error flag " +
                  std::to_string(h) + ")");
        return ARECGB_ERR_CUDA_BASE;
    }
    return 0;
}

static int train_step(Net *n, const float *x, const float *target, int N, float lr, float wd,
                      double *loss, cudaStream_t st) {
    int rc = forward(n, x, n->out, N, st);
    if (rc) return rc;
    const size_t P0 = (size_t)N * n->H * n->W;
    ARECGB_CUDA(cudaMemsetAsync(n->grads, 0, sizeof(float) * n->nparams, st));
    if (n->loss_levels > 0)
        multiscale_loss(n->out, target, n->pyr, n->dout, n->partials, N, n->H, n->W,
                        n->loss_levels, n->loss_ratio, 1.f / (float)P0, kLossBlocks, st);
    else
        mse(n->out, target, n->dout, n->partials, P0, 1.f / (float)P0, kLossBlocks, st);
    if ((rc = backward(n, n->dout, st))) return rc;
    n->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - powf(b1, (float)n->step), bc2 = 1.f - powf(b2, (float)n->step);
    adamw(n->params, n->grads, n->m, n->v, n->nparams, lr, b1, b2, 1e-8f, wd, bc1, bc2, st);
    n->mirrors_fresh = false;
    if ((rc = refresh_mirrors(n, st))) return rc;
    if (loss) {
        ARECGB_CUDA(cudaMemcpyAsync(n->h_partials, n->partials, sizeof(double) * kLossBlocks,
                                    cudaMemcpyDeviceToHost, st));
        if ((rc = check_err(n, st, "unet_train_step"))) return rc;
        double s = 0.0;
        for (int i = 0; i < kLossBlocks; i++) s += n->h_partials[i];
        *loss = s / (double)P0;
    }
    return 0;
}

// Warm start of a whole volume: x0 = s * net(x_early / s) slice by slice in
// chunks of the net's batch, s = RMS of x_early over the cylinder (so the
// network sees inputs of unit scale whatever the attenuation units).
static int warm_start(const Plan *p, Net *n, const float *x_early, float *x0, float *img_in,
                      float *img_out, cudaStream_t st) {
    if (n->H < p->nx || n->W < p->nx || n->H != n->W) {
        set_error("warm_start: the network's image size must be square and at least the "
                  "cylinder's width (" + std::to_string(p->nx) + ")");
        return ARECGB_ERR_ARG;
    }
    // RMS over all slices
    const int nb = 1024;
    double *part = nullptr;
    std::vector<double> hp(nb);
    ARECGB_CUDA(cudaMallocAsync(&part, sizeof(double) * nb, st));
    sumsq_partial(x_early, (size_t)p->nrays * p->ys, part, nb, st);
    count_launches(1);
    ARECGB_CUDA(cudaMemcpyAsync(hp.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
    ARECGB_CUDA(cudaFreeAsync(part, st));
    ARECGB_CUDA(cudaStreamSynchronize(st));
    double ss = 0.0;
    for (double v : hp) ss += v;
    const double rms = std::sqrt(ss / ((double)p->nrays * p->ny));
    if (!(rms > 0.0)) {  // zero input: the guess is zero too
        ARECGB_CUDA(cudaMemsetAsync(x0, 0, sizeof(float) * p->nrays * p->ys, st));
        return 0;
    }
    if (x0 != x_early)
        ARECGB_CUDA(cudaMemsetAsync(x0, 0, sizeof(float) * p->nrays * p->ys, st));
    const int npad = n->H;
    for (int y0 = 0; y0 < p->ny; y0 += n->maxN) {
        const int B = std::min(n->maxN, p->ny - y0);
        cyl_to_img(x_early, p->d_rows, img_in, p->nx, npad, p->ys, y0, B, (float)(1.0 / rms), st);
        int rc = forward(n, img_in, img_out, B, st);
        if (rc) return rc;
        img_to_cyl(img_out, p->d_rows, x0, p->nx, npad, p->ys, y0, B, (float)rms, st);
        count_launches(2);
    }
    ARECGB_CUDA(cudaGetLastError());
    return check_err(n, st, "warm_start");
}

}  // namespace unet
}  // namespace arecgb

using arecgb::unet::Net;

struct arecgb_unet;  // opaque handle = Net
static Net *N_(arecgb_unet *p) { return reinterpret_cast<Net *>(p); }

extern "C" {

int arecgb_unet_create(arecgb_unet **net, int height, int width, int max_batch, int train,
                       unsigned long long seed) {
    if (!net) {
        arecgb::set_error("arecgb_unet_create: null handle");
        return ARECGB_ERR_ARG;
    }
    Net *n = nullptr;
    int rc = arecgb::unet::create(&n, height, width, max_batch, train, seed);
    *net = reinterpret_cast<arecgb_unet *>(n);
    return rc;
}

int arecgb_unet_destroy(arecgb_unet *net) {
    arecgb::unet::destroy(N_(net));
    return 0;
}

long long arecgb_unet_num_params(const arecgb_unet *net) {
    return net ? (long long)reinterpret_cast<const Net *>(net)->nparams : 0;
}

int arecgb_unet_layer_offsets(const arecgb_unet *net, long long *w_off, long long *b_off,
                              int *cin, int *cout) {
    if (!net) return ARECGB_ERR_ARG;
    const Net *n = reinterpret_cast<const Net *>(net);
    for (int l = 0; l < arecgb::unet::NL; l++) {
        if (w_off) w_off[l] = (long long)n->woff[l];
        if (b_off) b_off[l] = (long long)n->boff[l];
        if (cin) cin[l] = arecgb::unet::kCin[l];
        if (cout) cout[l] = arecgb::unet::kCout[l];
    }
    return arecgb::unet::NL;
}

int arecgb_unet_get_params(const arecgb_unet *net, float *d_params, void *stream) {
    if (!net || !d_params) return ARECGB_ERR_ARG;
    const Net *n = reinterpret_cast<const Net *>(net);
    ARECGB_CUDA(cudaMemcpyAsync(d_params, n->params, sizeof(float) * n->nparams,
                                cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return 0;
}

int arecgb_unet_set_params(arecgb_unet *net, const float *d_params, void *stream) {
    if (!net || !d_params) return ARECGB_ERR_ARG;
    Net *n = N_(net);
    ARECGB_CUDA(cudaMemcpyAsync(n->params, d_params, sizeof(float) * n->nparams,
                                cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    if (n->train) {
        ARECGB_CUDA(cudaMemsetAsync(n->m, 0, sizeof(float) * n->nparams, (cudaStream_t)stream));
        ARECGB_CUDA(cudaMemsetAsync(n->v, 0, sizeof(float) * n->nparams, (cudaStream_t)stream));
        n->step = 0;
    }
    return arecgb::unet::refresh_mirrors(n, (cudaStream_t)stream);
}

int arecgb_unet_forward(arecgb_unet *net, const float *d_in, float *d_out, int n_images,
                        void *stream) {
    if (!net || !d_in || !d_out || n_images < 1 || n_images > N_(net)->maxN) {
        arecgb::set_error("arecgb_unet_forward: bad arguments (batch above the net's maximum?)");
        return ARECGB_ERR_ARG;
    }
    int rc = arecgb::unet::forward(N_(net), d_in, d_out, n_images, (cudaStream_t)stream);
    if (rc) return rc;
    return arecgb::unet::check_err(N_(net), (cudaStream_t)stream, "arecgb_unet_forward");
}

int arecgb_unet_backward(arecgb_unet *net, const float *d_dout, float *d_grads, void *stream) {
    if (!net || !d_dout || !N_(net)->train || !N_(net)->lastN) {
        arecgb::set_error("arecgb_unet_backward: needs a training net and a forward first");
        return ARECGB_ERR_ARG;
    }
    Net *n = N_(net);
    cudaStream_t st = (cudaStream_t)stream;
    ARECGB_CUDA(cudaMemsetAsync(n->grads, 0, sizeof(float) * n->nparams, st));
    int rc = arecgb::unet::backward(n, d_dout, st);
    if (rc) return rc;
    if (d_grads)
        ARECGB_CUDA(cudaMemcpyAsync(d_grads, n->grads, sizeof(float) * n->nparams,
                                    cudaMemcpyDeviceToDevice, st));
    return arecgb::unet::check_err(n, st, "arecgb_unet_backward");
}

int arecgb_unet_train_step(arecgb_unet *net, const float *d_in, const float *d_target,
                           int n_images, float lr, float weight_decay, double *loss,
                           void *stream) {
    if (!net || !d_in || !d_target || !N_(net)->train || n_images < 1 ||
        n_images > N_(net)->maxN) {
        arecgb::set_error("arecgb_unet_train_step: bad arguments");
        return ARECGB_ERR_ARG;
    }
    return arecgb::unet::train_step(N_(net), d_in, d_target, n_images, lr, weight_decay, loss,
                                    (cudaStream_t)stream);
}

int arecgb_unet_images_from_volume(const arecgb_plan *plan, const float *d_vol, float *d_img,
                                   int npad, int y0, int count, float scale, void *stream) {
    const arecgb::Plan *p = reinterpret_cast<const arecgb::Plan *>(plan);
    if (!p || !d_vol || !d_img || npad < p->nx || y0 < 0 || count < 0 || y0 + count > p->ny) {
        arecgb::set_error("arecgb_unet_images_from_volume: bad arguments");
        return ARECGB_ERR_ARG;
    }
    arecgb::unet::cyl_to_img(d_vol, p->d_rows, d_img, p->nx, npad, p->ys, y0, count, scale,
                             (cudaStream_t)stream);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

int arecgb_unet_images_to_volume(const arecgb_plan *plan, const float *d_img, float *d_vol,
                                 int npad, int y0, int count, float scale, void *stream) {
    const arecgb::Plan *p = reinterpret_cast<const arecgb::Plan *>(plan);
    if (!p || !d_vol || !d_img || npad < p->nx || y0 < 0 || count < 0 || y0 + count > p->ny) {
        arecgb::set_error("arecgb_unet_images_to_volume: bad arguments");
        return ARECGB_ERR_ARG;
    }
    arecgb::unet::img_to_cyl(d_img, p->d_rows, d_vol, p->nx, npad, p->ys, y0, count, scale,
                             (cudaStream_t)stream);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

int arecgb_unet_set_loss(arecgb_unet *net, int levels, float ratio) {
    Net *n = N_(net);
    if (!n || !n->train || levels < 0 || !(ratio > 0.f) || (levels > 0 &&
        (n->H % (1 << levels) || n->W % (1 << levels)))) {
        arecgb::set_error("arecgb_unet_set_loss: needs a training net, levels >= 0 with H and W "
                          "divisible by 2^levels, ratio > 0");
        return ARECGB_ERR_ARG;
    }
    n->loss_levels = levels;
    n->loss_ratio = ratio;
    return 0;
}

int arecgb_unet_shape(const arecgb_unet *net, int *height, int *width, int *max_batch) {
    const Net *n = reinterpret_cast<const Net *>(net);
    if (!n) {
        arecgb::set_error("arecgb_unet_shape: null network");
        return ARECGB_ERR_ARG;
    }
    if (height) *height = n->H;
    if (width) *width = n->W;
    if (max_batch) *max_batch = n->maxN;
    return 0;
}

int arecgb_warm_start(const arecgb_plan *plan, arecgb_unet *net, const float *d_x_early,
                      float *d_x0, float *d_img_in, float *d_img_out, void *stream) {
    const arecgb::Plan *p = reinterpret_cast<const arecgb::Plan *>(plan);
    if (!p || !net || !d_x_early || !d_x0 || !d_img_in || !d_img_out) {
        arecgb::set_error("arecgb_warm_start: null argument");
        return ARECGB_ERR_ARG;
    }
    return arecgb::unet::warm_start(p, N_(net), d_x_early, d_x0, d_img_in, d_img_out,
                                    (cudaStream_t)stream);
}

}  // extern "C"
