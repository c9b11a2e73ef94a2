// Layout conversion, FP64 reductions and the element-wise solver updates.
// All of these are HBM-bound: grid-stride loops over float4 where the layout
// allows, sized to a multiple of the SM count.
#include "arec_internal.cuh"
#include "arec_vector.cuh"

#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <cmath>

namespace arecgb {

// ---------------------------------------------------------------------------
// Sinogram layout: reference [na][ny][nx]  <->  device [na][nx][ys].
// 32x32 tiles through shared memory; both sides coalesced.
__global__ void __launch_bounds__(256)
    k_sino_to_dev(const float *__restrict__ in, float *__restrict__ out, int ny, int nx, int ys) {
    __shared__ float t[32][33];
    const int a = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const float *ia = in + (size_t)a * ny * nx;
    float *oa = out + (size_t)a * nx * ys;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int y = y0 + j, x = x0 + threadIdx.x;
        t[j][threadIdx.x] = (y < ny && x < nx) ? ia[(size_t)y * nx + x] : 0.f;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = x0 + j, y = y0 + threadIdx.x;
        if (x < nx && y < ys) oa[(size_t)x * ys + y] = t[threadIdx.x][j];
    }
}

__global__ void __launch_bounds__(256)
    k_sino_to_ref(const float *__restrict__ in, float *__restrict__ out, int ny, int nx, int ys) {
    __shared__ float t[32][33];
    const int a = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const float *ia = in + (size_t)a * nx * ys;
    float *oa = out + (size_t)a * ny * nx;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int x = x0 + j, y = y0 + threadIdx.x;
        t[j][threadIdx.x] = (x < nx && y < ny) ? ia[(size_t)x * ys + y] : 0.f;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int y = y0 + j, x = x0 + threadIdx.x;
        if (y < ny && x < nx) oa[(size_t)y * nx + x] = t[threadIdx.x][j];
    }
}

int sino_to_device_layout(const float *d_ref, float *d_dev, int na, int ny, int nx, int ys,
                          cudaStream_t st) {
    if (na <= 0 || ny <= 0 || nx <= 0 || ys < ny || na > 65535) {
        set_error("sino_to_device_layout: bad shape");
        return ARECGB_ERR_ARG;
    }
    dim3 grid((nx + 31) / 32, (ys + 31) / 32, na);
    k_sino_to_dev<<<grid, dim3(32, 8), 0, st>>>(d_ref, d_dev, ny, nx, ys);
    ARECGB_CUDA(cudaGetLastError());
    return ARECGB_OK;
}

int sino_to_reference_layout(const float *d_dev, float *d_ref, int na, int ny, int nx, int ys,
                             cudaStream_t st) {
    if (na <= 0 || ny <= 0 || nx <= 0 || ys < ny || na > 65535) {
        set_error("sino_to_reference_layout: bad shape");
        return ARECGB_ERR_ARG;
    }
    dim3 grid((nx + 31) / 32, (ny + 31) / 32, na);
    k_sino_to_ref<<<grid, dim3(32, 8), 0, st>>>(d_dev, d_ref, ny, nx, ys);
    ARECGB_CUDA(cudaGetLastError());
    return ARECGB_OK;
}

// ---------------------------------------------------------------------------
// Reductions.  Partial sums are combined in a fixed order, so results are
// reproducible run to run.
__global__ void __launch_bounds__(256) k_reduce_partials(const double *__restrict__ p, int n,
                                                         double *__restrict__ out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += p[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

int reduce_partials(const double *d_partials, int n, double *d_out, cudaStream_t st) {
    k_reduce_partials<<<1, 256, 0, st>>>(d_partials, n, d_out);
    ARECGB_CUDA(cudaGetLastError());
    return ARECGB_OK;
}

// sum(v*v): float products accumulated in double (reference areccgls.cpp:390-391).
__global__ void __launch_bounds__(256) k_sumsq(const float *__restrict__ v, size_t n,
                                               double *__restrict__ partials) {
    __shared__ double red[8];
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256)
        s += (double)__fmul_rn(v[i], v[i]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; w++) t += red[w];
        partials[blockIdx.x] = t;
    }
}

// sum(q*q*w): float products accumulated in double (areccgls_stat.cpp:651-652).
__global__ void __launch_bounds__(256) k_wsumsq(const float *__restrict__ v,
                                                const float *__restrict__ w, size_t n,
                                                double *__restrict__ partials) {
    __shared__ double red[8];
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256)
        s += (double)__fmul_rn(__fmul_rn(v[i], v[i]), w[i]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < 8; k++) t += red[k];
        partials[blockIdx.x] = t;
    }
}

// Statistical weights w = expf(-b) times the Tukey window (alpha 0.5) along the
// detector (init_weights, areccgls_stat.cpp:12-46; tukey_filter_x_inplace,
// imagetools.cpp:369-391); device sinogram layout [angle][bin][ys].
__global__ void __launch_bounds__(256) k_stat_weights(const float *__restrict__ b,
                                                      const double *__restrict__ hx,
                                                      float *__restrict__ w, size_t n, int nx,
                                                      int ys) {
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const int bin = (int)((i / ys) % nx);
        w[i] = (float)((double)expf(-b[i]) * hx[bin]);
    }
}

// s = (b - q) w, or s = b w when q is null (areccgls_stat.cpp:604-610).
__global__ void __launch_bounds__(256) k_sub_w(const float *__restrict__ b,
                                               const float *__restrict__ q,
                                               const float *__restrict__ w, float *__restrict__ s,
                                               size_t n) {
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const float r = q ? b[i] - q[i] : b[i];
        s[i] = r * w[i];
    }
}

int sumsq_partials(const float *d_v, size_t n, double *d_partials, int nblocks, cudaStream_t st) {
    k_sumsq<<<nblocks, 256, 0, st>>>(d_v, n, d_partials);
    ARECGB_CUDA(cudaGetLastError());
    return ARECGB_OK;
}

// ---------------------------------------------------------------------------
// CGLS (reference cyl_cgls_SQ, AREC3D/AREC3D/areccgls.cpp:375-456).  The scalar
// state lives in device memory; every kernel of an iteration returns at once
// when the solve has finished, so extra queued iterations cost nothing.

// p = g (first iteration) or p = g + beta*p, evaluated in double, stored float
// (areccgls.cpp:376-384).
__global__ void __launch_bounds__(256) k_cgls_p(SolveState *S, const float *__restrict__ g,
                                                float *__restrict__ p, size_t n4) {
    if (S->done) return;
    const bool first = S->iter == 1;
    const double beta = first ? 0.0 : S->gamma / S->gamma0;
    const float4 *g4 = reinterpret_cast<const float4 *>(g);
    float4 *p4 = reinterpret_cast<float4 *>(p);
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n4; i += (size_t)gridDim.x * 256) {
        float4 gv = g4[i];
        if (first) {
            p4[i] = gv;
        } else {
            float4 pv = p4[i];
            pv.x = (float)((double)gv.x + beta * (double)pv.x);
            pv.y = (float)((double)gv.y + beta * (double)pv.y);
            pv.z = (float)((double)gv.z + beta * (double)pv.z);
            pv.w = (float)((double)gv.w + beta * (double)pv.w);
            p4[i] = pv;
        }
    }
}

// alpha = gamma / ||A p||^2 (areccgls.cpp:389-396).
__global__ void k_cgls_alpha(SolveState *S) {
    if (S->done) return;
    S->alpha = S->gamma / S->qnorm2;
}

// x += alpha*p over the volume and s -= alpha*q over the sinogram, in double,
// stored float (areccgls.cpp:398-404).  One launch covers both arrays.
__global__ void __launch_bounds__(256) k_cgls_xs(SolveState *S, float *__restrict__ x,
                                                 const float *__restrict__ p, size_t nv4,
                                                 float *__restrict__ s,
                                                 const float *__restrict__ q, size_t ns4,
                                                 const float *__restrict__ w) {
    if (S->done) return;
    const double alpha = S->alpha;
    const size_t stride = (size_t)gridDim.x * 256;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < nv4 + ns4; i += stride) {
        float4 *dst;
        const float4 *src;
        double a;
        size_t j;
        if (i < nv4) {
            dst = reinterpret_cast<float4 *>(x);
            src = reinterpret_cast<const float4 *>(p);
            a = alpha;
            j = i;
        } else {
            dst = reinterpret_cast<float4 *>(s);
            src = reinterpret_cast<const float4 *>(q);
            a = -alpha;
            j = i - nv4;
        }
        float4 d = dst[j];
        const float4 v = src[j];
        if (w && i >= nv4) {
            // weighted residual: s - (alpha q) w (areccgls_stat.cpp:668-669)
            const float4 wt = reinterpret_cast<const float4 *>(w)[j];
            d.x = (float)((double)d.x + (a * (double)v.x) * (double)wt.x);
            d.y = (float)((double)d.y + (a * (double)v.y) * (double)wt.y);
            d.z = (float)((double)d.z + (a * (double)v.z) * (double)wt.z);
            d.w = (float)((double)d.w + (a * (double)v.w) * (double)wt.w);
        } else {
            d.x = (float)((double)d.x + a * (double)v.x);
            d.y = (float)((double)d.y + a * (double)v.y);
            d.z = (float)((double)d.z + a * (double)v.z);
            d.w = (float)((double)d.w + a * (double)v.w);
        }
        dst[j] = d;
    }
}

// New gamma, relative residual, best-iterate tracking and the stopping test
// (areccgls.cpp:409-453).
__global__ void k_cgls_gamma(SolveState *S, double *history) {
    if (S->done) return;
    S->gamma0 = S->gamma;
    S->gamma = S->gnorm2;
    const double rnorm = sqrt(S->gamma);
    const double rel = rnorm / S->denom;
    const int it = S->iter;
    if (history) history[it - 1] = rel;
    S->rel = rel;
    S->iterations = it;
    if (rnorm < S->rnorm_min) {
        S->rnorm_min = rnorm;
        S->iterbest = it;
        S->save = 1;
    }
    if (rel < (double)S->tol || it >= S->maxit) S->done = 1;
    S->iter = it + 1;
}

// xsave = x when the previous iteration improved on the best residual
// (areccgls.cpp:423-428).  Runs at the start of the next iteration (x is
// unchanged in between) and once more after the last one.
__global__ void __launch_bounds__(256) k_cgls_save(SolveState *S, const float *__restrict__ x,
                                                   float *__restrict__ xs, size_t n4) {
    if (!S->save) return;
    const float4 *x4 = reinterpret_cast<const float4 *>(x);
    float4 *s4 = reinterpret_cast<float4 *>(xs);
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n4; i += (size_t)gridDim.x * 256)
        s4[i] = x4[i];
}

__global__ void k_cgls_save_done(SolveState *S) { S->save = 0; }

// ---------------------------------------------------------------------------
// SIRT (reference cyl_sirt_SQ, AREC3D/AREC3D/arecsirt.cpp:277-362).

// First iteration: grad = A^T b; partial sums of float b*b and double grad^2
// (arecsirt.cpp:285-306).
__global__ void __launch_bounds__(256) k_sirt_first(const float *__restrict__ bvol,
                                                    float *__restrict__ grad, size_t n,
                                                    double *__restrict__ pb,
                                                    double *__restrict__ pr) {
    __shared__ double rb[8], rr[8];
    double sb = 0.0, sr = 0.0;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const float b = bvol[i];
        grad[i] = b;
        sb += (double)__fmul_rn(b, b);
        sr += (double)b * (double)b;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sb += __shfl_down_sync(0xffffffffu, sb, o);
        sr += __shfl_down_sync(0xffffffffu, sr, o);
    }
    if ((threadIdx.x & 31) == 0) {
        rb[threadIdx.x >> 5] = sb;
        rr[threadIdx.x >> 5] = sr;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tb = 0.0, tr = 0.0;
        for (int w = 0; w < 8; w++) {
            tb += rb[w];
            tr += rr[w];
        }
        pb[blockIdx.x] = tb;
        pr[blockIdx.x] = tr;
    }
}

// Later iterations: grad = bvol - pvol (float); partial sums of grad^2 in double
// (arecsirt.cpp:298-306).
__global__ void __launch_bounds__(256) k_sirt_grad(const float *__restrict__ bvol,
                                                   const float *__restrict__ pvol,
                                                   float *__restrict__ grad, size_t n,
                                                   double *__restrict__ pr) {
    __shared__ double rr[8];
    double sr = 0.0;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) {
        const float gv = __fsub_rn(bvol[i], pvol[i]);
        grad[i] = gv;
        sr += (double)gv * (double)gv;
    }
    for (int o = 16; o > 0; o >>= 1) sr += __shfl_down_sync(0xffffffffu, sr, o);
    if ((threadIdx.x & 31) == 0) rr[threadIdx.x >> 5] = sr;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0;
        for (int w = 0; w < 8; w++) tr += rr[w];
        pr[blockIdx.x] = tr;
    }
}

// x += lam*grad in float, product rounded before the sum (arecsirt.cpp:354-355).
__global__ void __launch_bounds__(256) k_sirt_update(float *__restrict__ x,
                                                     const float *__restrict__ grad, float lam,
                                                     size_t n) {
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256)
        x[i] = __fadd_rn(x[i], __fmul_rn(lam, grad[i]));
}

// ---------------------------------------------------------------------------
int grid_for(size_t n, int per_thread) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t want = (n / per_thread + 255) / 256;
    size_t cap = (size_t)sms * 8;
    if (want < 1) want = 1;
    return (int)(want < cap ? want : cap);
}

}  // namespace arecgb

// ===========================================================================
// Solver drivers.
namespace arecgb {

__global__ void k_sub(const float *__restrict__ a, const float *__restrict__ b,
                      float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256)
        out[i] = __fsub_rn(a[i], b[i]);
}

__global__ void k_cgls_init(SolveState *S, int maxit, float tol, double rnorm_ref) {
    S->gamma = S->gnorm2;
    S->gamma0 = 0.0;
    S->alpha = 0.0;
    S->rnorm0 = sqrt(S->gamma);
    S->denom = rnorm_ref > 0.0 ? rnorm_ref : S->rnorm0;
    S->rnorm_min = S->rnorm0;
    S->rel = 1.0;
    S->tol = tol;
    S->iter = 1;
    S->maxit = maxit;
    S->iterbest = maxit - 1;
    S->iterations = 0;
    S->done = maxit < 1 ? 1 : 0;
    S->save = 0;
}

static int ensure_workspace(Plan *p, int nvol, int nsin) {
    const size_t nv = vol_floats(p), ns = sin_floats(p);
    for (int i = 0; i < nvol; i++)
        if (!p->d_vol[i]) {
            ARECGB_CUDA(cudaMalloc(&p->d_vol[i], sizeof(float) * nv));
            ARECGB_CUDA(cudaMemset(p->d_vol[i], 0, sizeof(float) * nv));
        }
    for (int i = 0; i < nsin; i++)
        if (!p->d_sin[i]) {
            ARECGB_CUDA(cudaMalloc(&p->d_sin[i], sizeof(float) * ns));
            ARECGB_CUDA(cudaMemset(p->d_sin[i], 0, sizeof(float) * ns));
        }
    return ARECGB_OK;
}

constexpr int kRedBlocks = kSredBlocks;

int ensure_red(Plan *p) {
    if (!p->d_sred) ARECGB_CUDA(cudaMalloc(&p->d_sred, sizeof(double) * (2 * kSredBlocks + 2)));
    if (!p->h_sred && cudaMallocHost(&p->h_sred, sizeof(double) * 2) != cudaSuccess) {
        p->h_sred = nullptr;
        set_error("pinned allocation failed");
        return ARECGB_ERR_NOMEM;
    }
    return 0;
}

// One CGLS iteration (reference areccgls.cpp:375-456) as a fixed launch sequence.
static int cgls_iteration(Plan *p, SolveState *S, double *hist, float *x, float *s, float *q,
                          float *g, float *pd, float *xs, const float *w, cudaStream_t st) {
    const size_t nv = vol_floats(p), ns = sin_floats(p);
    const int gv = grid_for(nv, 16), gs = grid_for(nv + ns, 16);
    k_cgls_save<<<gv, 256, 0, st>>>(S, x, xs, nv / 4);
    k_cgls_save_done<<<1, 1, 0, st>>>(S);
    k_cgls_p<<<gv, 256, 0, st>>>(S, g, pd, nv / 4);
    int rc = forward_project(p, pd, q, w ? nullptr : &S->qnorm2, &S->done, st);
    if (rc) return rc;
    if (w) {  // ||A p||^2 weighted
        k_wsumsq<<<kRedBlocks, 256, 0, st>>>(q, w, ns, p->d_partials);
        rc = reduce_partials(p->d_partials, kRedBlocks, &S->qnorm2, st);
        if (rc) return rc;
        count_launches(2);
    }
    k_cgls_alpha<<<1, 1, 0, st>>>(S);
    k_cgls_xs<<<gs, 256, 0, st>>>(S, x, pd, nv / 4, s, q, ns / 4, w);
    rc = back_project(p, s, g, &S->gnorm2, &S->done, st);
    if (rc) return rc;
    k_cgls_gamma<<<1, 1, 0, st>>>(S, hist);
    count_launches(6);
    ARECGB_CUDA(cudaGetLastError());
    return ARECGB_OK;
}

// CGLS over n independent problems (one plan each, uneven shapes allowed).
// Per problem: s = b - A x0 (x0 = 0 unless warm), g = A^T s, gamma = ||g||^2
// (areccgls.cpp:323-372), launched eagerly with the first iteration (which
// also configures every kernel).  Then one CUDA graph captures one iteration
// of ALL problems, each problem a parallel branch, and the solve replays it;
// a problem that has met its stopping test turns its kernels into no-ops, and
// the host polls the n done flags with one copy after 1, 2, 4, 8, 8, ...
// iterations.  Finally the reference's best-iterate restore, per problem.
int cgls_batch(Plan *const *plans, const float *const *d_b, float *const *d_x, const int *warm,
               int n, int maxit, float tol, const double *rnorm_ref, double *const *hist_host,
               arecgb_solve_info *info, cudaStream_t st, const float *const *d_w) {
    if (n < 1 || !plans || !d_b || !d_x) {
        set_error("cgls: bad batch arguments");
        return ARECGB_ERR_ARG;
    }
    for (int i = 0; i < n; i++) {
        if (!plans[i] || !d_b[i] || !d_x[i]) {
            set_error("cgls: null plan or buffer in the batch");
            return ARECGB_ERR_ARG;
        }
        for (int j = 0; j < i; j++)
            if (plans[j] == plans[i]) {
                set_error("cgls: a plan appears twice in the batch (each needs its own workspace)");
                return ARECGB_ERR_ARG;
            }
        int rc = ensure_workspace(plans[i], 3, 2);
        if (rc) return rc;
    }
    const int cap = maxit > 0 ? maxit : 1;
    SolveState *S = nullptr, *H = nullptr;
    double *hist = nullptr;
    cudaStream_t cs = nullptr;
    std::vector<cudaStream_t> bs;
    std::vector<cudaEvent_t> ev;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = 0;
    long long per_iter = 0;
    auto fail = [&](cudaError_t e, const char *what) {
        set_error(std::string("cgls: ") + what + ": " + cudaGetErrorString(e));
        rc = cuda_status(e);
    };
    auto iteration = [&](int i, cudaStream_t s_) {
        Plan *p = plans[i];
        return cgls_iteration(p, S + i, hist + (size_t)i * cap, d_x[i], p->d_sin[0], p->d_sin[1],
                              p->d_vol[0], p->d_vol[1], p->d_vol[2], d_w ? d_w[i] : nullptr, s_);
    };
    // state, history, stream and events from the first plan's solver
    // scratch, grown when this batch needs more
    Plan *q0 = plans[0];
    cudaError_t e = cudaSuccess;
    const size_t s_bytes = sizeof(SolveState) * n, h_bytes = sizeof(double) * n * (size_t)cap;
    if (q0->cstate_bytes < s_bytes) {
        cudaFree(q0->d_cstate);
        if (q0->h_cstate) cudaFreeHost(q0->h_cstate);
        q0->d_cstate = q0->h_cstate = nullptr;
        q0->cstate_bytes = 0;
        e = cudaMalloc(&q0->d_cstate, s_bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&q0->h_cstate, s_bytes);
        if (e == cudaSuccess) q0->cstate_bytes = s_bytes;
    }
    if (e == cudaSuccess && q0->chist_bytes < h_bytes) {
        cudaFree(q0->d_chist);
        q0->d_chist = nullptr;
        q0->chist_bytes = 0;
        e = cudaMalloc(&q0->d_chist, h_bytes);
        if (e == cudaSuccess) q0->chist_bytes = h_bytes;
    }
    if (e == cudaSuccess && !q0->solve_stream)
        e = cudaStreamCreateWithFlags(&q0->solve_stream, cudaStreamNonBlocking);
    while (e == cudaSuccess && (int)q0->solve_ev.size() < n + 2) {
        cudaEvent_t x;
        e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
        if (e == cudaSuccess) q0->solve_ev.push_back(x);
    }
    while (e == cudaSuccess && n > 1 && (int)q0->solve_bs.size() < n) {
        cudaStream_t x;
        e = cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking);
        if (e == cudaSuccess) q0->solve_bs.push_back(x);
    }
    if (e == cudaSuccess) {
        S = static_cast<SolveState *>(q0->d_cstate);
        H = static_cast<SolveState *>(q0->h_cstate);
        hist = q0->d_chist;
        cs = q0->solve_stream;
        ev.assign(q0->solve_ev.begin(), q0->solve_ev.begin() + (n + 2));
        if (n > 1) bs.assign(q0->solve_bs.begin(), q0->solve_bs.begin() + n);
    } else {
        fail(e, "setup");
    }
    // the solve runs on cs, ordered after the caller's stream
    if (!rc) {
        e = cudaEventRecord(ev[0], st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev[0], 0);
        if (e == cudaSuccess) e = cudaMemsetAsync(S, 0, sizeof(SolveState) * n, cs);
        if (e != cudaSuccess) fail(e, "setup");
    }
    for (int i = 0; !rc && i < n; i++) {
        Plan *p = plans[i];
        const size_t nv = vol_floats(p), ns = sin_floats(p);
        float *s_ = p->d_sin[0], *q = p->d_sin[1], *g = p->d_vol[0];
        const float *wi = d_w ? d_w[i] : nullptr;
        if (warm && warm[i]) {
            rc = forward_project(p, d_x[i], q, nullptr, nullptr, cs);
            if (rc) break;
            if (wi)
                k_sub_w<<<grid_for(ns, 16), 256, 0, cs>>>(d_b[i], q, wi, s_, ns);
            else
                k_sub<<<grid_for(ns, 16), 256, 0, cs>>>(d_b[i], q, s_, ns);
            count_launches(1);
        } else {
            cudaMemsetAsync(d_x[i], 0, sizeof(float) * nv, cs);
            if (wi) {
                k_sub_w<<<grid_for(ns, 16), 256, 0, cs>>>(d_b[i], nullptr, wi, s_, ns);
                count_launches(1);
            } else {
                cudaMemcpyAsync(s_, d_b[i], sizeof(float) * ns, cudaMemcpyDeviceToDevice, cs);
            }
        }
        rc = back_project(p, s_, g, &S[i].gnorm2, nullptr, cs);
        if (rc) break;
        k_cgls_init<<<1, 1, 0, cs>>>(S + i, maxit, tol, rnorm_ref ? rnorm_ref[i] : 0.0);
        count_launches(1);
    }
    // first iteration eagerly, then capture one iteration of every problem
    for (int i = 0; !rc && maxit > 0 && i < n; i++) rc = iteration(i, cs);
    int launched = maxit > 0 ? 1 : 0;
    if (!rc && maxit > 1) {
        const long long c0 = launch_count();
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            fail(e, "stream capture");
        } else {
            if (n == 1) {
                rc = iteration(0, cs);
            } else {
                cudaEventRecord(ev[1], cs);
                for (int i = 0; !rc && i < n; i++) {
                    cudaStreamWaitEvent(bs[i], ev[1], 0);
                    rc = iteration(i, bs[i]);
                    cudaEventRecord(ev[2 + i], bs[i]);
                    cudaStreamWaitEvent(cs, ev[2 + i], 0);
                }
            }
            e = cudaStreamEndCapture(cs, &graph);
            if (!rc && e != cudaSuccess) fail(e, "stream capture");
            if (!rc) {
                e = cudaGraphInstantiate(&exec, graph, 0);
                if (e != cudaSuccess) fail(e, "graph instantiation");
            }
        }
        per_iter = launch_count() - c0;
        // the captured launches run only when the graph is replayed (counted there)
        count_launches(-(int)per_iter);
    }
    // replay until every problem has stopped
    int batch = 1;
    while (!rc) {
        e = cudaMemcpyAsync(H, S, sizeof(SolveState) * n, cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
        if (e != cudaSuccess) {
            fail(e, "poll");
            break;
        }
        bool all = true;
        for (int i = 0; i < n; i++) all = all && H[i].done;
        if (all || launched >= maxit) break;
        const int nb = std::min(batch, maxit - launched);
        for (int k = 0; k < nb && !rc; k++) {
            e = cudaGraphLaunch(exec, cs);
            if (e != cudaSuccess) fail(e, "graph launch");
            count_launches((int)per_iter);
        }
        launched += nb;
        batch = std::min(batch * 2, 8);
    }
    // flush pending best-iterate copies, then restore them where the reference would
    for (int i = 0; !rc && i < n; i++) {
        Plan *p = plans[i];
        const size_t nv = vol_floats(p);
        k_cgls_save<<<grid_for(nv, 16), 256, 0, cs>>>(S + i, d_x[i], p->d_vol[2], nv / 4);
        k_cgls_save_done<<<1, 1, 0, cs>>>(S + i);
        count_launches(2);
    }
    if (!rc) {
        e = cudaMemcpyAsync(H, S, sizeof(SolveState) * n, cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
        if (e != cudaSuccess) fail(e, "final state");
    }
    for (int i = 0; !rc && i < n; i++) {
        Plan *p = plans[i];
        if (H[i].iterbest < maxit - 1)
            cudaMemcpyAsync(d_x[i], p->d_vol[2], sizeof(float) * vol_floats(p),
                            cudaMemcpyDeviceToDevice, cs);
        if (hist_host && hist_host[i] && H[i].iterations > 0)
            cudaMemcpyAsync(hist_host[i], hist + (size_t)i * cap,
                            sizeof(double) * std::min(H[i].iterations, cap), cudaMemcpyDeviceToHost,
                            cs);
        if (info) {
            info[i].iterations = H[i].iterations;
            info[i].iterbest = H[i].iterbest;
            info[i].restarts = 0;
            info[i].status = 0;
            info[i].lam_final = 0.f;
            info[i].rnorm0 = H[i].rnorm0;
            info[i].rel_final = H[i].rel;
        }
    }
    if (!rc) {
        e = cudaStreamSynchronize(cs);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) fail(e, "finish");
    }
    // the caller's stream continues after the solve
    if (cs && !ev.empty()) {
        cudaEventRecord(ev[0], cs);
        cudaStreamWaitEvent(st, ev[0], 0);
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamSynchronize(cs);  // the scratch is reused by the next solve
    return rc;
}

int cgls(Plan *p, const float *d_b, float *d_x, int warm, int maxit, float tol, double rnorm_ref,
         double *hist_host, arecgb_solve_info *info, cudaStream_t st) {
    return cgls_batch(&p, &d_b, &d_x, &warm, 1, maxit, tol, &rnorm_ref, &hist_host, info, st,
                      nullptr);
}

// Statistically weighted CGLS (cyl_cgls[_KB|_SQ]_stat, areccgls_stat.cpp:49-731):
// the CGLS above with w = stat weights of b on the residual and in ||A p||^2;
// the stopping test is relative to the initial weighted gradient norm.
int cgls_stat(Plan *p, const float *d_b, float *d_x, int warm, int maxit, float tol,
              double *hist_host, arecgb_solve_info *info, cudaStream_t st) {
    const size_t ns = sin_floats(p);
    if (!p->d_w) ARECGB_CUDA(cudaMalloc(&p->d_w, sizeof(float) * ns));
    std::vector<double> hx(p->nx);
    const double alpha = 0.5, pi = std::atan(1.0) * 4.0;
    const double xa = 0.5 * alpha * (p->nx - 1), xb = (1.0 - 0.5 * alpha) * (p->nx - 1);
    const double A = 2.0 * pi / alpha;
    for (int x = 0; x < p->nx; x++) {
        const double va = 0.5 * (1.0 + std::cos(A * (1.0 * x / (p->nx - 1) - alpha / 2)));
        const double vb = 0.5 * (1.0 + std::cos(A * (1.0 * x / (p->nx - 1) - 1.0 + alpha / 2)));
        hx[x] = x < xa ? va : (x > xb ? vb : 1.0);
    }
    double *d_hx = nullptr;
    ARECGB_CUDA(cudaMallocAsync(&d_hx, sizeof(double) * p->nx, st));
    ARECGB_CUDA(cudaMemcpyAsync(d_hx, hx.data(), sizeof(double) * p->nx, cudaMemcpyHostToDevice, st));
    k_stat_weights<<<grid_for(ns, 16), 256, 0, st>>>(d_b, d_hx, p->d_w, ns, p->nx, p->ys);
    count_launches(1);
    ARECGB_CUDA(cudaFreeAsync(d_hx, st));
    ARECGB_CUDA(cudaStreamSynchronize(st));  // hx is host memory
    const float *w = p->d_w;
    const double zero = 0.0;
    return cgls_batch(&p, &d_b, &d_x, &warm, 1, maxit, tol, &zero, &hist_host, info, st, &w);
}

// SIRT with the reference's control flow (arecsirt.cpp:267-362): the step size
// is halved and the solve restarted from zero (at most 20 times) whenever the
// relative gradient norm grows; the squared norm of A^T b keeps accumulating
// across restarts as in the reference.  The decision needs the norms on the
// host, one small copy per iteration.
int sirt(Plan *p, const float *d_b, float *d_x, float lam, int maxit, float tol,
         double *hist_host, arecgb_solve_info *info, int verbose, cudaStream_t st) {
    int rc = ensure_workspace(p, 3, 1);
    if (rc) return rc;
    const size_t nv = vol_floats(p);
    float *bvol = p->d_vol[0], *pvol = p->d_vol[1], *grad = p->d_vol[2], *proj = p->d_sin[0];
    if ((rc = ensure_red(p))) return rc;
    double *red = p->d_sred, *h_red = p->h_sred;
    double relnrm0 = 1.00001, bnorm2 = 0.0, bnorm = 0.0, atb_norm = 0.0, rel_last = 0.0;
    int restarts = 0, iter = 1, count = 0;
    const int nblk = std::min(kRedBlocks, grid_for(nv, 8));
    cudaMemsetAsync(d_x, 0, sizeof(float) * nv, st);
    while (iter <= maxit) {
        double rn2;
        if (iter == 1) {
            if (restarts == 0) {
                rc = back_project(p, d_b, bvol, nullptr, nullptr, st);
                if (rc) break;
            }
            k_sirt_first<<<nblk, 256, 0, st>>>(bvol, grad, nv, red, red + kRedBlocks);
            k_reduce_partials<<<1, 256, 0, st>>>(red, nblk, red + 2 * kRedBlocks);
            k_reduce_partials<<<1, 256, 0, st>>>(red + kRedBlocks, nblk, red + 2 * kRedBlocks + 1);
            count_launches(3);
        } else {
            rc = forward_project(p, d_x, proj, nullptr, nullptr, st);
            if (rc) break;
            rc = back_project(p, proj, pvol, nullptr, nullptr, st);
            if (rc) break;
            k_sirt_grad<<<nblk, 256, 0, st>>>(bvol, pvol, grad, nv, red + kRedBlocks);
            k_reduce_partials<<<1, 256, 0, st>>>(red + kRedBlocks, nblk, red + 2 * kRedBlocks + 1);
            count_launches(2);
        }
        cudaError_t e = cudaMemcpyAsync(h_red, red + 2 * kRedBlocks, sizeof(double) * 2,
                                        cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(std::string("sirt: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
            break;
        }
        if (iter == 1) {
            if (restarts == 0) atb_norm = std::sqrt(h_red[0]);
            bnorm2 += h_red[0];
            bnorm = std::sqrt(bnorm2);
        }
        rn2 = h_red[1];
        const double rnorm = std::sqrt(rn2);
        const double relnrm = rnorm / bnorm;
        rel_last = relnrm;
        if (hist_host && count < maxit) hist_host[count] = relnrm;
        count++;
        if (verbose)
            printf("iter = %3d, rnorm / bnorm = %11.3e, rnorm = %11.3e\n", iter, relnrm, rnorm);
        if (relnrm > relnrm0) {
            if (restarts > 20) {
                if (verbose) printf("Failure to converge, even with lam = %11.3e\n", lam);
                break;
            }
            ++restarts;
            iter = 1;
            lam /= 2.0;
            relnrm0 = 1.0001;
            cudaMemsetAsync(d_x, 0, sizeof(float) * nv, st);
            if (verbose) printf("reducing lam to %11.3e, restarting\n", lam);
            continue;
        }
        if (relnrm < tol || relnrm > relnrm0) {
            if (verbose) {
                printf("Terminating with rnorm/bnorm = %11.3e, tol = %11.3e, ", relnrm, tol);
                printf("relnrm0 = %11.3e\n", relnrm0);
            }
            break;
        }
        relnrm0 = relnrm;
        k_sirt_update<<<grid_for(nv, 8), 256, 0, st>>>(d_x, grad, lam, nv);
        count_launches(1);
        ++iter;
    }
    if (rc == 0) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(std::string("sirt: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    if (info) {
        info->iterations = count;
        info->iterbest = 0;
        info->restarts = restarts;
        info->status = 0;
        info->lam_final = lam;
        info->rnorm0 = atb_norm;  // ||A^T b||: the CGLS denominator for a warm start
        info->rel_final = rel_last;
    }
    return rc;
}

}  // namespace arecgb
