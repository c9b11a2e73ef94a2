// Preprocessing of the image stack before reconstruction (reference
// AREC3D/AREC3D/AREC3D.cpp:81,105):
//
//   take_log        arecImageTakeLog       arecImage.cpp:358-381
//   periodic_decomp periodicDecomposition  imagetools.cpp:77-114
//                     with makePeriodicSlice imagetools.cpp:17-75
//
// Periodic-plus-smooth decomposition (Moisan 2011), per image d [ny][nx]:
//   v    = the boundary jumps of d (rows 0 and ny-1, columns 0 and nx-1; the
//          column jumps are added onto the row jumps at the corners, in float,
//          as the reference builds v)
//   S    = IDFT2( DFT2(v) / (2 cos(2 pi i/nx) + 2 cos(2 pi j/ny) - 4) ) / (nx ny),
//          the zero frequency set to 0
//   d   -= exp(-dist^2 / 50) * S,   dist = distance to the nearest border.
// v is zero off the border, so DFT2(v) needs only 1-D transforms of its two
// rows and of its interior column jumps:
//   V[j,i] = Rtop[i] + e^{+2 pi i j/ny} Rbot[i] + Ccol[j] (1 - e^{+2 pi i i/nx})
// (FP64 direct sums; any nx, ny).  The inverse transform is two complex
// matrix products on the CUDA cores in FP32, over the half spectrum
// i = 0 .. nx/2 (S is real, the spectrum Hermitian):
//   T[y,i] = sum_j W[j,i] e^{+2 pi i j y/ny}                (k_pd_cols)
//   S[y,x] = (sum_i c_i Re(T[y,i] e^{+2 pi i i x/nx})) / (nx ny),
//            c_0 = c_{nx/2, nx even} = 1, else 2            (k_pd_rows, with the
//                                                            border update fused)
// Any size; twiddles are host tables computed in double.
#include <math.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "arec_internal.cuh"

namespace arecgb {

namespace {

__global__ void k_take_log(float *x, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float v = x[i];
        // -log(v) of the float overload, as the double value rounded to float
        x[i] = v > 0.0f ? -(float)log((double)v) : 0.0f;
    }
}

struct PdTables {
    const double2 *ex, *ey;  // e^{+2 pi i k / n} for k < nx, k < ny (double)
    const float2 *fx, *fy;   // the same in float
};

// Boundary jumps and their 1-D DFTs, FP64, one block per slice.
//   out[z]: Rtop[0..nh), Rbot[0..nh), Ccol[0..ny)   (double2)
__global__ void k_pd_edges(const float *__restrict__ d, int nx, int ny, int nh, PdTables tb,
                           double2 *__restrict__ out) {
    const int z = blockIdx.x;
    const float *im = d + (size_t)z * nx * ny;
    const float *top = im, *bot = im + (size_t)(ny - 1) * nx;
    double2 *R0 = out + (size_t)z * (2 * nh + ny), *R1 = R0 + nh, *Cc = R1 + nh;
    // v on row 0 and row ny-1 (with the corner column jumps, float adds)
    auto vtop = [&](int x) -> float {
        float v = __fsub_rn(bot[x], top[x]);
        if (x == 0) v = __fadd_rn(v, __fsub_rn(top[nx - 1], top[0]));
        if (x == nx - 1) v = __fadd_rn(v, __fsub_rn(top[0], top[nx - 1]));
        return v;
    };
    auto vbot = [&](int x) -> float {
        float v = __fsub_rn(top[x], bot[x]);
        if (x == 0) v = __fadd_rn(v, __fsub_rn(bot[nx - 1], bot[0]));
        if (x == nx - 1) v = __fadd_rn(v, __fsub_rn(bot[0], bot[nx - 1]));
        return v;
    };
    // forward DFT: e^{-2 pi i k x / n} = conj(table[(k x) mod n])
    for (int i = threadIdx.x; i < nh; i += blockDim.x) {
        double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
        for (int x = 0; x < nx; x++) {
            const double2 w = tb.ex[(int)(((long long)i * x) % nx)];
            const double a = vtop(x), b = vbot(x);
            ar += a * w.x;
            ai -= a * w.y;
            br += b * w.x;
            bi -= b * w.y;
        }
        R0[i] = make_double2(ar, ai);
        R1[i] = make_double2(br, bi);
    }
    for (int j = threadIdx.x; j < ny; j += blockDim.x) {
        double cr = 0.0, ci = 0.0;
        for (int y = 1; y < ny - 1; y++) {
            const double2 w = tb.ey[(int)(((long long)j * y) % ny)];
            const double c = __fsub_rn(im[(size_t)y * nx + nx - 1], im[(size_t)y * nx]);
            cr += c * w.x;
            ci -= c * w.y;
        }
        Cc[j] = make_double2(cr, ci);
    }
}

// W[j][i] = V[j,i] / D[j,i] (float), W[0][0] = 0; i < nh.
__global__ void k_pd_w(const double2 *__restrict__ edges, int nx, int ny, int nh, PdTables tb,
                       float2 *__restrict__ W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, z = blockIdx.z;
    if (i >= nh) return;
    const double2 *R0 = edges + (size_t)z * (2 * nh + ny), *R1 = R0 + nh, *Cc = R1 + nh;
    const double2 ej = tb.ey[j], ei = tb.ex[i];
    const double2 r0 = R0[i], r1 = R1[i], c = Cc[j];
    // V = r0 + ej r1 + c (1 - ei)
    const double vr = r0.x + (ej.x * r1.x - ej.y * r1.y) + (c.x * (1.0 - ei.x) + c.y * ei.y);
    const double vi = r0.y + (ej.x * r1.y + ej.y * r1.x) + (c.y * (1.0 - ei.x) - c.x * ei.y);
    const double D = (2 * ei.x + 2 * ej.x) - 4;
    float2 w = make_float2((float)(vr / D), (float)(vi / D));
    if (i == 0 && j == 0) w = make_float2(0.0f, 0.0f);
    W[((size_t)z * ny + j) * nh + i] = w;
}

constexpr int kTile = 64, kKc = 16, kPdThreads = 256;

// T[y][i] = sum_j E_y[(j y) mod ny] W[j][i]: 64 x 64 tile of (y, i) per block,
// 4 x 4 per thread (rows ty + 16 m, columns tx + 16 n).
__global__ void __launch_bounds__(kPdThreads)
    k_pd_cols(const float2 *__restrict__ W, int ny, int nh, PdTables tb, float2 *__restrict__ T) {
    __shared__ float2 As[kKc][kTile], Bs[kKc][kTile];
    const int z = blockIdx.z, y0 = blockIdx.y * kTile, i0 = blockIdx.x * kTile;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const float2 *Wz = W + (size_t)z * ny * nh;
    float ar[4][4], ai[4][4];
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) ar[m][n] = ai[m][n] = 0.0f;
    for (int j0 = 0; j0 < ny; j0 += kKc) {
        for (int e = t; e < kKc * kTile; e += kPdThreads) {
            const int kk = e / kTile, c = e % kTile, j = j0 + kk;
            const int y = y0 + c, i = i0 + c;
            As[kk][c] = (j < ny && y < ny) ? tb.fy[(int)(((long long)j * y) % ny)]
                                           : make_float2(0.0f, 0.0f);
            Bs[kk][c] = (j < ny && i < nh) ? Wz[(size_t)j * nh + i] : make_float2(0.0f, 0.0f);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kKc; kk++) {
            float2 a[4], b[4];
#pragma unroll
            for (int m = 0; m < 4; m++) a[m] = As[kk][ty + 16 * m];
#pragma unroll
            for (int n = 0; n < 4; n++) b[n] = Bs[kk][tx + 16 * n];
#pragma unroll
            for (int m = 0; m < 4; m++)
#pragma unroll
                for (int n = 0; n < 4; n++) {
                    ar[m][n] = fmaf(a[m].x, b[n].x, ar[m][n]);
                    ar[m][n] = fmaf(-a[m].y, b[n].y, ar[m][n]);
                    ai[m][n] = fmaf(a[m].x, b[n].y, ai[m][n]);
                    ai[m][n] = fmaf(a[m].y, b[n].x, ai[m][n]);
                }
        }
        __syncthreads();
    }
    float2 *Tz = T + (size_t)z * ny * nh;
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const int y = y0 + ty + 16 * m, i = i0 + tx + 16 * n;
            if (y < ny && i < nh) Tz[(size_t)y * nh + i] = make_float2(ar[m][n], ai[m][n]);
        }
}

// S[y][x] = (sum_i c_i Re(T[y][i] E_x[(i x) mod nx])) / (nx ny), then
// d[y][x] -= exp(-dist^2/50) S[y][x] (double arithmetic, float result).
__global__ void __launch_bounds__(kPdThreads)
    k_pd_rows(const float2 *__restrict__ T, int nx, int ny, int nh, PdTables tb,
              float *__restrict__ d, float *__restrict__ s_out) {
    __shared__ float2 As[kKc][kTile + 1];  // padded: filled along kk
    __shared__ float2 Bs[kKc][kTile];
    const int z = blockIdx.z, y0 = blockIdx.y * kTile, x0 = blockIdx.x * kTile;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const float2 *Tz = T + (size_t)z * ny * nh;
    float acc[4][4];
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) acc[m][n] = 0.0f;
    for (int i0 = 0; i0 < nh; i0 += kKc) {
        for (int e = t; e < kKc * kTile; e += kPdThreads) {
            {  // A[i][y] = T[y][i], read along i (contiguous in T)
                const int kk = e % kKc, c = e / kKc, i = i0 + kk, y = y0 + c;
                As[kk][c] = (i < nh && y < ny) ? Tz[(size_t)y * nh + i] : make_float2(0.0f, 0.0f);
            }
            const int kk = e / kTile, c = e % kTile, i = i0 + kk;
            const int x = x0 + c;
            float2 b = make_float2(0.0f, 0.0f);
            if (i < nh && x < nx) {
                const float ci = (i == 0 || 2 * i == nx) ? 1.0f : 2.0f;
                const float2 w = tb.fx[(int)(((long long)i * x) % nx)];
                b = make_float2(ci * w.x, ci * w.y);
            }
            Bs[kk][c] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kKc; kk++) {
            float2 a[4], b[4];
#pragma unroll
            for (int m = 0; m < 4; m++) a[m] = As[kk][ty + 16 * m];
#pragma unroll
            for (int n = 0; n < 4; n++) b[n] = Bs[kk][tx + 16 * n];
#pragma unroll
            for (int m = 0; m < 4; m++)
#pragma unroll
                for (int n = 0; n < 4; n++) {
                    acc[m][n] = fmaf(a[m].x, b[n].x, acc[m][n]);
                    acc[m][n] = fmaf(-a[m].y, b[n].y, acc[m][n]);
                }
        }
        __syncthreads();
    }
    const float nn = (float)(nx * ny);
    float *dz = d + (size_t)z * nx * ny;
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const int y = y0 + ty + 16 * m, x = x0 + tx + 16 * n;
            if (y >= ny || x >= nx) continue;
            const float S = __fdiv_rn(acc[m][n], nn);
            if (s_out) {  // makePeriodicSlice: the smooth part itself
                s_out[((size_t)z * ny + y) * nx + x] = S;
                continue;
            }
            const double dist =
                1.0 * (double)min(min(x, abs(nx - 1 - x)), min(y, abs(ny - 1 - y)));
            const double Wg = exp(-1.0 * dist * dist / (2 * 5.0 * 5.0));
            float *p = dz + (size_t)y * nx + x;
            *p = (float)__dsub_rn((double)*p, __dmul_rn(Wg, (double)S));
        }
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace

int take_log(float *d_x, size_t n, cudaStream_t st) {
    if (n == 0) return 0;
    const int blocks = (int)std::min<size_t>(4096, (n + 255) / 256);
    k_take_log<<<blocks, 256, 0, st>>>(d_x, n);
    count_launches(1);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

// s_out != NULL: write the smooth parts S there ([nz][ny][nx]) and leave d.
int periodic_decomp(float *d, int nz, int ny, int nx, float *s_out, cudaStream_t st) {
    if (nz < 0 || nx < 2 || ny < 2 || nx > 65536 || ny > 65535) {
        set_error("periodic_decomposition: sizes must be 2 <= nx <= 65536, 2 <= ny <= 65535");
        return ARECGB_ERR_ARG;
    }
    if (nz == 0) return 0;
    const int nh = nx / 2 + 1;
    // twiddle tables e^{+2 pi i k / n}, host libm in double
    std::vector<double2> ex(nx), ey(ny);
    std::vector<float2> fx(nx), fy(ny);
    const double two_pi = 2.0 * (std::atan(1.0) * 4);
    for (int k = 0; k < nx; k++) {
        ex[k] = make_double2(std::cos(two_pi * k / nx), std::sin(two_pi * k / nx));
        fx[k] = make_float2((float)ex[k].x, (float)ex[k].y);
    }
    for (int k = 0; k < ny; k++) {
        ey[k] = make_double2(std::cos(two_pi * k / ny), std::sin(two_pi * k / ny));
        fy[k] = make_float2((float)ey[k].x, (float)ey[k].y);
    }
    const size_t per_slice = sizeof(double2) * (2 * (size_t)nh + ny) +
                             2 * sizeof(float2) * (size_t)ny * nh;
    const int batch = (int)std::max<size_t>(
        1, std::min<size_t>(std::min<size_t>((size_t)nz, 65535), (size_t(1) << 30) / per_slice));
    const size_t tab = sizeof(double2) * (nx + ny) + sizeof(float2) * (nx + ny);
    const size_t off_e = (tab + 255) / 256 * 256;
    const size_t off_w = off_e + ((sizeof(double2) * (2 * (size_t)nh + ny) * batch + 255) / 256) * 256;
    const size_t off_t = off_w + ((sizeof(float2) * (size_t)ny * nh * batch + 255) / 256) * 256;
    const size_t bytes = off_t + sizeof(float2) * (size_t)ny * nh * batch;
    DevBuf buf;
    ARECGB_CUDA(cudaMalloc(&buf.p, bytes));
    char *b0 = (char *)buf.p;
    double2 *d_ex = (double2 *)b0, *d_ey = d_ex + nx;
    float2 *d_fx = (float2 *)(d_ey + ny), *d_fy = d_fx + nx;
    ARECGB_CUDA(cudaMemcpyAsync(d_ex, ex.data(), sizeof(double2) * nx, cudaMemcpyHostToDevice, st));
    ARECGB_CUDA(cudaMemcpyAsync(d_ey, ey.data(), sizeof(double2) * ny, cudaMemcpyHostToDevice, st));
    ARECGB_CUDA(cudaMemcpyAsync(d_fx, fx.data(), sizeof(float2) * nx, cudaMemcpyHostToDevice, st));
    ARECGB_CUDA(cudaMemcpyAsync(d_fy, fy.data(), sizeof(float2) * ny, cudaMemcpyHostToDevice, st));
    PdTables tb{d_ex, d_ey, d_fx, d_fy};
    double2 *edges = (double2 *)(b0 + off_e);
    float2 *W = (float2 *)(b0 + off_w), *T = (float2 *)(b0 + off_t);
    for (int z0 = 0; z0 < nz; z0 += batch) {
        const int nb = std::min(batch, nz - z0);
        float *dz = d + (size_t)z0 * nx * ny;
        k_pd_edges<<<nb, 256, 0, st>>>(dz, nx, ny, nh, tb, edges);
        k_pd_w<<<dim3((nh + 127) / 128, ny, nb), 128, 0, st>>>(edges, nx, ny, nh, tb, W);
        k_pd_cols<<<dim3((nh + kTile - 1) / kTile, (ny + kTile - 1) / kTile, nb), kPdThreads, 0,
                    st>>>(W, ny, nh, tb, T);
        k_pd_rows<<<dim3((nx + kTile - 1) / kTile, (ny + kTile - 1) / kTile, nb), kPdThreads, 0,
                    st>>>(T, nx, ny, nh, tb, dz, s_out ? s_out + (size_t)z0 * nx * ny : nullptr);
        count_launches(4);
        ARECGB_CUDA(cudaGetLastError());
    }
    // the scratch is freed after the work that reads it
    ARECGB_CUDA(cudaStreamSynchronize(st));
    return 0;
}

}  // namespace arecgb
