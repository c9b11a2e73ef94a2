// Per (ray, angle) projector weights, shared by the forward and the back
// projector so that A and A^T use bit-identical coefficients.
//
// Every float operation here is an explicit round-to-nearest intrinsic
// (__fadd_rn/__fmul_rn/__fmaf_rn/__fdiv_rn): the compiler may not contract or
// reorder them, so both kernels evaluate exactly the same arithmetic.
//
// Position of ray k at angle a (reference, AREC3D/AREC3D/arecproject.cpp:605-607):
//   xb = xc*cos + zc*sin + xcent   in double, with cos/sin = cosf/sinf of the
// float angle (exact floats) and xc, zc the ray's offsets from the centre.
// Here xb is carried as an unevaluated float pair (hi + lo) built from exact
// products (FMA) and error-free sums, i.e. to ~2^-48 relative, so the centre bin
// rint(xb) and the fractional offset agree with the double computation except
// within ~1e-12 px of a rounding boundary.
#pragma once

#include "arec_internal.cuh"

namespace arecgb {

static __device__ float c_kb_lut[512] = {
#include "kb_lut_table.inc"
};

// Tap triple: coefficients of bins iqx-1, iqx, iqx+1.
struct Taps {
    int iqx;
    float w0, w1, w2;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// xb as (u, lo): u = float sum, lo = accumulated rounding errors.
__device__ __forceinline__ void ray_position(const float4 ray, const AngleParams &ap, float r_hi,
                                             float r_lo, float &u, float &lo) {
    float p1 = __fmul_rn(ray.x, ap.c);
    float e1 = __fmaf_rn(ray.x, ap.c, -p1);
    float p2 = __fmul_rn(ray.y, ap.s);
    float e2 = __fmaf_rn(ray.y, ap.s, -p2);
    float t, et, eu;
    two_sum(p1, p2, t, et);
    two_sum(t, r_hi, u, eu);
    float l = __fadd_rn(e1, e2);
    l = __fadd_rn(l, et);
    l = __fadd_rn(l, eu);
    l = __fadd_rn(l, r_lo);
    l = __fmaf_rn(ray.z, ap.c, l);
    l = __fmaf_rn(ray.w, ap.s, l);
    lo = l;
}

// rint(u + lo) with ties to even, and d with (u + lo) - rint(u + lo) = d + lo.
// n = rintf(u) leaves d = u - n exact with |d| <= 0.5; since |lo| is below half
// an ulp of u, only d = +-0.5 (u on a half-integer, where rintf chose the even
// neighbour) can round the other way, and then the sign of lo decides.
__device__ __forceinline__ int round_centre(float u, float lo, float &d) {
    float n = rintf(u);
    d = __fsub_rn(u, n);
    if (d == 0.5f && lo > 0.0f) {
        n = __fadd_rn(n, 1.0f);
        d = -0.5f;
    } else if (d == -0.5f && lo < 0.0f) {
        n = __fsub_rn(n, 1.0f);
        d = 0.5f;
    }
    return (int)n;
}

// Square-pixel footprint CDF (reference AREC3D/AREC3D/arecproject.h:24-47):
// 0 below -b, 1 above b, the linear piece within a+1e-3 first, then the two
// quadratics (written as k1*(x+b)^2 and 1 - k1*(b-x)^2).
__device__ __forceinline__ float sq_cdf(float x, const AngleParams &ap) {
    float lin = __fmaf_rn(ap.sq_ymax, x, ap.sq_c2);
    float tl = __fadd_rn(x, ap.sq_b);
    float ql = __fmul_rn(__fmul_rn(ap.sq_k1, tl), tl);
    float tr = __fsub_rn(ap.sq_b, x);
    float qr = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(ap.sq_k1, tr), tr));
    float v = 0.0f;
    if (x > ap.sq_a) v = qr;
    if (x < -ap.sq_a) v = ql;
    if (x > -ap.sq_aeps && x < ap.sq_aeps) v = lin;
    if (x > ap.sq_b) v = 1.0f;
    if (x < -ap.sq_b) v = 0.0f;
    return v;
}

// interp1_R_MOD (reference arecproject.cpp:340-346) on a float argument:
//   x = |x| / DR;  i = (int)x;  x -= i;
//   float( double(L[i]) * (1.0 - x) + double(float(L[i+1] * x)) )
// The double sum is formed exactly from float pairs and rounded once.
__device__ __forceinline__ float kb_interp(float x) {
    const float dr = 0x1.899c10p-9f;  // (float)(3.0 / 999)
    x = fabsf(x);
    x = __fdiv_rn(x, dr);
    int ind = (int)x;
    ind = ind > 510 ? 510 : ind;
    x = __fsub_rn(x, (float)ind);
    float l0 = c_kb_lut[ind], l1 = c_kb_lut[ind + 1];
    float right = __fmul_rn(l1, x);
    float om, om_e;
    two_sum(1.0f, -x, om, om_e);     // 1 - x exactly as om + om_e
    float p = __fmul_rn(l0, om);
    float pe = __fmaf_rn(l0, om, -p); // l0*om exactly as p + pe
    pe = __fmaf_rn(l0, om_e, pe);
    float s, se;
    two_sum(p, right, s, se);
    return __fadd_rn(s, __fadd_rn(se, pe));
}

// float(d - k + lo) for small integer k, via an error-free d - k.
__device__ __forceinline__ float frac_arg(float d, float k, float lo) {
    float s, e;
    two_sum(d, -k, s, e);
    return __fadd_rn(s, __fadd_rn(e, lo));
}

template <int W>
__device__ __forceinline__ Taps ray_taps(const float4 ray, const AngleParams &ap, float r_hi,
                                         float r_lo) {
    float u, lo;
    ray_position(ray, ap, r_hi, r_lo, u, lo);
    Taps t;
    if (W == ARECGB_SQ) {
        // iqx = rint(xb); xv = iqx - xb; w_j = F(xv + j - 0.5) - F(xv + j - 1.5)
        // with F(xv - 1.5) = 0 and F(xv + 1.5) = 1 since |xv| <= 0.5 < 1.5 - b
        // (reference arecproject.cpp:610-620).
        float d;
        t.iqx = round_centre(u, lo, d);
        float xv = -__fadd_rn(d, lo);
        float f1 = sq_cdf(__fsub_rn(xv, 0.5f), ap);
        float f2 = sq_cdf(__fadd_rn(xv, 0.5f), ap);
        t.w0 = f1;
        t.w1 = __fsub_rn(f2, f1);
        t.w2 = __fsub_rn(1.0f, f2);
    } else if (W == ARECGB_KB) {
        // iqx = rint(xb); w_j = interp(float(xb - (iqx + j - 1)))
        // (reference arecproject.cpp:370-382).
        float d;
        t.iqx = round_centre(u, lo, d);
        t.w0 = kb_interp(frac_arg(d, -1.0f, lo));
        t.w1 = kb_interp(__fadd_rn(d, lo));
        t.w2 = kb_interp(frac_arg(d, 1.0f, lo));
    } else {
        // LIN: xb stored as float, b = floor(xb); 1-d to bin b-1 and d to bin b
        // (reference arecproject.cpp:78-87); written as centre b with w2 = 0.
        float xbf = __fadd_rn(u, lo);
        float fl = floorf(xbf);
        float d = __fsub_rn(xbf, fl);
        t.iqx = (int)fl;
        t.w0 = __fsub_rn(1.0f, d);
        t.w1 = d;
        t.w2 = 0.0f;
    }
    return t;
}

}  // namespace arecgb
