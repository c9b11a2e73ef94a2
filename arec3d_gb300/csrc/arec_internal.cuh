// Internal definitions shared by the CUDA translation units of libarec_gb300.
//
// Data layout in HBM (slice index fastest everywhere, `ys` = slice count padded
// to a multiple of 8 so every row starts on 32 bytes and a lane's vector of
// 1/2/4/8 slices never straddles the padded end):
//   volume     x[ray][ys]        rays of the cylinder in the reference's order
//                                (iz-major, ix-minor; AREC3D/AREC3D/arecImage.cpp:72-84)
//   sinogram   q[angle][bin][ys] detector bin before slice (the reference keeps
//                                [angle][slice][bin]; the boundary transposes)
// Padding slices are zero on input and stay zero through every operator.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "arec_gb300.h"

namespace arecgb {

// ---------------------------------------------------------------------------
// Per-angle constants, computed on the host in double like the reference and
// rounded once to float.
struct AngleParams {
    float c, s;          // cosf/sinf of the float angle: exact floats (see arec_geometry.cu)
    float sq_a, sq_b;    // square-pixel footprint breakpoints (arecproject.h:11-22)
    float sq_aeps;       // a + 1e-3: the linear piece's test bound (arecproject.h:34)
    float sq_ymax;       // plateau height 1/(b+a)
    float sq_c2;         // 0.5*ymax*(b+a): intercept of the linear piece
    float sq_k1;         // 0.5*ymax/(b-a): curvature of the quadratic pieces
    int orient;          // 0: sweep rows (|c| >= |s|), 1: sweep columns
    float pad[3];
};

struct RowInfo {
    int start;  // ray index of the first pixel of row iz
    int lo, hi; // first/last ix of the row inside the cylinder
    int pad;
};

struct ColInfo {
    int lo, hi; // first/last iz of column ix inside the cylinder
    int start;  // index of pixel (lo, ix) in column-major ray order
    int pad;
};

struct Plan {
    int weighting = 0;   // ARECGB_LIN / ARECGB_KB / ARECGB_SQ
    double radius = 0;
    int nx = 0, nrays = 0, ny = 0, ys = 0, na = 0;
    float r_hi = 0, r_lo = 0;   // centre (radius, or (int)radius+1 for LIN) as a float pair
    std::vector<float> angles;
    int device = 0;

    // device tables
    float4 *d_ray = nullptr;      // per ray: (xc_hi, zc_hi, xc_lo, zc_lo) offsets from the centre
    AngleParams *d_ang = nullptr;
    RowInfo *d_rows = nullptr;    // nx rows
    ColInfo *d_cols = nullptr;    // nx columns
    int4 *d_groups = nullptr;     // forward-projection angle groups: (first, count, orient, 0),
    int ngroups = 0;              //   the row-sweeping (orient 0) groups first
    int ngroups_o[2] = {0, 0};    // groups per orientation
    int fp_band = 64;             // forward projection: lines per band launch
    int bp_nsc = 0;               // back projection: slice chunks per block (0 = by size)
    int bp_vec = 0;               // back projection: floats per lane (0 = vec)
    int fp_vec = 0;               // forward projection (SQ, KB): floats per lane (0 = vec)

    // Optional tables (SQ, KB; built at creation when device memory allows,
    // see plan_build_tables): the taps of every (ray, angle) for the forward
    // projector and the back projector's per-(tile, angle) ring plans.  The
    // kernels compute the same values without them.
    float4 *d_taps = nullptr;     // [ngroups][nrays][4], rays in each group's line order
    int *d_kinv = nullptr;        // column-major ray index -> ray index
    int *d_lin_off = nullptr;     // linear weighting: per angle, rays by first bin (offsets)
    int *d_lin_list = nullptr;    //   and the rays themselves (see k_lin_index)
    float *d_xT = nullptr;        // [nrays][ys]: x in column-major ray order (column sweeps)
    float4 *d_bpw = nullptr;      // [ntiles][na][32]
    int2 *d_bpf = nullptr;        // [ntiles][na]
    size_t table_bytes = 0;
    int tuned = 0;                // launch shapes chosen by plan_autotune
    int2 *d_tiles = nullptr;      // back-projection ray tiles: (ix0, iz0) of 8x4-pixel tiles
    int ntiles = 0;
    int *d_err = nullptr;         // device error flag (nonzero: a kernel saw an impossible case)

    // launch shapes (set at creation; see arec_project.cu)
    int vec = 4;                  // floats per lane along slices
    int fp_bins = 16;             // detector bins per forward-projection block
    int bp_rays = 32;             // rays per back-projection block

    // FP64 reduction partial sums (one per block of FP / BP)
    double *d_partials = nullptr;
    int n_partials = 0;

    // scratch owned by the plan for the reference-compatible entry points
    float *d_vol[4] = {nullptr, nullptr, nullptr, nullptr};
    float *d_sin[3] = {nullptr, nullptr, nullptr};
    float *d_w = nullptr;          // statistical weights of the weighted CGLS (device layout)
    float *d_stage = nullptr;      // staging buffer in the reference layout
    size_t stage_floats = 0;
    float *h_pinned = nullptr;     // pinned host staging
    size_t pinned_floats = 0;
    float *d_img[2] = {nullptr, nullptr};  // warm-start network images (arecgb_reconstruct_host)
    float *d_ramp = nullptr;      // ramp filter taps (odd distances), built on first use
    int ramp_n = 0;
    size_t img_floats = 0;

    cudaStream_t stream = nullptr; // plan-owned stream for the compatible entry points

    // solver scratch, allocated on first use and kept (no allocation or
    // free, and so no device synchronisation, per solve): SIRT's reduction
    // partials and its two pinned results; the CGLS driver's per-problem
    // state (device and pinned copy), residual history, stream, events and
    // branch streams (a batch keeps them in its first plan)
    double *d_sred = nullptr, *h_sred = nullptr;
    void *d_cstate = nullptr, *h_cstate = nullptr;
    size_t cstate_bytes = 0;
    double *d_chist = nullptr;
    size_t chist_bytes = 0;
    cudaStream_t solve_stream = nullptr;
    std::vector<cudaEvent_t> solve_ev;
    std::vector<cudaStream_t> solve_bs;

    // optional projector timing: CUDA events around every forward / back
    // projection (arecgb_plan_timing); pairs are reused across calls
    mutable bool timing = false;
    mutable std::vector<cudaEvent_t> ev_fp, ev_bp;  // start, stop, start, stop, ...
    mutable size_t n_fp = 0, n_bp = 0;
};

// Kernel launches issued by this library (all threads), for reporting.
void count_launches(int n);
long long launch_count();

constexpr int kTileX = 8, kTileZ = 4;  // back-projection ray tile (32 rays)
constexpr int kGroupAngles = 4;        // angles per forward-projection block
constexpr int kFpBins = 8;             // detector bins per forward-projection block

// Geometry / plans (arec_geometry.cu)
// tables = false: never build the optional projector tables (the kernels then
// compute the same values as they go; for callers that budget device memory).
int plan_create(Plan **out, int weighting, double radius, int ny, int nangles,
                const float *angles_host, bool tables = true);
void plan_destroy(Plan *p);
size_t vol_floats(const Plan *p);
size_t sin_floats(const Plan *p);

// Operators (arec_project.cu)
int forward_project(const Plan *p, const float *d_x, float *d_q, double *d_norm2,
                    const int *d_skip, cudaStream_t st);
int back_project(const Plan *p, const float *d_s, float *d_g, double *d_norm2,
                 const int *d_skip, cudaStream_t st);
int fp_grid_blocks(const Plan *p);
int plan_timing(const Plan *p, int mode, double *fp_ms, long long *fp_calls, double *bp_ms,
                long long *bp_calls);
int plan_autotune(Plan *p, float *d_x, float *d_q, cudaStream_t st);
int plan_build_tables(Plan *p);
int bp_grid_blocks(const Plan *p);

// Filtered back projection (arec_fbp.cu): the Ram-Lak ramp filter along bins
// (weight pi / nangles folded in), and x = A^T (ramp * b) [with ||A^T b||^2].
int ramp_filter(Plan *p, const float *d_s, float *d_f, cudaStream_t st);
int fbp(Plan *p, const float *d_b, float *d_x, float *d_work, double *d_norm2, cudaStream_t st);

// The solvers' reduction scratch (arec_solver.cu): d_sred holds 2 kSredBlocks
// partials and two results, h_sred two pinned doubles.
constexpr int kSredBlocks = 1024;
int ensure_red(Plan *p);

// Layout kernels and vector ops (arec_vector.cu)
int sino_to_device_layout(const float *d_ref, float *d_dev, int na, int ny, int nx, int ys,
                          cudaStream_t st);
int sino_to_reference_layout(const float *d_dev, float *d_ref, int na, int ny, int nx, int ys,
                             cudaStream_t st);
int reduce_partials(const double *d_partials, int n, double *d_out, cudaStream_t st);

// error helpers
int cuda_status(cudaError_t e);
void set_error(const std::string &msg);

#define ARECGB_CUDA(call)                                        \
    do {                                                         \
        cudaError_t e__ = (call);                                \
        if (e__ != cudaSuccess) {                                \
            ::arecgb::set_error(std::string(#call) + ": " +      \
                                cudaGetErrorString(e__));        \
            return ::arecgb::cuda_status(e__);                   \
        }                                                        \
    } while (0)

}  // namespace arecgb
