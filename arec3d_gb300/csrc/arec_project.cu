// Projector dispatch: launch shapes, weighting selection and the FP64 norm.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "arec_project_impl.cuh"

namespace arecgb {

int launch_bp_lin(const OpArgs &, int, int, dim3, const float *, float *, const CUtensorMap &,
                 int, cudaStream_t);
int launch_bp_kb(const OpArgs &, int, int, dim3, const float *, float *, const CUtensorMap &,
                 int, cudaStream_t);
int launch_bp_sq(const OpArgs &, int, int, dim3, const float *, float *, const CUtensorMap &,
                 int, cudaStream_t);
int launch_fp_lin(const OpArgs &, int, const float *, float *, cudaStream_t);
int launch_lin_index(const OpArgs &, int *, int *, cudaStream_t);
int launch_tables_sq(const OpArgs &, int, float4 *, float4 *, int2 *, cudaStream_t);
int launch_tables_kb(const OpArgs &, int, float4 *, float4 *, int2 *, cudaStream_t);
int launch_fpb_kb(const OpArgs &, int, dim3, const float *, float *, int, int, int, int,
                  const CUtensorMap &, const CUtensorMap &, cudaStream_t);
int launch_fpb_sq(const OpArgs &, int, dim3, const float *, float *, int, int, int, int,
                  const CUtensorMap &, const CUtensorMap &, cudaStream_t);
int sumsq_partials(const float *d_v, size_t n, double *d_partials, int nblocks, cudaStream_t st);

static OpArgs make_args(const Plan *p, const int *skip) {
    OpArgs A;
    A.ray = p->d_ray;
    A.ang = p->d_ang;
    A.rows = p->d_rows;
    A.cols = p->d_cols;
    A.groups = p->d_groups;
    A.tiles = p->d_tiles;
    A.nx = p->nx;
    A.nrays = p->nrays;
    A.ys = p->ys;
    A.na = p->na;
    A.ngroups = p->ngroups;
    A.r_hi = p->r_hi;
    A.r_lo = p->r_lo;
    A.partials = p->d_partials;
    A.skip = skip;
    A.err = p->d_err;
    A.taps = p->d_taps;
    A.bpw = p->d_bpw;
    A.bpf = p->d_bpf;
    A.kinv = p->d_kinv;
    A.lin_off = p->d_lin_off;
    A.lin_list = p->d_lin_list;
    return A;
}

// Back projection: floats per lane (the plan's, or the autotuner's choice).
static int bp_vec(const Plan *p) { return p->bp_vec ? p->bp_vec : p->vec; }

// Slice chunks per block: two warps' worth of slices when there are that many.
static int slice_chunks(const Plan *p) {
    const int v = bp_vec(p);
    if (p->bp_nsc == 1 || (p->bp_nsc == 2 && p->ys > 32 * v)) return p->bp_nsc;
    return p->ys > 32 * v ? 2 : 1;
}

static int slice_blocks(const Plan *p) {
    const int span = 32 * bp_vec(p) * slice_chunks(p);
    return (p->ys + span - 1) / span;
}

constexpr int kNormBlocks = 1024;

// Forward projection (banded kernels): floats per lane.
static int fp_vec(const Plan *p) { return p->fp_vec ? p->fp_vec : p->vec; }

static int fp_slice_blocks(const Plan *p) {
    const int v = fp_vec(p);
    return (p->ys + 32 * v - 1) / (32 * v);
}

// The forward projector's FP64 norm is a separate pass over q (1024 partials).
int fp_grid_blocks(const Plan *) { return kNormBlocks; }

int bp_grid_blocks(const Plan *p) { return p->ntiles * slice_blocks(p); }

// Event pair i of a timing list (created on first use).
static int timing_event(std::vector<cudaEvent_t> &v, size_t i, cudaEvent_t *out) {
    while (v.size() <= i) {
        cudaEvent_t e;
        ARECGB_CUDA(cudaEventCreate(&e));
        v.push_back(e);
    }
    *out = v[i];
    return 0;
}

static int timing_mark(const Plan *p, bool fp, bool stop, cudaStream_t st) {
    if (!p->timing) return 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone)
        return 0;  // a captured iteration is timed by its eager calls only
    std::vector<cudaEvent_t> &v = fp ? p->ev_fp : p->ev_bp;
    size_t &n = fp ? p->n_fp : p->n_bp;
    cudaEvent_t e;
    int rc = timing_event(v, 2 * n + (stop ? 1 : 0), &e);
    if (rc) return rc;
    ARECGB_CUDA(cudaEventRecord(e, st));
    if (stop) n++;
    return 0;
}

int plan_timing(const Plan *p, int mode, double *fp_ms, long long *fp_calls, double *bp_ms,
                long long *bp_calls) {
    if (mode == 1) {
        p->timing = true;
        p->n_fp = p->n_bp = 0;
        return 0;
    }
    double t[2] = {0.0, 0.0};
    for (int k = 0; k < 2; k++) {
        const std::vector<cudaEvent_t> &v = k ? p->ev_bp : p->ev_fp;
        const size_t n = k ? p->n_bp : p->n_fp;
        if (n) ARECGB_CUDA(cudaEventSynchronize(v[2 * n - 1]));
        for (size_t i = 0; i < n; i++) {
            float ms = 0.f;
            ARECGB_CUDA(cudaEventElapsedTime(&ms, v[2 * i], v[2 * i + 1]));
            t[k] += ms;
        }
    }
    if (fp_ms) *fp_ms = t[0];
    if (bp_ms) *bp_ms = t[1];
    if (fp_calls) *fp_calls = (long long)p->n_fp;
    if (bp_calls) *bp_calls = (long long)p->n_bp;
    if (mode == 0) p->timing = false;
    return 0;
}

// q = 0 unless the solve has finished (then the call leaves q alone).
__global__ void __launch_bounds__(256) k_zero_unless(float4 *q, size_t n4, const int *skip) {
    if (skip && *skip) return;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n4; i += (size_t)gridDim.x * 256)
        q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

int forward_project(const Plan *p, const float *d_x, float *d_q, double *d_norm2,
                    const int *d_skip, cudaStream_t st) {
    const OpArgs A = make_args(p, d_skip);
    const size_t nq = sin_floats(p);
    int rc = timing_mark(p, true, false, st);
    if (rc) return rc;
    if (p->weighting == ARECGB_LIN) {
        ARECGB_CUDA(cudaMemsetAsync(d_q, 0, sizeof(float) * nq, st));
        rc = launch_fp_lin(A, p->vec, d_x, d_q, st);
        count_launches(1);
    } else {
        // zero q, then each (orientation, line band) launch adds its part
        k_zero_unless<<<(unsigned)std::min<size_t>(152 * 8, (nq / 4 + 255) / 256), 256, 0, st>>>(
            reinterpret_cast<float4 *>(d_q), nq / 4, d_skip);
        const int ntile = (p->nx + kFpBins - 1) / kFpBins;
        rc = 0;
        // With the tables: tensor maps over x and over its column-major copy
        // (gathered here when there are column sweeps), box = 8 rays x SPAN
        // slices; the kernels stage a line's n pixels as ceil(n / 8) boxes.
        CUtensorMap tmx, tmxT;
        memset(&tmx, 0, sizeof(tmx));
        memset(&tmxT, 0, sizeof(tmxT));
        if (A.taps) {
            const int span = 32 * fp_vec(p);
            if (p->ngroups_o[1]) {
                const int ys4 = p->ys / 4;
                const size_t n4 = (size_t)p->nrays * ys4;
                k_ray_gather<<<(unsigned)std::min<size_t>(152 * 16, (n4 + 255) / 256), 256, 0, st>>>(
                    reinterpret_cast<const float4 *>(d_x), reinterpret_cast<float4 *>(p->d_xT),
                    p->d_kinv, p->nrays, ys4);
                count_launches(1);
            }
            if (!encode_rows_map(&tmx, d_x, p->ys, p->nrays, span, kFpBox) ||
                !encode_rows_map(&tmxT, p->d_xT, p->ys, p->nrays, span, kFpBox)) {
                set_error("forward_project: tensor map encoding failed");
                return ARECGB_ERR_ARG;
            }
        }
        for (int o = 0; o < 2 && !rc; o++) {
            const int ngo = p->ngroups_o[o];
            if (!ngo) continue;
            const int g0 = o ? p->ngroups_o[0] : 0;
            const dim3 grid(ngo * ntile, fp_slice_blocks(p));
            for (int lo = 0; lo < p->nx && !rc; lo += p->fp_band) {
                const int hi = std::min(p->nx, lo + p->fp_band);
                rc = p->weighting == ARECGB_KB
                         ? launch_fpb_kb(A, fp_vec(p), grid, d_x, d_q, g0, ngo, lo, hi, tmx, tmxT, st)
                         : launch_fpb_sq(A, fp_vec(p), grid, d_x, d_q, g0, ngo, lo, hi, tmx, tmxT, st);
                count_launches(1);
            }
        }
        count_launches(1);
    }
    ARECGB_CUDA(cudaGetLastError());
    if (rc) return ARECGB_ERR_ARG;
    if (d_norm2) {
        rc = sumsq_partials(d_q, nq, p->d_partials, kNormBlocks, st);
        if (rc) return rc;
        rc = reduce_partials(p->d_partials, kNormBlocks, d_norm2, st);
        if (rc) return rc;
        count_launches(2);
    }
    return timing_mark(p, true, true, st);
}

int back_project(const Plan *p, const float *d_s, float *d_g, double *d_norm2,
                 const int *d_skip, cudaStream_t st) {
    const OpArgs A = make_args(p, d_skip);
    const int nsc = slice_chunks(p);
    dim3 grid(p->ntiles, slice_blocks(p));
    // the footprint of an angle as one TMA tile (kBpFoot bins x the block's slices,
    // at most 256: one slice chunk per block up to VEC 8)
    CUtensorMap tms;
    memset(&tms, 0, sizeof(tms));
    const int span = 32 * bp_vec(p) * nsc;
    int use_tma = p->weighting != ARECGB_LIN && span <= 256 &&
                  encode_sino_map(&tms, d_s, p->ys, p->nx, p->na, span, kBpFoot);
    {
        const char *env = getenv("ARECGB_BP_TMA");
        if (env && env[0] == '0') use_tma = 0;
    }
    int rc = timing_mark(p, false, false, st);
    if (rc) return rc;
    count_launches(d_norm2 ? 2 : 1);
    if (p->weighting == ARECGB_LIN)
        rc = launch_bp_lin(A, bp_vec(p), nsc, grid, d_s, d_g, tms, use_tma, st);
    else if (p->weighting == ARECGB_KB)
        rc = launch_bp_kb(A, bp_vec(p), nsc, grid, d_s, d_g, tms, use_tma, st);
    else
        rc = launch_bp_sq(A, bp_vec(p), nsc, grid, d_s, d_g, tms, use_tma, st);
    ARECGB_CUDA(cudaGetLastError());
    if (rc) return ARECGB_ERR_ARG;
    if (d_norm2) {
        rc = reduce_partials(p->d_partials, grid.x * grid.y, d_norm2, st);
        if (rc) return rc;
    }
    return timing_mark(p, false, true, st);
}

// Tables for the SQ and KB projectors: the taps of every (angle group, ray)
// (ngroups x nrays x 4 x 16 B: 15.8 GB at 1024^2 x 1200 angles) and the back
// projector's ring plans (ntiles x na x 520 B: 16.3 GB).  Built when they take
// at most 40 % of the free device memory and ARECGB_PLAN_TABLES is not "0";
// otherwise the kernels compute the same values as they go.  The tables hold
// exactly what the kernels would compute (the same device functions), so
// results do not depend on them.
// The linear weighting's ray index (per angle, the rays grouped by first bin:
// na x (nrays + nx + 2) ints), which makes its forward projection a gather
// with a fixed summation order.  Built when it takes at most 40 % of the free
// memory (else the forward projection scatters with atomics).
static int plan_build_lin_index(Plan *p) {
    const size_t b_off = sizeof(int) * (size_t)p->na * (p->nx + 2);
    const size_t b_list = sizeof(int) * (size_t)p->na * p->nrays;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
    if ((double)(b_off + b_list) > 0.4 * (double)free_b) return 0;
    if (cudaMalloc(&p->d_lin_off, b_off) != cudaSuccess ||
        cudaMalloc(&p->d_lin_list, b_list) != cudaSuccess) {
        cudaGetLastError();  // not sticky: run with the scatter
        cudaFree(p->d_lin_off);
        cudaFree(p->d_lin_list);
        p->d_lin_off = nullptr;
        p->d_lin_list = nullptr;
        return 0;
    }
    const OpArgs A = make_args(p, nullptr);
    launch_lin_index(A, p->d_lin_off, p->d_lin_list, p->stream);
    count_launches(1);
    ARECGB_CUDA(cudaGetLastError());
    ARECGB_CUDA(cudaStreamSynchronize(p->stream));
    p->table_bytes = b_off + b_list;
    return 0;
}

int plan_build_tables(Plan *p) {
    if (p->weighting == ARECGB_LIN) return plan_build_lin_index(p);
    const char *env = getenv("ARECGB_PLAN_TABLES");
    if (env && env[0] == '0') return 0;
    const size_t b_taps = sizeof(float4) * (size_t)p->ngroups * p->nrays * 4 +
                          sizeof(float) * (size_t)p->nrays * p->ys;  // + x's column-major copy
    const size_t b_bpw = sizeof(float4) * (size_t)p->ntiles * p->na * 32;
    const size_t b_bpf = sizeof(int2) * (size_t)p->ntiles * p->na;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
    if ((double)(b_taps + b_bpw + b_bpf) > 0.4 * (double)free_b) return 0;
    if (cudaMalloc(&p->d_taps, sizeof(float4) * (size_t)p->ngroups * p->nrays * 4) != cudaSuccess ||
        cudaMalloc(&p->d_xT, sizeof(float) * (size_t)p->nrays * p->ys) != cudaSuccess ||
        cudaMalloc(&p->d_bpw, b_bpw) != cudaSuccess || cudaMalloc(&p->d_bpf, b_bpf) != cudaSuccess) {
        cudaGetLastError();  // an allocation failure is not sticky; run without tables
        cudaFree(p->d_taps);
        cudaFree(p->d_xT);
        cudaFree(p->d_bpw);
        cudaFree(p->d_bpf);
        p->d_taps = nullptr;
        p->d_xT = nullptr;
        p->d_bpw = nullptr;
        p->d_bpf = nullptr;
        return 0;
    }
    OpArgs A = make_args(p, nullptr);
    const int rc = p->weighting == ARECGB_KB
                       ? launch_tables_kb(A, p->ntiles, p->d_taps, p->d_bpw, p->d_bpf, p->stream)
                       : launch_tables_sq(A, p->ntiles, p->d_taps, p->d_bpw, p->d_bpf, p->stream);
    count_launches(2);
    ARECGB_CUDA(cudaGetLastError());
    ARECGB_CUDA(cudaStreamSynchronize(p->stream));
    int err = 0;
    ARECGB_CUDA(cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (rc || err) {
        set_error("plan_build_tables: a tile's footprint exceeds the staged width");
        return ARECGB_ERR_ARG;
    }
    p->table_bytes = b_taps + b_bpw + b_bpf;
    return 0;
}

// Autotuner: times the forward projector for band heights of 32, 64 and 128
// lines and the back projector with one or two slice chunks per block on the
// caller's buffers (x: a volume, q: a sinogram of this plan; both overwritten),
// best of two runs each after a warm-up run, and keeps the fastest shapes.
int plan_autotune(Plan *p, float *d_x, float *d_q, cudaStream_t st) {
    if (p->weighting == ARECGB_LIN) return 0;  // the linear pair has no shapes to choose
    cudaEvent_t e0, e1;
    ARECGB_CUDA(cudaEventCreate(&e0));
    ARECGB_CUDA(cudaEventCreate(&e1));
    auto best_of = [&](auto &&fn, float *ms) -> int {
        int rc = fn();  // warm-up
        if (rc) return rc;
        *ms = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            ARECGB_CUDA(cudaEventRecord(e0, st));
            if ((rc = fn())) return rc;
            ARECGB_CUDA(cudaEventRecord(e1, st));
            ARECGB_CUDA(cudaEventSynchronize(e1));
            float t = 0.f;
            ARECGB_CUDA(cudaEventElapsedTime(&t, e0, e1));
            *ms = std::min(*ms, t);
        }
        return 0;
    };
    int rc = 0;
    const bool was_timing = p->timing;
    p->timing = false;
    // forward projection: band height x floats per lane (the plan's or half)
    int best_band = p->fp_band, best_fvec = 0;
    float best = 1e30f;
    for (int fv : {p->vec, p->vec / 2}) {
        if (fv < 1 || rc) continue;
        p->fp_vec = fv;
        for (int band : {32, 64, 128}) {
            if (band > 2 * p->nx && band != 32) continue;
            p->fp_band = band;
            float ms;
            if ((rc = best_of([&] { return forward_project(p, d_x, d_q, nullptr, nullptr, st); },
                              &ms)))
                break;
            if (ms < best) {
                best = ms;
                best_band = band;
                best_fvec = fv;
            }
        }
    }
    p->fp_band = best_band;
    p->fp_vec = best_fvec;
    // back projection: (floats per lane, slice chunks per block) in
    // {(vec, 1), (vec, 2), (vec / 2, 1)}: half the vector width halves the
    // accumulators and the staged rows (more blocks per SM)
    int best_nsc = 0, best_vec = 0;
    best = 1e30f;
    const int shapes[3][2] = {{p->vec, 1}, {p->vec, 2}, {p->vec / 2, 1}};
    for (const auto &sh : shapes) {
        if (rc) break;
        const int v = sh[0], nsc = sh[1];
        if (v < 1 || (nsc == 2 && p->ys <= 32 * v)) continue;
        p->bp_vec = v;
        p->bp_nsc = nsc;
        float ms;
        if ((rc = best_of([&] { return back_project(p, d_q, d_x, nullptr, nullptr, st); }, &ms)))
            break;
        if (ms < best) {
            best = ms;
            best_nsc = nsc;
            best_vec = v;
        }
    }
    p->bp_nsc = best_nsc;
    p->bp_vec = best_vec;
    p->tuned = rc ? 0 : 1;
    p->timing = was_timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

}  // namespace arecgb
