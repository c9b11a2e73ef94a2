// Projector dispatch: launch shapes, weighting selection and the FP64 norm.
#include "arec_project_impl.cuh"

namespace arecgb {

int launch_bp_lin(const OpArgs &, int, int, dim3, const float *, float *, cudaStream_t);
int launch_bp_kb(const OpArgs &, int, int, dim3, const float *, float *, cudaStream_t);
int launch_bp_sq(const OpArgs &, int, int, dim3, const float *, float *, cudaStream_t);
int launch_fp_lin(const OpArgs &, int, int, dim3, const float *, float *, cudaStream_t);
int launch_fp_kb(const OpArgs &, int, int, dim3, const float *, float *, cudaStream_t);
int launch_fp_sq(const OpArgs &, int, int, dim3, const float *, float *, cudaStream_t);
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
    return A;
}

// Slice chunks per block: two warps' worth of slices when there are that many.
static int slice_chunks(const Plan *p) { return p->ys > 32 * p->vec ? 2 : 1; }

static int slice_blocks(const Plan *p) {
    const int span = 32 * p->vec * slice_chunks(p);
    return (p->ys + span - 1) / span;
}

static int fp_slice_blocks(const Plan *p) { return (p->ys + 32 * p->vec - 1) / (32 * p->vec); }

int fp_grid_blocks(const Plan *p) {
    if (p->weighting == ARECGB_LIN) return 1024;  // sum-of-squares pass over q
    const int ntile = (p->nx + kFpBins - 1) / kFpBins;
    return p->ngroups * ntile * fp_slice_blocks(p);
}

int bp_grid_blocks(const Plan *p) { return p->ntiles * slice_blocks(p); }

int forward_project(const Plan *p, const float *d_x, float *d_q, double *d_norm2,
                    const int *d_skip, cudaStream_t st) {
    const OpArgs A = make_args(p, d_skip);
    const int nsc = slice_chunks(p);
    int rc;
    if (p->weighting == ARECGB_LIN) {
        ARECGB_CUDA(cudaMemsetAsync(d_q, 0, sizeof(float) * sin_floats(p), st));
        rc = launch_fp_lin(A, p->vec, nsc, dim3(1), d_x, d_q, st);
        ARECGB_CUDA(cudaGetLastError());
        if (rc) return ARECGB_ERR_ARG;
        if (d_norm2) {
            rc = sumsq_partials(d_q, sin_floats(p), p->d_partials, 1024, st);
            if (rc) return rc;
            return reduce_partials(p->d_partials, 1024, d_norm2, st);
        }
        return ARECGB_OK;
    }
    const int ntile = (p->nx + kFpBins - 1) / kFpBins;
    dim3 grid(p->ngroups * ntile, fp_slice_blocks(p));
    rc = p->weighting == ARECGB_KB ? launch_fp_kb(A, p->vec, nsc, grid, d_x, d_q, st)
                                   : launch_fp_sq(A, p->vec, nsc, grid, d_x, d_q, st);
    ARECGB_CUDA(cudaGetLastError());
    if (rc) return ARECGB_ERR_ARG;
    if (d_norm2) return reduce_partials(p->d_partials, grid.x * grid.y, d_norm2, st);
    return ARECGB_OK;
}

int back_project(const Plan *p, const float *d_s, float *d_g, double *d_norm2,
                 const int *d_skip, cudaStream_t st) {
    const OpArgs A = make_args(p, d_skip);
    const int nsc = slice_chunks(p);
    dim3 grid(p->ntiles, slice_blocks(p));
    int rc;
    if (p->weighting == ARECGB_LIN)
        rc = launch_bp_lin(A, p->vec, nsc, grid, d_s, d_g, st);
    else if (p->weighting == ARECGB_KB)
        rc = launch_bp_kb(A, p->vec, nsc, grid, d_s, d_g, st);
    else
        rc = launch_bp_sq(A, p->vec, nsc, grid, d_s, d_g, st);
    ARECGB_CUDA(cudaGetLastError());
    if (rc) return ARECGB_ERR_ARG;
    if (d_norm2) return reduce_partials(p->d_partials, grid.x * grid.y, d_norm2, st);
    return ARECGB_OK;
}

}  // namespace arecgb
