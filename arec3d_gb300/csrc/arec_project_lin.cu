// Projector instantiations for weighting ARECGB_LIN (see arec_project_impl.cuh).
#include "arec_project_impl.cuh"

namespace arecgb {

int launch_bp_lin(const OpArgs &A, int vec, int nsc, dim3 grid, const float *s, float *g,
               const CUtensorMap &tms, int use_tma, cudaStream_t st) {
    return launch_bp<ARECGB_LIN>(A, vec, nsc, grid, s, g, tms, use_tma, st);
}

int launch_fp_lin(const OpArgs &A, int vec, const float *x, float *q, cudaStream_t st) {
    return launch_fp<ARECGB_LIN>(A, vec, x, q, st);
}

int launch_lin_index(const OpArgs &A, int *off, int *list, cudaStream_t st) {
    k_lin_index<<<(A.na + 63) / 64, 64, 0, st>>>(A, off, list);
    return 0;
}

}  // namespace arecgb
