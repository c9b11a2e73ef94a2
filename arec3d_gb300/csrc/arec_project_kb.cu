// Projector instantiations for weighting ARECGB_KB (see arec_project_impl.cuh).
#include "arec_project_impl.cuh"

namespace arecgb {

int launch_bp_kb(const OpArgs &A, int vec, int nsc, dim3 grid, const float *s, float *g,
               cudaStream_t st) {
    return launch_bp<ARECGB_KB>(A, vec, nsc, grid, s, g, st);
}

int launch_fp_kb(const OpArgs &A, int vec, int nsc, dim3 grid, const float *x, float *q,
               cudaStream_t st) {
    return launch_fp<ARECGB_KB, kFpBins>(A, vec, nsc, grid, x, q, st);
}

}  // namespace arecgb
