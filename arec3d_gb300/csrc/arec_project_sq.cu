// Projector instantiations for weighting ARECGB_SQ (see arec_project_impl.cuh).
#include "arec_project_impl.cuh"

namespace arecgb {

int launch_bp_sq(const OpArgs &A, int vec, int nsc, dim3 grid, const float *s, float *g,
               const CUtensorMap &tms, int use_tma, cudaStream_t st) {
    return launch_bp<ARECGB_SQ>(A, vec, nsc, grid, s, g, tms, use_tma, st);
}

int launch_fpb_sq(const OpArgs &A, int vec, dim3 grid, const float *x, float *q, int g0, int ngo,
                int lo, int hi, const CUtensorMap &tmx, const CUtensorMap &tmxT, cudaStream_t st) {
    return launch_fpb<ARECGB_SQ, kFpBins>(A, vec, grid, x, q, g0, ngo, lo, hi, tmx, tmxT, st);
}

int launch_tables_sq(const OpArgs &A, int ntiles, float4 *taps, float4 *bpw, int2 *bpf,
                    cudaStream_t st) {
    return launch_tables<ARECGB_SQ>(A, ntiles, taps, bpw, bpf, st);
}

}  // namespace arecgb
