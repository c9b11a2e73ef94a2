// Device-resident solver state and the element-wise kernels of the solvers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace arecgb {

// Scalars of one CGLS solve, kept in device memory so an iteration needs no
// host round trip.  FP64 throughout (reference areccgls.cpp:269-270).
struct SolveState {
    double gamma, gamma0, alpha;
    double qnorm2, gnorm2;       // written by the projectors' fused reductions
    double rnorm0, rnorm_min, denom, rel;
    float tol;
    int iter, maxit, iterbest, iterations;
    int done, save;
};

int grid_for(size_t n, int per_thread);

}  // namespace arecgb
