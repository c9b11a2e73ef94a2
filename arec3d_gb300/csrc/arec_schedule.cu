// Uneven batches larger than device memory: a resident-subset scheduler over
// the batched CGLS (arec_solver.cu::cgls_batch).
//
// The reference reconstructs one cylinder per run, split over MPI ranks by
// slabs of slices (AREC3D/AREC3D/AREC3D.cpp:293-315 -> areccgls.cpp:245-478).
// Here many cylinders of uneven radius, detector width, slice and angle
// counts are solved on one GPU.  Their inputs and results stay resident; the
// solver workspace (three volume vectors and two sinograms per problem, plus
// the plan's geometry tables) does not fit for all of them at once, so the
// problems are packed into waves whose workspace fits a byte budget (first
// fit, largest first).  Per wave: one plan per problem (without the optional
// projector tables: they would cost 32 B per ray and angle), the optional
// learned warm start per problem (SIRT -> U-Net), then one batched CGLS in
// which every iteration of all the wave's problems is one CUDA graph launch
// (each problem a parallel branch; a converged problem's kernels become
// no-ops).  The wave's plans are destroyed before the next wave.
#include <math.h>
#include <string.h>

#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <chrono>
#include <numeric>
#include <string>
#include <vector>

#include "arec_gb300.h"
#include "arec_internal.cuh"

namespace arecgb {
int cgls_batch(Plan *const *plans, const float *const *d_b, float *const *d_x, const int *warm,
               int n, int maxit, float tol, const double *rnorm_ref, double *const *hist_host,
               arecgb_solve_info *info, cudaStream_t st, const float *const *d_w);
int sirt(Plan *p, const float *d_b, float *d_x, float lam, int maxit, float tol,
         double *hist_host, arecgb_solve_info *info, int verbose, cudaStream_t st);
}  // namespace arecgb

using namespace arecgb;

namespace {

// Detector bins and rays of the reference's cylinder of this radius
// (arecAllocateCylImage, AREC3D/AREC3D/arecImage.cpp:29-86: truncating mask).
void cylinder_counts(double radius, int *nx, int *nrays) {
    const int n = (int)std::lround(2 * radius + 1);
    const int r2 = (int)(radius * radius);
    long long nr = 0;
    for (int iz = 0; iz < n; iz++) {
        const int zs = (int)(iz - radius);
        for (int ix = 0; ix < n; ix++) {
            const int xs = (int)(ix - radius);
            if (zs * zs + xs * xs <= r2) nr++;
        }
    }
    *nx = n;
    *nrays = (int)nr;
}

int round8(int n) { return (n + 7) / 8 * 8; }

}  // namespace

extern "C" {

int arecgb_cylinder_info(double radius, int ny, int *nx, int *nrays, int *ys) {
    if (!(radius >= 0.0) || radius > 8192.0 || ny < 1) {
        set_error("arecgb_cylinder_info: need 0 <= radius <= 8192 and ny >= 1");
        return ARECGB_ERR_ARG;
    }
    int a = 0, b = 0;
    cylinder_counts(radius, &a, &b);
    if (nx) *nx = a;
    if (nrays) *nrays = b;
    if (ys) *ys = round8(ny);
    return 0;
}

int arecgb_solve_uneven(const arecgb_problem *probs, int n, size_t budget_bytes,
                        arecgb_unet *const *nets, int n_nets, int sirt_iters,
                        double sirt_lam_scale, int maxit, float tol, arecgb_solve_info *info,
                        int *wave_of, void *stream) {
    if (!probs || n < 1 || maxit < 0 || n_nets < 0 || sirt_iters < 0 || (n_nets > 0 && !nets)) {
        set_error("arecgb_solve_uneven: bad arguments");
        return ARECGB_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the networks (the same parameters at several image sizes): each problem
    // takes the smallest whose images hold its width
    std::vector<int> netH(n_nets), netB(n_nets);
    size_t img_floats = 0;
    for (int k = 0; k < n_nets; k++) {
        int H = 0, W = 0, B = 0;
        int rc = arecgb_unet_shape(nets[k], &H, &W, &B);
        if (rc) return rc;
        netH[k] = std::min(H, W);
        netB[k] = B;
        img_floats = std::max(img_floats, (size_t)H * W * B);
    }
    std::vector<int> net_of(n, -1);
    // workspace bytes per problem: CGLS's 3 volume + 2 sinogram vectors, the
    // ray table and a margin for the plan's other tables and partials
    std::vector<size_t> bytes(n);
    for (int i = 0; i < n; i++) {
        const arecgb_problem &q = probs[i];
        if (q.weighting < ARECGB_LIN || q.weighting > ARECGB_SQ || q.ny < 1 || q.nangles < 1 ||
            !q.angles || !q.d_b || !q.d_x || !(q.radius >= 0.0) || q.radius > 8192.0) {
            set_error("arecgb_solve_uneven: bad problem " + std::to_string(i));
            return ARECGB_ERR_ARG;
        }
        int nx = 0, nr = 0;
        cylinder_counts(q.radius, &nx, &nr);
        for (int k = 0; k < n_nets; k++)
            if (netH[k] >= nx && (net_of[i] < 0 || netH[k] < netH[net_of[i]])) net_of[i] = k;
        if (n_nets > 0 && net_of[i] < 0) {
            set_error("arecgb_solve_uneven: problem " + std::to_string(i) + " is " +
                      std::to_string(nx) + " bins wide, wider than every network's images");
            return ARECGB_ERR_ARG;
        }
        const size_t ys = (size_t)round8(q.ny);
        bytes[i] = sizeof(float) * (3 * (size_t)nr * ys + 2 * (size_t)q.nangles * nx * ys) +
                   sizeof(float4) * (size_t)nr + (64u << 20);
    }
    // waves: first fit, largest first
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return bytes[a] > bytes[b]; });
    std::vector<std::vector<int>> waves;
    std::vector<size_t> load;
    for (int i : order) {
        size_t w = 0;
        while (w < waves.size() && load[w] + bytes[i] > budget_bytes) w++;
        if (w == waves.size()) {  // a problem above the budget gets a wave of its own
            waves.emplace_back();
            load.push_back(0);
        }
        waves[w].push_back(i);
        load[w] += bytes[i];
    }
    // the network's image scratch, shared by all waves
    float *img[2] = {nullptr, nullptr};
    auto free_img = [&]() {
        cudaFree(img[0]);
        cudaFree(img[1]);
    };
    if (n_nets > 0) {
        for (auto &p : img) {
            cudaError_t e = cudaMalloc(&p, sizeof(float) * img_floats);
            if (e != cudaSuccess) {
                free_img();
                set_error(std::string("arecgb_solve_uneven: ") + cudaGetErrorString(e));
                return cuda_status(e);
            }
        }
    }
    // ARECGB_PROGRESS=1: one line per wave on stderr (problems, seconds of
    // plan creation, warm start and batched CGLS; the phases then synchronise)
    const char *prog_env = getenv("ARECGB_PROGRESS");
    const bool progress = prog_env && prog_env[0] == '1';
    using clk = std::chrono::steady_clock;
    auto lap = [&](clk::time_point &t) {
        if (progress) cudaStreamSynchronize(st);
        const auto now = clk::now();
        const double s_ = std::chrono::duration<double>(now - t).count();
        t = now;
        return s_;
    };
    int rc = 0;
    for (size_t w = 0; !rc && w < waves.size(); w++) {
        const std::vector<int> &wv = waves[w];
        const int m = (int)wv.size();
        clk::time_point t_w = clk::now();
        double t_plan = 0, t_warm = 0, t_cgls = 0;
        std::vector<Plan *> plans(m, nullptr);
        std::vector<const float *> bs(m);
        std::vector<float *> xs(m);
        std::vector<int> warm(m, 0);
        std::vector<double> rref(m, 0.0);
        std::vector<arecgb_solve_info> inf(m);
        for (int j = 0; !rc && j < m; j++) {
            const arecgb_problem &q = probs[wv[j]];
            rc = plan_create(&plans[j], q.weighting, q.radius, q.ny, q.nangles, q.angles, false);
            bs[j] = q.d_b;
            xs[j] = q.d_x;
            if (wave_of) wave_of[wv[j]] = (int)w;
        }
        t_plan = lap(t_w);
        // the learned warm start, problem by problem: the network's input (SIRT
        // at the step the network was trained with, or with sirt_iters = 0 the
        // filtered back projection), then x0 = net(input) scaled back
        for (int j = 0; !rc && n_nets > 0 && j < m; j++) {
            Plan *p = plans[j];
            arecgb_unet *net = nets[net_of[wv[j]]];
            if (sirt_iters == 0) {
                // the filtered sinogram goes to the sinogram scratch CGLS uses next
                if (!p->d_sin[0]) {
                    const size_t ns = sin_floats(p);
                    cudaError_t e = cudaMalloc(&p->d_sin[0], sizeof(float) * ns);
                    if (e == cudaSuccess) e = cudaMemsetAsync(p->d_sin[0], 0, sizeof(float) * ns, st);
                    if (e != cudaSuccess) {
                        set_error(std::string("arecgb_solve_uneven: ") + cudaGetErrorString(e));
                        rc = cuda_status(e);
                        break;
                    }
                }
                if ((rc = ensure_red(p))) break;
                double *d_n2 = p->d_sred + 2 * kSredBlocks;
                rc = fbp(p, bs[j], xs[j], p->d_sin[0], d_n2, st);
                if (!rc) {
                    cudaError_t e = cudaMemcpyAsync(p->h_sred, d_n2, sizeof(double),
                                                    cudaMemcpyDeviceToHost, st);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                    if (e != cudaSuccess) {
                        set_error(std::string("arecgb_solve_uneven: ") + cudaGetErrorString(e));
                        rc = cuda_status(e);
                    }
                }
                rref[j] = rc ? 0.0 : sqrt(p->h_sred[0]);  // ||A^T b||: the cold start's
            } else {
                arecgb_solve_info si;
                memset(&si, 0, sizeof(si));
                const float lam = (float)(sirt_lam_scale / ((double)p->na * (double)p->nx));
                rc = sirt(p, bs[j], xs[j], lam, sirt_iters, 0.0f, nullptr, &si, 0, st);
                rref[j] = si.rnorm0;  // ||A^T b||: the cold start's denominator
            }
            if (!rc)
                rc = arecgb_warm_start(reinterpret_cast<arecgb_plan *>(p), net, xs[j], xs[j],
                                       img[0], img[1], st);
            warm[j] = 1;
        }
        t_warm = lap(t_w);
        if (!rc)
            rc = cgls_batch(plans.data(), bs.data(), xs.data(), warm.data(), m, maxit, tol,
                            rref.data(), nullptr, inf.data(), st, nullptr);
        t_cgls = lap(t_w);
        if (progress)
            fprintf(stderr, "arecgb_solve_uneven: wave %zu of %zu, %d problems (%.1f GB): plans "
                    "%.2f s, warm start %.2f s, CGLS %.2f s\n", w + 1, waves.size(), m,
                    load[w] / 1e9, t_plan, t_warm, t_cgls);
        for (int j = 0; j < m; j++) {
            if (info && !rc) info[wv[j]] = inf[j];
            plan_destroy(plans[j]);
        }
    }
    free_img();
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(std::string("arecgb_solve_uneven: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    return rc;
}

}  // extern "C"
