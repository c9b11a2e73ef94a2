// C ABI of libarec_gb300 (include/arec_gb300.h) and the reference-compatible
// layer (include/arec_compat.h): the reference's own entry points over host
// `arecImage` buffers, backed by the device kernels.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "arec_compat.h"
#include "arec_internal.cuh"

namespace arecgb {
const char *last_error();
int cgls_batch(Plan *const *plans, const float *const *d_b, float *const *d_x, const int *warm,
               int n, int maxit, float tol, const double *rnorm_ref, double *const *hist_host,
               arecgb_solve_info *info, cudaStream_t st, const float *const *d_w);
int cgls_stat(Plan *p, const float *d_b, float *d_x, int warm, int maxit, float tol,
              double *hist_host, arecgb_solve_info *info, cudaStream_t st);
int cgls(Plan *p, const float *d_b, float *d_x, int warm, int maxit, float tol, double rnorm_ref,
         double *hist_host, arecgb_solve_info *info, cudaStream_t st);
int sirt(Plan *p, const float *d_b, float *d_x, float lam, int maxit, float tol,
         double *hist_host, arecgb_solve_info *info, int verbose, cudaStream_t st);
int cc_shifts(const float *d1, const float *d2, int nz, int ny, int nx, float *sx, float *sy,
              int *ix, int *iy, cudaStream_t st);
int ccorr_image(const float *dx, const float *dy, float *dc, int ny, int nx, cudaStream_t st);
int fshift_stack(const float *d_in, float *d_out, int nz, int ny, int nx, const float *d_sx,
                 const float *d_sy, cudaStream_t st);
int peak_search(const float *dc, int nz, int ny, int nx, float *sx, float *sy, int *ix, int *iy,
                cudaStream_t st);
int rot_cc_angles(const float *d1, const float *d2, int nz, int ny, int nx, int r2, float *d_angles,
                  cudaStream_t st);
int rotate_stack(float *d_img, const float *d_ref, int nz, int ny, int nx, float *d_angles,
                 int kind, int *n_rot, double *mean_cc, cudaStream_t st);
int ncc_filtered(const float *d_a, const float *d_a2, const float *d_b, int nz, int ny, int nx,
                 double *d_cc, int npairs, cudaStream_t st);
int take_log(float *d_x, size_t n, cudaStream_t st);
int profile_shifts(const float *d_prof, int prof_y, int prof_x, int pad, int successive,
                   double *shifts, double *spread, cudaStream_t st);
int periodic_decomp(float *d, int nz, int ny, int nx, float *s_out, cudaStream_t st);
}  // namespace arecgb

using namespace arecgb;

static Plan *P(arecgb_plan *p) { return reinterpret_cast<Plan *>(p); }
static const Plan *P(const arecgb_plan *p) { return reinterpret_cast<const Plan *>(p); }

static int bind_device(const Plan *p) {
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != p->device) ARECGB_CUDA(cudaSetDevice(p->device));
    return 0;
}

// ===========================================================================
// Core C ABI.
extern "C" {

const char *arecgb_last_error(void) { return last_error(); }
int arecgb_version(void) { return 10000; }

int arecgb_plan_create(arecgb_plan **plan, int weighting, double radius, int ny, int nangles,
                       const float *angles) {
    if (!plan) {
        set_error("arecgb_plan_create: null plan pointer");
        return ARECGB_ERR_ARG;
    }
    Plan *p = nullptr;
    int rc = plan_create(&p, weighting, radius, ny, nangles, angles);
    *plan = reinterpret_cast<arecgb_plan *>(p);
    return rc;
}

int arecgb_plan_destroy(arecgb_plan *plan) {
    plan_destroy(P(plan));
    return ARECGB_OK;
}

int arecgb_plan_info(const arecgb_plan *plan, int *nx, int *nrays, int *ys) {
    if (!plan) {
        set_error("arecgb_plan_info: null plan");
        return ARECGB_ERR_ARG;
    }
    if (nx) *nx = P(plan)->nx;
    if (nrays) *nrays = P(plan)->nrays;
    if (ys) *ys = P(plan)->ys;
    return ARECGB_OK;
}

int arecgb_plan_check(arecgb_plan *plan) {
    if (!plan) return ARECGB_ERR_ARG;
    int rc = bind_device(P(plan));
    if (rc) return rc;
    int flag = 0;
    ARECGB_CUDA(cudaMemcpy(&flag, P(plan)->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    ARECGB_CUDA(cudaMemset(P(plan)->d_err, 0, sizeof(int)));
    return flag;
}

int arecgb_project(arecgb_plan *plan, const float *d_x, float *d_q, double *d_norm2,
                   void *stream) {
    if (!plan || !d_x || !d_q) {
        set_error("arecgb_project: null argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(P(plan));
    if (rc) return rc;
    return forward_project(P(plan), d_x, d_q, d_norm2, nullptr, (cudaStream_t)stream);
}

int arecgb_backproject(arecgb_plan *plan, const float *d_s, float *d_g, double *d_norm2,
                       void *stream) {
    if (!plan || !d_s || !d_g) {
        set_error("arecgb_backproject: null argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(P(plan));
    if (rc) return rc;
    return back_project(P(plan), d_s, d_g, d_norm2, nullptr, (cudaStream_t)stream);
}

int arecgb_fbp(arecgb_plan *plan, const float *d_b, float *d_x, float *d_work,
               double *d_atb_norm2, void *stream) {
    if (!plan || !d_b || !d_x || !d_work) {
        set_error("arecgb_fbp: null argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(P(plan));
    if (rc) return rc;
    return fbp(P(plan), d_b, d_x, d_work, d_atb_norm2, (cudaStream_t)stream);
}

int arecgb_ramp_filter(arecgb_plan *plan, const float *d_s, float *d_f, void *stream) {
    if (!plan || !d_s || !d_f) {
        set_error("arecgb_ramp_filter: null argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(P(plan));
    if (rc) return rc;
    return ramp_filter(P(plan), d_s, d_f, (cudaStream_t)stream);
}

int arecgb_cgls(arecgb_plan *plan, const float *d_b, float *d_x, int warm, int maxit, float tol,
                double rnorm_ref, double *rel_history, arecgb_solve_info *info, void *stream) {
    if (!plan || !d_b || !d_x || maxit < 0) {
        set_error("arecgb_cgls: bad argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(P(plan));
    if (rc) return rc;
    return cgls(P(plan), d_b, d_x, warm, maxit, tol, rnorm_ref, rel_history, info,
                (cudaStream_t)stream);
}

int arecgb_sirt(arecgb_plan *plan, const float *d_b, float *d_x, float lam, int maxit, float tol,
                double *rel_history, arecgb_solve_info *info, void *stream) {
    if (!plan || !d_b || !d_x || maxit < 0) {
        set_error("arecgb_sirt: bad argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(P(plan));
    if (rc) return rc;
    return sirt(P(plan), d_b, d_x, lam, maxit, tol, rel_history, info, 0, (cudaStream_t)stream);
}

int arecgb_sino_from_reference(const float *d_ref, float *d_dev, int na, int ny, int nx, int ys,
                               void *stream) {
    return sino_to_device_layout(d_ref, d_dev, na, ny, nx, ys, (cudaStream_t)stream);
}

int arecgb_sino_to_reference(const float *d_dev, float *d_ref, int na, int ny, int nx, int ys,
                             void *stream) {
    return sino_to_reference_layout(d_dev, d_ref, na, ny, nx, ys, (cudaStream_t)stream);
}

int arecgb_cgls_batch(arecgb_plan *const *plans, const float *const *d_b, float *const *d_x,
                      const int *warm, int n, int maxit, float tol, const double *rnorm_ref,
                      arecgb_solve_info *info, void *stream) {
    if (n < 1 || !plans) {
        set_error("arecgb_cgls_batch: bad arguments");
        return ARECGB_ERR_ARG;
    }
    return cgls_batch(reinterpret_cast<Plan *const *>(plans), d_b, d_x, warm, n, maxit, tol,
                      rnorm_ref, nullptr, info, (cudaStream_t)stream, nullptr);
}

int arecgb_cgls_stat(arecgb_plan *plan, const float *d_b, float *d_x, int warm, int maxit,
                     float tol, double *rel_history, arecgb_solve_info *info, void *stream) {
    if (!plan || !d_b || !d_x) {
        set_error("arecgb_cgls_stat: null argument");
        return ARECGB_ERR_ARG;
    }
    return cgls_stat(P(plan), d_b, d_x, warm, maxit, tol, rel_history, info, (cudaStream_t)stream);
}

int arecgb_plan_timing(arecgb_plan *plan, int mode, double *fp_ms, long long *fp_calls,
                       double *bp_ms, long long *bp_calls) {
    if (!plan || mode < 0 || mode > 2) {
        set_error("arecgb_plan_timing: bad arguments");
        return ARECGB_ERR_ARG;
    }
    return plan_timing(P(plan), mode, fp_ms, fp_calls, bp_ms, bp_calls);
}

long long arecgb_launch_count(void) { return launch_count(); }

int arecgb_plan_autotune(arecgb_plan *plan, float *d_x, float *d_q, int *fp_band, int *bp_nsc,
                         void *stream) {
    if (!plan || !d_x || !d_q) {
        set_error("arecgb_plan_autotune: null argument");
        return ARECGB_ERR_ARG;
    }
    int rc = plan_autotune(P(plan), d_x, d_q, (cudaStream_t)stream);
    if (fp_band) *fp_band = P(plan)->fp_band;
    if (bp_nsc) *bp_nsc = P(plan)->bp_nsc;
    return rc;
}

int arecgb_plan_set_shapes(arecgb_plan *plan, int fp_band, int fp_vec, int bp_vec, int bp_nsc) {
    if (!plan) {
        set_error("arecgb_plan_set_shapes: null plan");
        return ARECGB_ERR_ARG;
    }
    Plan *p = reinterpret_cast<Plan *>(plan);
    auto vec_ok = [&](int v) { return v == p->vec || (v == p->vec / 2 && v >= 1); };
    if ((fp_band != 32 && fp_band != 64 && fp_band != 128) || !vec_ok(fp_vec) || !vec_ok(bp_vec) ||
        (bp_nsc != 1 && bp_nsc != 2)) {
        set_error("arecgb_plan_set_shapes: band must be 32, 64 or 128, vectors the plan's VEC or "
                  "half of it, chunks 1 or 2");
        return ARECGB_ERR_ARG;
    }
    p->fp_band = fp_band;
    p->fp_vec = fp_vec;
    p->bp_vec = bp_vec;
    p->bp_nsc = bp_nsc;
    p->tuned = 1;
    return 0;
}

long long arecgb_plan_table_bytes(const arecgb_plan *plan) {
    return plan ? (long long)reinterpret_cast<const Plan *>(plan)->table_bytes : 0;
}

int arecgb_plan_shapes(const arecgb_plan *plan, int *fp_band, int *fp_vec, int *bp_vec,
                       int *bp_nsc) {
    if (!plan) {
        set_error("arecgb_plan_shapes: null plan");
        return ARECGB_ERR_ARG;
    }
    const Plan *p = reinterpret_cast<const Plan *>(plan);
    if (fp_band) *fp_band = p->fp_band;
    if (fp_vec) *fp_vec = p->fp_vec ? p->fp_vec : p->vec;
    if (bp_vec) *bp_vec = p->bp_vec ? p->bp_vec : p->vec;
    if (bp_nsc) *bp_nsc = p->bp_nsc;
    return 0;
}

int arecgb_cc_shifts(const float *d_img1, const float *d_img2, int nz, int ny, int nx,
                     float *d_sx, float *d_sy, int *d_ix, int *d_iy, void *stream) {
    return cc_shifts(d_img1, d_img2, nz, ny, nx, d_sx, d_sy, d_ix, d_iy, (cudaStream_t)stream);
}

int arecgb_ccorr2d_device(const float *d_x, const float *d_y, float *d_c, int ny, int nx,
                          void *stream) {
    return ccorr_image(d_x, d_y, d_c, ny, nx, (cudaStream_t)stream);
}

int arecgb_fshift2d_device(const float *d_in, float *d_out, int nz, int ny, int nx,
                           const float *d_sx, const float *d_sy, void *stream) {
    return fshift_stack(d_in, d_out, nz, ny, nx, d_sx, d_sy, (cudaStream_t)stream);
}

int arecgb_rot_cc_images(const float *d_img1, const float *d_img2, int nz, int ny, int nx, int r2,
                         float *d_angles, void *stream) {
    return rot_cc_angles(d_img1, d_img2, nz, ny, nx, r2, d_angles, (cudaStream_t)stream);
}

int arecgb_rotate_images(float *d_img, int nz, int ny, int nx, const float *d_angles,
                         void *stream) {
    // kind 0 only reads the angles
    return rotate_stack(d_img, nullptr, nz, ny, nx, const_cast<float *>(d_angles), 0, nullptr,
                        nullptr, (cudaStream_t)stream);
}

int arecgb_rotate_images_skew(float *d_img, int nz, int ny, int nx, float *d_angles,
                              void *stream) {
    return rotate_stack(d_img, nullptr, nz, ny, nx, d_angles, 1, nullptr, nullptr,
                        (cudaStream_t)stream);
}

int arecgb_rotate_images_skew_safe(float *d_img, const float *d_ref, int nz, int ny, int nx,
                                   float *d_angles, int *n_rot, double *mean_cc, void *stream) {
    return rotate_stack(d_img, d_ref, nz, ny, nx, d_angles, 2, n_rot, mean_cc,
                        (cudaStream_t)stream);
}

int arecgb_ncc_filtered(const float *d_a, const float *d_b, int nz, int ny, int nx, double *d_cc,
                        void *stream) {
    return ncc_filtered(d_a, nullptr, d_b, nz, ny, nx, d_cc, 1, (cudaStream_t)stream);
}

int arecgb_profile_shifts(const float *d_profiles, int prof_y, int prof_x, int pad,
                          int successive, double *shifts, double *spread, void *stream) {
    return profile_shifts(d_profiles, prof_y, prof_x, pad, successive, shifts, spread,
                          (cudaStream_t)stream);
}

int arecgb_take_log(float *d_data, size_t n, void *stream) {
    return take_log(d_data, n, (cudaStream_t)stream);
}

int arecgb_periodic_decomposition(float *d_images, int nz, int ny, int nx, float *d_smooth,
                                  void *stream) {
    return periodic_decomp(d_images, nz, ny, nx, d_smooth, (cudaStream_t)stream);
}

}  // extern "C"

// ===========================================================================
// Reference-compatible layer.

namespace {

std::mutex g_mu;

bool quiet() {
    const char *q = getenv("ARECGB_QUIET");
    return q && q[0] && q[0] != '0';
}

// Plans keyed by geometry; the compatible entry points rebuild nothing when
// called again on the same cylinder and angles.
struct Key {
    int w;
    double r;
    int ny, dev;
    std::vector<float> ang;
    bool operator<(const Key &o) const {
        return std::tie(w, r, ny, dev, ang) < std::tie(o.w, o.r, o.ny, o.dev, o.ang);
    }
};
std::map<Key, Plan *> g_plans;
std::vector<Key> g_lru;
constexpr size_t kMaxPlans = 6;

int cached_plan(Plan **out, int w, double radius, int ny, int na, const float *angles) {
    int dev = 0;
    cudaGetDevice(&dev);
    Key k{w, radius, ny, dev, std::vector<float>(angles, angles + na)};
    auto it = g_plans.find(k);
    if (it != g_plans.end()) {
        *out = it->second;
        auto pos = std::find_if(g_lru.begin(), g_lru.end(),
                                [&](const Key &x) { return !(x < k) && !(k < x); });
        if (pos != g_lru.end()) {
            g_lru.erase(pos);
            g_lru.push_back(k);
        }
        return 0;
    }
    while (g_plans.size() >= kMaxPlans && !g_lru.empty()) {
        auto old = g_plans.find(g_lru.front());
        if (old != g_plans.end()) {
            plan_destroy(old->second);
            g_plans.erase(old);
        }
        g_lru.erase(g_lru.begin());
    }
    Plan *p = nullptr;
    int rc = plan_create(&p, w, radius, ny, na, angles);
    if (rc) return rc;
    g_plans[k] = p;
    g_lru.push_back(k);
    *out = p;
    return 0;
}

int ensure(float **buf, size_t n) {
    if (*buf) return 0;
    ARECGB_CUDA(cudaMalloc(buf, sizeof(float) * std::max<size_t>(n, 1)));
    ARECGB_CUDA(cudaMemset(*buf, 0, sizeof(float) * std::max<size_t>(n, 1)));
    return 0;
}

int ensure_stage(Plan *p, size_t n) {
    if (p->d_stage && p->stage_floats >= n) return 0;
    cudaFree(p->d_stage);
    p->d_stage = nullptr;
    p->stage_floats = 0;
    ARECGB_CUDA(cudaMalloc(&p->d_stage, sizeof(float) * std::max<size_t>(n, 1)));
    p->stage_floats = n;
    return 0;
}

// Host -> device volume ([nrays][ny] -> [nrays][ys]).
int upload_volume(Plan *p, const float *h, float *d) {
    ARECGB_CUDA(cudaMemcpy2DAsync(d, sizeof(float) * p->ys, h, sizeof(float) * p->ny,
                                  sizeof(float) * p->ny, p->nrays, cudaMemcpyHostToDevice,
                                  p->stream));
    return 0;
}

int download_volume(Plan *p, const float *d, float *h) {
    ARECGB_CUDA(cudaMemcpy2DAsync(h, sizeof(float) * p->ny, d, sizeof(float) * p->ys,
                                  sizeof(float) * p->ny, p->nrays, cudaMemcpyDeviceToHost,
                                  p->stream));
    return 0;
}

// Host [na][ny][nx] -> device [na][nx][ys].
int upload_sino(Plan *p, const float *h, float *d) {
    const size_t n = (size_t)p->na * p->ny * p->nx;
    int rc = ensure_stage(p, n);
    if (rc) return rc;
    ARECGB_CUDA(cudaMemcpyAsync(p->d_stage, h, sizeof(float) * n, cudaMemcpyHostToDevice,
                                p->stream));
    return sino_to_device_layout(p->d_stage, d, p->na, p->ny, p->nx, p->ys, p->stream);
}

int download_sino(Plan *p, const float *d, float *h) {
    const size_t n = (size_t)p->na * p->ny * p->nx;
    int rc = ensure_stage(p, n);
    if (rc) return rc;
    rc = sino_to_reference_layout(d, p->d_stage, p->na, p->ny, p->nx, p->ys, p->stream);
    if (rc) return rc;
    ARECGB_CUDA(cudaMemcpyAsync(h, p->d_stage, sizeof(float) * n, cudaMemcpyDeviceToHost,
                                p->stream));
    return 0;
}

int sync_plan(Plan *p) {
    ARECGB_CUDA(cudaStreamSynchronize(p->stream));
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

// Host replica of arecAllocateCylImage (AREC3D/AREC3D/arecImage.cpp:29-86).
int alloc_cyl(arecImage *im, double radius, int height) {
    int nx = (int)std::round(2 * radius + 1);
    im->nx = nx;
    im->ny = height;
    im->nz = nx;
    im->radius = radius;
    im->height = height;
    int r2 = (int)(radius * radius);
    int nr = 0;
    for (int iz = 0; iz < nx; iz++) {
        int zs = (int)(iz - radius);
        for (int ix = 0; ix < nx; ix++) {
            int xs = (int)(ix - radius);
            if (zs * zs + xs * xs <= r2) nr++;
        }
    }
    im->nrays = nr;
    im->nnz = nr * height;
    im->data = (float *)calloc((size_t)nr * height, sizeof(float));
    im->cord = (int *)calloc((size_t)nr * 2, sizeof(int));
    im->is_cyl = 1;
    if (!im->data || !im->cord) return -1;
    int k = 0;
    for (int iz = 0; iz < nx; iz++) {
        int zs = (int)(iz - radius);
        for (int ix = 0; ix < nx; ix++) {
            int xs = (int)(ix - radius);
            if (zs * zs + xs * xs <= r2) {
                im->cord[2 * k] = ix;
                im->cord[2 * k + 1] = iz;
                k++;
            }
        }
    }
    return 0;
}

thread_local std::vector<double> g_trace;
thread_local arecgb_solve_info g_trace_info;

// arecProject2D[_KB|_SQ] (AREC3D/AREC3D/arecproject.cpp:19,351,540).
int compat_project(int w, const arecImage &cyl, const float *angles, int nangles,
                   arecImage *proj) {
    if (!cyl.is_cyl) {
        if (!quiet()) fprintf(stderr, "invalid input volume format. Must be cylindrical!\n");
        return 1;
    }
    if (proj->nx != cyl.nx || proj->ny != cyl.ny) {
        if (!quiet()) fprintf(stderr, "arecProject2D: inconsistent dimension!\n");
        return 2;
    }
    if (cyl.nnz != cyl.nrays * cyl.ny || nangles > proj->nz || nangles < 0) {
        if (!quiet()) fprintf(stderr, "arecProject2D: problem with nnz count!\n");
        return 2;
    }
    const size_t per = (size_t)proj->nx * proj->ny;
    if (nangles == 0) {
        memset(proj->data, 0, sizeof(float) * per * proj->nz);
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    Plan *p = nullptr;
    int rc = cached_plan(&p, w, cyl.radius, cyl.ny, nangles, angles);
    if (rc) return rc;
    if (p->nrays != cyl.nrays || p->nx != cyl.nx) {
        set_error("arecProject2D: cylinder does not match its radius");
        return 2;
    }
    if ((rc = ensure(&p->d_vol[3], vol_floats(p))) || (rc = ensure(&p->d_sin[2], sin_floats(p))))
        return rc;
    if ((rc = upload_volume(p, cyl.data, p->d_vol[3]))) return rc;
    if ((rc = forward_project(p, p->d_vol[3], p->d_sin[2], nullptr, nullptr, p->stream)))
        return rc;
    if ((rc = download_sino(p, p->d_sin[2], proj->data))) return rc;
    if ((rc = sync_plan(p))) return rc;
    if (proj->nz > nangles)
        memset(proj->data + per * nangles, 0, sizeof(float) * per * (proj->nz - nangles));
    return 0;
}

// arecBackProject2D[_KB|_SQ] (arecproject.cpp:109,447,650).
int compat_backproject(int w, const arecImage &img, const float *angles, int nangles,
                       arecImage *vol) {
    if (img.nz != nangles) return 1;
    if (vol->nx != img.nx || vol->ny != img.ny) {
        if (!quiet()) fprintf(stderr, "arecBackProject2D: image and volume sizes don't match\n");
        return -1;
    }
    if (!vol->is_cyl) {
        if (!quiet())
            fprintf(stderr, "arecBackProject2D: cylindrical volume not properly set!\n");
        return -1;
    }
    if (vol->nnz != vol->nrays * vol->ny) {
        if (!quiet()) fprintf(stderr, "arecProject2D: problem with nnz count!\n");
        return 2;
    }
    if (nangles == 0) {
        memset(vol->data, 0, sizeof(float) * vol->nnz);
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    Plan *p = nullptr;
    int rc = cached_plan(&p, w, vol->radius, vol->ny, nangles, angles);
    if (rc) return rc;
    if (p->nrays != vol->nrays || p->nx != vol->nx) {
        set_error("arecBackProject2D: cylinder does not match its radius");
        return -1;
    }
    if ((rc = ensure(&p->d_vol[3], vol_floats(p))) || (rc = ensure(&p->d_sin[2], sin_floats(p))))
        return rc;
    if ((rc = upload_sino(p, img.data, p->d_sin[2]))) return rc;
    if ((rc = back_project(p, p->d_sin[2], p->d_vol[3], nullptr, nullptr, p->stream))) return rc;
    if ((rc = download_volume(p, p->d_vol[3], vol->data))) return rc;
    return sync_plan(p);
}

// cyl_cgls[_KB|_SQ] and cyl_sirt[_KB|_SQ].
// Weight range line of init_weights (areccgls_stat.cpp:36-44), from the host images.
static void print_stat_weight_range(const arecImage &im) {
    const int nx = im.nx;
    std::vector<double> hx(nx);
    const double alpha = 0.5, pi = std::atan(1.0) * 4.0, A = 2.0 * pi / alpha;
    const double xa = 0.5 * alpha * (nx - 1), xb = (1.0 - 0.5 * alpha) * (nx - 1);
    for (int x = 0; x < nx; x++) {
        const double va = 0.5 * (1.0 + std::cos(A * (1.0 * x / (nx - 1) - alpha / 2)));
        const double vb = 0.5 * (1.0 + std::cos(A * (1.0 * x / (nx - 1) - 1.0 + alpha / 2)));
        hx[x] = x < xa ? va : (x > xb ? vb : 1.0);
    }
    float mn = 1e6f, mx = -1e6f;
    const size_t n = (size_t)im.nx * im.ny * im.nz;
    for (size_t i = 0; i < n; i++) {
        const float w = (float)((double)expf(-im.data[i]) * hx[i % nx]);
        mn = std::min(mn, w);
        mx = std::max(mx, w);
    }
    printf("Statweight min: %f max: %f \n", mn, mx);
}

int compat_solve(bool is_cgls, int w, const arecImage &images, const float *angles,
                 arecImage *xvol, float lam, int maxit, float tol, bool stat = false) {
    const int nx = images.nx, ny = images.ny, nz = images.nz;
    // radius = 0.5*(nx-1) (areccgls.cpp:49, arecsirt.cpp:37); the KB CGLS and
    // the weighted CGLS use the integer nx/2 (areccgls_KB.cpp:37,
    // areccgls_stat.cpp:73), which fails for even nx.
    const bool kb_int_radius = is_cgls && (w == ARECGB_KB || stat);
    if (stat && !quiet()) print_stat_weight_range(images);
    const double radius = kb_int_radius ? (double)(nx / 2) : 0.5 * (nx - 1);
    const bool v = !quiet();
    const bool warm = xvol->data != NULL;
    if (!warm) {
        if (is_cgls && v) printf("mypid = 0, null data\n");
        if (alloc_cyl(xvol, radius, ny)) {
            set_error("solver: host allocation failed");
            return ARECGB_ERR_NOMEM;
        }
    }
    if (kb_int_radius && (nx % 2 == 0)) {
        // The reference's gradient volume then has nx+1 columns and the first
        // back-projection returns -1 (areccgls_KB.cpp:112-113).
        return -1;
    }
    if (xvol->nrays <= 0 || xvol->nnz != xvol->nrays * ny) {
        set_error("solver: xvol does not match the images");
        return 2;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    Plan *p = nullptr;
    int rc = cached_plan(&p, w, radius, ny, nz, angles);
    if (rc) return rc;
    if (p->nrays != xvol->nrays) {
        set_error("solver: xvol does not match the images");
        return 2;
    }
    if ((rc = ensure(&p->d_vol[3], vol_floats(p))) || (rc = ensure(&p->d_sin[2], sin_floats(p))))
        return rc;
    if ((rc = upload_sino(p, images.data, p->d_sin[2]))) return rc;
    if (is_cgls && warm && (rc = upload_volume(p, xvol->data, p->d_vol[3]))) return rc;
    if (v) {
        printf("%snrays = %d, nnz = %d\n", is_cgls && (w == ARECGB_SQ || stat) ? "cyl: " : "",
               xvol->nrays, xvol->nnz);
        if (kb_int_radius)
            printf("nx = %d, ny = %d, radius = %d, height = %d\n", nx, ny, (int)radius, ny);
        else
            printf("nx = %d, ny = %d, radius = %4.2f, height = %d\n", nx, ny, radius, ny);
    }
    std::vector<double> hist((size_t)std::max(maxit, 1), 0.0);
    arecgb_solve_info info;
    memset(&info, 0, sizeof(info));
    const auto t0 = std::chrono::steady_clock::now();
    if (is_cgls && stat)
        rc = cgls_stat(p, p->d_sin[2], p->d_vol[3], warm ? 1 : 0, maxit, tol, hist.data(), &info,
                       p->stream);
    else if (is_cgls)
        rc = cgls(p, p->d_sin[2], p->d_vol[3], warm ? 1 : 0, maxit, tol, 0.0, hist.data(), &info,
                  p->stream);
    else
        rc = sirt(p, p->d_sin[2], p->d_vol[3], lam, maxit, tol, hist.data(), &info, v ? 1 : 0,
                  p->stream);
    if (rc) return rc;
    if ((rc = download_volume(p, p->d_vol[3], xvol->data))) return rc;
    if ((rc = sync_plan(p))) return rc;
    g_trace.assign(hist.begin(), hist.begin() + std::min(info.iterations, maxit));
    g_trace_info = info;
    if (is_cgls && v) {
        printf("CG iter = 0, resnrm = %11.3e\n", info.rnorm0);
        for (int i = 0; i < std::min(info.iterations, maxit); i++)
            printf("CG iter = %3d, rnorm / bnorm = %11.3e, rnorm = %11.3e\n", i + 1, hist[i],
                   hist[i] * info.rnorm0);
        if (info.iterations > 0 && hist[info.iterations - 1] < tol)
            printf("Terminating with rnorm/bnorm = %11.3e, tol = %11.3e, ",
                   hist[info.iterations - 1], tol);
        if (info.iterbest < maxit - 1) printf("retrieve the best solution\n");
    }
    if (v) {
        const double secs =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        printf("Total time in %s = %11.3e\n", is_cgls ? "CG" : "SIRT", secs);
    }
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// extern "C" aliases for C/FFI callers.
extern "C" {

int arecgb_reconstruct_host(arecgb_plan *plan, const float *b_host, float *x_host,
                            arecgb_unet *net, int sirt_iters, float sirt_lam, int maxit,
                            float tol, arecgb_solve_info *info, void *stream) {
    Plan *p = reinterpret_cast<Plan *>(plan);
    if (!p || !b_host || !x_host || maxit < 0 || sirt_iters < 0) {
        set_error("arecgb_reconstruct_host: bad argument");
        return ARECGB_ERR_ARG;
    }
    int rc = bind_device(p);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nsin = (size_t)p->na * p->ny * p->nx;
    // ARECGB_PROGRESS=1: the phases' seconds on stderr (each phase then synchronises)
    const char *prog_env = getenv("ARECGB_PROGRESS");
    const bool progress = prog_env && prog_env[0] == '1';
    using clk = std::chrono::steady_clock;
    clk::time_point t_ph = clk::now();
    double ph[6] = {0, 0, 0, 0, 0, 0};  // upload, layout, input, network, CGLS, download
    auto lap = [&](int k) {
        if (!progress) return;
        cudaStreamSynchronize(st);
        const auto now = clk::now();
        ph[k] += std::chrono::duration<double>(now - t_ph).count();
        t_ph = now;
    };
    if ((rc = ensure(&p->d_vol[3], vol_floats(p))) || (rc = ensure(&p->d_sin[2], sin_floats(p))) ||
        (rc = ensure_stage(p, nsin)))
        return rc;
    int H = 0, W = 0, B = 0;
    if (net) {
        if ((rc = arecgb_unet_shape(net, &H, &W, &B))) return rc;
        const size_t n = (size_t)H * W * B;
        if (p->img_floats < n) {
            for (auto &v : p->d_img) {
                cudaFree(v);
                v = nullptr;
            }
            p->img_floats = 0;
            for (auto &v : p->d_img) ARECGB_CUDA(cudaMalloc(&v, sizeof(float) * n));
            p->img_floats = n;
        }
    }
    float *d_b = p->d_sin[2], *d_x = p->d_vol[3];
    lap(5);  // (allocations on first use: not a phase)
    ph[5] = 0;
    ARECGB_CUDA(cudaMemcpyAsync(p->d_stage, b_host, sizeof(float) * nsin, cudaMemcpyHostToDevice,
                                st));
    lap(0);
    if ((rc = sino_to_device_layout(p->d_stage, d_b, p->na, p->ny, p->nx, p->ys, st))) return rc;
    lap(1);
    arecgb_solve_info si, ci;
    memset(&si, 0, sizeof(si));
    memset(&ci, 0, sizeof(ci));
    if (net && sirt_iters == 0) {
        // the filtered back projection as the network's input; ||A^T b||, the
        // cold start's denominator, from one more back projection
        if ((rc = ensure(&p->d_sin[0], sin_floats(p))) || (rc = ensure_red(p))) return rc;
        double *d_n2 = p->d_sred + 2 * kSredBlocks;
        if ((rc = fbp(p, d_b, d_x, p->d_sin[0], d_n2, st))) return rc;
        ARECGB_CUDA(cudaMemcpyAsync(p->h_sred, d_n2, sizeof(double), cudaMemcpyDeviceToHost, st));
        lap(2);
        if ((rc = arecgb_warm_start(plan, net, d_x, d_x, p->d_img[0], p->d_img[1], st)))
            return rc;
        ARECGB_CUDA(cudaStreamSynchronize(st));
        lap(3);
        rc = cgls(p, d_b, d_x, 1, maxit, tol, sqrt(p->h_sred[0]), nullptr, &ci, st);
    } else if (net) {
        if ((rc = sirt(p, d_b, d_x, sirt_lam, sirt_iters, 0.0f, nullptr, &si, 0, st))) return rc;
        lap(2);
        if ((rc = arecgb_warm_start(plan, net, d_x, d_x, p->d_img[0], p->d_img[1], st)))
            return rc;
        lap(3);
        rc = cgls(p, d_b, d_x, 1, maxit, tol, si.rnorm0, nullptr, &ci, st);
    } else {
        rc = cgls(p, d_b, d_x, 0, maxit, tol, 0.0, nullptr, &ci, st);
    }
    if (rc) return rc;
    lap(4);
    ARECGB_CUDA(cudaMemcpy2DAsync(x_host, sizeof(float) * p->ny, d_x, sizeof(float) * p->ys,
                                  sizeof(float) * p->ny, p->nrays, cudaMemcpyDeviceToHost, st));
    ARECGB_CUDA(cudaStreamSynchronize(st));
    lap(5);
    if (progress)
        fprintf(stderr, "arecgb_reconstruct_host: upload %.3f s, layout %.3f s, first "
                "reconstruction %.3f s, network %.3f s, CGLS %.3f s, download %.3f s\n",
                ph[0], ph[1], ph[2], ph[3], ph[4], ph[5]);
    if (info) *info = ci;
    return 0;
}

int arecgb_arecAllocateCBImage(arecImage *cb, int nx, int ny, int nz) {
    cb->nx = nx;
    cb->ny = ny;
    cb->nz = nz;
    cb->data = (float *)calloc((size_t)nx * ny * nz, sizeof(float));
    cb->is_cyl = 0;
    cb->cord = NULL;
    return cb->data ? 0 : -1;
}

int arecgb_arecAllocateCylImage(arecImage *cyl, double radius, int height) {
    return alloc_cyl(cyl, radius, height);
}

// ImageCyl2CB (AREC3D/AREC3D/arecImage.cpp:163-232): scatter [ray][y] into the cube.
int arecgb_ImageCyl2CB(arecImage cyl, arecImage cb, int nx, int ny, int nz) {
    if (!cyl.data) return -1;
    if (nx != cb.nx || ny != cb.ny || nz != cb.nz) return 1;
    if (nx != 2 * cyl.radius + 1 || nz != 2 * cyl.radius + 1 || ny != cyl.height) return 1;
    if (!cb.data) return -1;
    for (int j = 0; j < cyl.nrays; j++) {
        int ix = cyl.cord[2 * j], iz = cyl.cord[2 * j + 1];
        if (iz >= nz || ix >= nx) return -2;
        for (int iy = 0; iy < ny; iy++)
            cb.data[((size_t)iz * ny + iy) * nx + ix] = cyl.data[(size_t)j * ny + iy];
    }
    return 0;
}

// ImageCB2Cyl (arecImage.cpp:88-161): gather the disk of the cube into [ray][y].
int arecgb_ImageCB2Cyl(arecImage cb, arecImage cyl, int xcent, int zcent, double radius,
                       int height) {
    (void)xcent;
    (void)zcent;
    (void)radius;
    (void)height;
    if (!cyl.data) return -1;
    radius = cyl.radius;
    height = cyl.height;
    if (cyl.nnz <= 0 || cyl.nrays <= 0 || radius <= 0 || height <= 0) return 1;
    if (!cyl.cord) return -1;
    const int nx = cb.nx, ny = cb.ny, nz = cb.nz;
    int r2 = (int)(radius * radius), nnz = 0, nr = 0;
    for (int iz = 0; iz < nz; iz++) {
        int zs = (int)(iz - radius);
        for (int ix = 0; ix < nx; ix++) {
            int xs = (int)(ix - radius);
            if (xs * xs + zs * zs <= r2) {
                for (int iy = 0; iy < ny; iy++)
                    cyl.data[nnz++] = cb.data[((size_t)iz * ny + iy) * nx + ix];
                cyl.cord[2 * nr] = ix;
                cyl.cord[2 * nr + 1] = iz;
                nr++;
            }
        }
    }
    return (nnz != cyl.nnz || nr != cyl.nrays) ? -2 : 0;
}

void arecgb_arecImageFree(arecImage *im) {
    if (im->is_cyl) {
        free(im->cord);
        im->cord = NULL;
    }
    free(im->data);
    im->data = NULL;
}

// reset / soft_noneg (arecImage.cpp:796-826).
void arecgb_reset(arecImage *im) {
    size_t n = im->is_cyl ? (size_t)im->nnz : (size_t)im->nx * im->ny * im->nz;
    memset(im->data, 0, sizeof(float) * n);
}

void arecgb_soft_noneg(arecImage *im) {
    size_t n = im->is_cyl ? (size_t)im->nnz : (size_t)im->nx * im->ny * im->nz;
    for (size_t i = 0; i < n; i++)
        if (im->data[i] < 0.0f) im->data[i] *= 0.5f;
}

int arecgb_arecProject2D(arecImage c, float *a, int n, arecImage *p) {
    return compat_project(ARECGB_LIN, c, a, n, p);
}
int arecgb_arecProject2D_KB(arecImage c, float *a, int n, arecImage *p) {
    return compat_project(ARECGB_KB, c, a, n, p);
}
int arecgb_arecProject2D_SQ(arecImage c, float *a, int n, arecImage *p) {
    return compat_project(ARECGB_SQ, c, a, n, p);
}
int arecgb_arecBackProject2D(arecImage i, float *a, int n, arecImage *v) {
    return compat_backproject(ARECGB_LIN, i, a, n, v);
}
int arecgb_arecBackProject2D_KB(arecImage i, float *a, int n, arecImage *v) {
    return compat_backproject(ARECGB_KB, i, a, n, v);
}
int arecgb_arecBackProject2D_SQ(arecImage i, float *a, int n, arecImage *v) {
    return compat_backproject(ARECGB_SQ, i, a, n, v);
}

int arecgb_cyl_sirt(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                    float tol) {
    return compat_solve(false, ARECGB_LIN, im, a, x, lam, maxit, tol);
}
int arecgb_cyl_sirt_KB(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                       float tol) {
    return compat_solve(false, ARECGB_KB, im, a, x, lam, maxit, tol);
}
int arecgb_cyl_sirt_SQ(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                       float tol) {
    return compat_solve(false, ARECGB_SQ, im, a, x, lam, maxit, tol);
}
int arecgb_cyl_cgls(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                    float tol) {
    return compat_solve(true, ARECGB_LIN, im, a, x, lam, maxit, tol);
}
int arecgb_cyl_cgls_KB(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                       float tol) {
    return compat_solve(true, ARECGB_KB, im, a, x, lam, maxit, tol);
}
int arecgb_cyl_cgls_SQ(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                       float tol) {
    return compat_solve(true, ARECGB_SQ, im, a, x, lam, maxit, tol);
}
int arecgb_cyl_cgls_stat(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                         float tol) {
    return compat_solve(true, ARECGB_LIN, im, a, x, lam, maxit, tol, true);
}
int arecgb_cyl_cgls_KB_stat(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                            float tol) {
    return compat_solve(true, ARECGB_KB, im, a, x, lam, maxit, tol, true);
}
int arecgb_cyl_cgls_SQ_stat(MPI_Comm, arecImage im, float *a, arecImage *x, float lam, int maxit,
                            float tol) {
    return compat_solve(true, ARECGB_SQ, im, a, x, lam, maxit, tol, true);
}

// init_weights (areccgls_stat.cpp:12-46): w = expf(-p) times the Tukey window
// along x, in a newly allocated cube image.
int arecgb_init_weights(MPI_Comm, arecImage pr, arecImage *weights) {
    const int nx = pr.nx;
    if (arecgb_arecAllocateCBImage(weights, pr.nx, pr.ny, pr.nz) != 0) return 1;
    std::vector<double> hx(nx);
    const double alpha = 0.5, pi = std::atan(1.0) * 4.0, A = 2.0 * pi / alpha;
    const double xa = 0.5 * alpha * (nx - 1), xb = (1.0 - 0.5 * alpha) * (nx - 1);
    for (int x = 0; x < nx; x++) {
        const double va = 0.5 * (1.0 + std::cos(A * (1.0 * x / (nx - 1) - alpha / 2)));
        const double vb = 0.5 * (1.0 + std::cos(A * (1.0 * x / (nx - 1) - 1.0 + alpha / 2)));
        hx[x] = x < xa ? va : (x > xb ? vb : 1.0);
    }
    const size_t n = (size_t)pr.nx * pr.ny * pr.nz;
    for (size_t i = 0; i < n; i++)
        weights->data[i] = (float)((double)expf(-pr.data[i]) * hx[i % nx]);
    if (!quiet()) {
        float mn = 1e6f, mx = -1e6f;
        for (size_t i = 0; i < n; i++) {
            mn = std::min(mn, weights->data[i]);
            mx = std::max(mx, weights->data[i]);
        }
        printf("Statweight min: %f max: %f \n", mn, mx);
    }
    return 0;
}

// arecCCImages (AREC3D/AREC3D/arecImage.cpp:384-434): shifts of each image of
// images2 against the same-index image of images1.
int arecgb_arecCCImages(MPI_Comm, arecImage i1, arecImage i2, float *sx, float *sy) {
    if (i1.nx != i2.nx || i1.ny != i2.ny || i1.nz != i2.nz) {
        if (!quiet()) fprintf(stderr, "arecCCImages: mismatch in dimension:\n");
        return -1;
    }
    const int nx = i1.nx, ny = i1.ny, nz = i1.nz;
    if (nz <= 0) return 0;
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t n = (size_t)nx * ny * nz;
    float *d1 = nullptr, *d2 = nullptr, *dsx = nullptr;
    cudaStream_t st = nullptr;
    int rc = 0;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d1, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&d2, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&dsx, sizeof(float) * 2 * nz);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d1, i1.data, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d2, i2.data, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        set_error(std::string("arecCCImages: ") + cudaGetErrorString(e));
        rc = cuda_status(e);
    }
    if (!rc) rc = cc_shifts(d1, d2, nz, ny, nx, dsx, dsx + nz, nullptr, nullptr, st);
    if (!rc) {
        e = cudaMemcpyAsync(sx, dsx, sizeof(float) * nz, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sy, dsx + nz, sizeof(float) * nz, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(std::string("arecCCImages: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    if (st) cudaStreamSynchronize(st);
    cudaFree(d1);
    cudaFree(d2);
    cudaFree(dsx);
    if (st) cudaStreamDestroy(st);
    return rc;
}

// Rotational alignment over host stacks: copy in, run on the device, copy out.
// kind -1: arecRotCCImages (angles out); 0, 1, 2: arecRotateImages, _skew,
// _skew_safe (images and angles in place).
static int rot_host(const char *who, int kind, const arecImage &a, const arecImage *b, int r2,
                    float *angles, int *n_rot, double *mean_cc) {
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (nz <= 0) return 0;
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t n = (size_t)nx * ny * nz;
    const bool two = b != nullptr;
    float *d1 = nullptr, *d2 = nullptr, *da = nullptr;
    cudaStream_t st = nullptr;
    int rc = 0;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d1, sizeof(float) * n);
    if (e == cudaSuccess && two) e = cudaMalloc(&d2, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&da, sizeof(float) * nz);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d1, a.data, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && two)
        e = cudaMemcpyAsync(d2, b->data, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && kind >= 0)
        e = cudaMemcpyAsync(da, angles, sizeof(float) * nz, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        set_error(std::string(who) + ": " + cudaGetErrorString(e));
        rc = cuda_status(e);
    }
    if (!rc) {
        if (kind < 0)
            rc = rot_cc_angles(d1, d2, nz, ny, nx, r2, da, st);
        else
            rc = rotate_stack(d1, d2, nz, ny, nx, da, kind, n_rot, mean_cc, st);
    }
    if (!rc) {
        e = cudaMemcpyAsync(angles, da, sizeof(float) * nz, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && kind >= 0)
            e = cudaMemcpyAsync(a.data, d1, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(std::string(who) + ": " + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    if (st) cudaStreamSynchronize(st);
    cudaFree(d1);
    cudaFree(d2);
    cudaFree(da);
    if (st) cudaStreamDestroy(st);
    return rc;
}

// arecRotCCImages (AREC3D/AREC3D/arecImage.cpp:555-598): rotation of each image
// of images2 against the same-index image of images1, degrees.
int arecgb_arecRotCCImages(MPI_Comm, arecImage i1, arecImage i2, int r2, float *angles) {
    if (i1.nx != i2.nx || i1.ny != i2.ny || i1.nz != i2.nz) {
        if (!quiet()) fprintf(stderr, "arecRotCCImages2: mismatch in dimension:\n");
        return -1;
    }
    return rot_host("arecRotCCImages", -1, i1, &i2, r2, angles, nullptr, nullptr);
}

// arecRotateImages (AREC3D/AREC3D/arecImage.cpp:674-690): bilinear rotation.
void arecgb_arecRotateImages(arecImage *images, float *angles) {
    if (rot_host("arecRotateImages", 0, *images, nullptr, 0, angles, nullptr, nullptr) &&
        !quiet())
        fprintf(stderr, "arecRotateImages: %s\n", last_error());
}

// arecRotateImages_skew (AREC3D/AREC3D/arecImage.cpp:692-738).
void arecgb_arecRotateImages_skew(arecImage *images, float *angles) {
    if (rot_host("arecRotateImages_skew", 1, *images, nullptr, 0, angles, nullptr, nullptr) &&
        !quiet())
        fprintf(stderr, "arecRotateImages_skew: %s\n", last_error());
}

// arecRotateImages_skew_safe (AREC3D/AREC3D/arecImage.cpp:740-790).
void arecgb_arecRotateImages_skew_safe(arecImage *images, arecImage *images_ref, float *angles) {
    int n_rot = 0;
    double mean_cc = 0.0;
    const int rc = rot_host("arecRotateImages_skew_safe", 2, *images, images_ref, 0, angles,
                            &n_rot, &mean_cc);
    if (quiet()) return;
    if (rc)
        fprintf(stderr, "arecRotateImages_skew_safe: %s\n", last_error());
    else
        printf("arecRotateImages_skew_safe: Mean CC=%4.4f n_rot=%d/%d\n", mean_cc, n_rot,
               images->nz);
}

// Preprocessing over host stacks: copy in, run on the device, copy out.
// kind 0: arecImageTakeLog (n values); 1: periodicDecomposition; 2:
// makePeriodicSlice (smooth part of one image into out).
static int pre_host(const char *who, int kind, float *data, size_t n, int nz, int ny, int nx,
                    float *out) {
    if (n == 0) return 0;
    std::lock_guard<std::mutex> lk(g_mu);
    float *d = nullptr;
    cudaStream_t st = nullptr;
    int rc = 0;
    const size_t nbuf = kind == 2 ? 2 * n : n;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(float) * nbuf);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, data, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        set_error(std::string(who) + ": " + cudaGetErrorString(e));
        rc = cuda_status(e);
    }
    if (!rc) {
        if (kind == 0)
            rc = take_log(d, n, st);
        else
            rc = periodic_decomp(d, nz, ny, nx, kind == 2 ? d + n : nullptr, st);
    }
    if (!rc) {
        e = cudaMemcpyAsync(kind == 2 ? out : data, kind == 2 ? d + n : d, sizeof(float) * n,
                            cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(std::string(who) + ": " + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    if (st) cudaStreamSynchronize(st);
    cudaFree(d);
    if (st) cudaStreamDestroy(st);
    return rc;
}

// arecImageTakeLog (AREC3D/AREC3D/arecImage.cpp:358-381): in place.
void arecgb_arecImageTakeLog(arecImage image) {
    const size_t n = image.is_cyl != 1 ? (size_t)image.nx * image.ny * image.nz : (size_t)image.nnz;
    if (pre_host("arecImageTakeLog", 0, image.data, n, 0, 0, 0, nullptr) && !quiet())
        fprintf(stderr, "arecImageTakeLog: %s\n", last_error());
}

// periodicDecomposition (AREC3D/AREC3D/imagetools.cpp:77-114): in place.
void arecgb_periodicDecomposition(arecImage img) {
    const size_t n = (size_t)img.nx * img.ny * img.nz;
    if (pre_host("periodicDecomposition", 1, img.data, n, img.nz, img.ny, img.nx, nullptr) &&
        !quiet())
        fprintf(stderr, "periodicDecomposition: %s\n", last_error());
}

// makePeriodicSlice (AREC3D/AREC3D/imagetools.cpp:17-75): smooth part of one image.
void arecgb_makePeriodicSlice(int nx, int ny, float *data, float *out) {
    if (pre_host("makePeriodicSlice", 2, data, (size_t)nx * ny, 1, ny, nx, out) && !quiet())
        fprintf(stderr, "makePeriodicSlice: %s\n", last_error());
}

// ccorr2d (AREC3D/AREC3D/align2dstack.cpp:480-521).
// The reference's ccorr2d, fshift2d and speak return nothing; a failure here
// (a rejected size, a CUDA error) leaves the output untouched and is reported
// on stderr, as the other void entry points do, unless ARECGB_QUIET is set.
static void report_void(const char *fn) {
    if (!quiet()) fprintf(stderr, "%s: %s\n", fn, last_error());
}

void arecgb_ccorr2d(int nx, int ny, float *x, float *y, float *c) {
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t n = (size_t)nx * ny;
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * 3 * n) != cudaSuccess) {
        set_error("ccorr2d: device allocation failed");
        report_void("ccorr2d");
        return;
    }
    cudaMemcpy(d, x, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(d + n, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (ccorr_image(d, d + n, d + 2 * n, ny, nx, 0) == 0)
        cudaMemcpy(c, d + 2 * n, sizeof(float) * n, cudaMemcpyDeviceToHost);
    else
        report_void("ccorr2d");
    cudaFree(d);
}

// fshift2d (AREC3D/AREC3D/align2dstack.cpp:566-630) on host buffers.
void arecgb_fshift2d(int nx, int ny, float *in, float *out, float sx, float sy) {
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t n = (size_t)nx * ny;
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * (2 * n + 2)) != cudaSuccess) {
        set_error("fshift2d: device allocation failed");
        report_void("fshift2d");
        return;
    }
    const float s2[2] = {sx, sy};
    cudaMemcpy(d, in, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(d + 2 * n, s2, sizeof(float) * 2, cudaMemcpyHostToDevice);
    if (fshift_stack(d, d + n, 1, ny, nx, d + 2 * n, d + 2 * n + 1, 0) == 0)
        cudaMemcpy(out, d + n, sizeof(float) * n, cudaMemcpyDeviceToHost);
    else
        report_void("fshift2d");
    cudaFree(d);
}

// speak (AREC3D/AREC3D/align2dstack.cpp:1059-1105).
void arecgb_speak(int nx, int ny, float *data, float *xt, float *yt) {
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t n = (size_t)nx * ny;
    float *d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * (n + 2)) != cudaSuccess) {
        set_error("speak: device allocation failed");
        report_void("speak");
        return;
    }
    cudaMemcpy(d, data, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (peak_search(d, 1, ny, nx, d + n, d + n + 1, nullptr, nullptr, 0) == 0) {
        cudaMemcpy(xt, d + n, sizeof(float), cudaMemcpyDeviceToHost);
        cudaMemcpy(yt, d + n + 1, sizeof(float), cudaMemcpyDeviceToHost);
    } else {
        report_void("speak");
    }
    cudaFree(d);
}

int arecgb_last_trace(double *rel, int cap, arecgb_solve_info *info) {
    int n = std::min<int>(cap, (int)g_trace.size());
    if (rel)
        for (int i = 0; i < n; i++) rel[i] = g_trace[i];
    if (info) *info = g_trace_info;
    return n;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The reference's own C++ symbols (same mangled names as its headers declare).
int arecProject2D(arecImage c, float *a, int n, arecImage *p) { return arecgb_arecProject2D(c, a, n, p); }
int arecProject2D_KB(arecImage c, float *a, int n, arecImage *p) { return arecgb_arecProject2D_KB(c, a, n, p); }
int arecProject2D_SQ(arecImage c, float *a, int n, arecImage *p) { return arecgb_arecProject2D_SQ(c, a, n, p); }
int arecBackProject2D(arecImage i, float *a, int n, arecImage *v) { return arecgb_arecBackProject2D(i, a, n, v); }
int arecBackProject2D_KB(arecImage i, float *a, int n, arecImage *v) { return arecgb_arecBackProject2D_KB(i, a, n, v); }
int arecBackProject2D_SQ(arecImage i, float *a, int n, arecImage *v) { return arecgb_arecBackProject2D_SQ(i, a, n, v); }
int cyl_sirt(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_sirt(m, i, a, x, l, it, t); }
int cyl_sirt_KB(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_sirt_KB(m, i, a, x, l, it, t); }
int cyl_sirt_SQ(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_sirt_SQ(m, i, a, x, l, it, t); }
int cyl_cgls(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_cgls(m, i, a, x, l, it, t); }
int cyl_cgls_KB(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_cgls_KB(m, i, a, x, l, it, t); }
int cyl_cgls_SQ(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_cgls_SQ(m, i, a, x, l, it, t); }
int cyl_cgls_stat(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_cgls_stat(m, i, a, x, l, it, t); }
int cyl_cgls_KB_stat(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_cgls_KB_stat(m, i, a, x, l, it, t); }
int cyl_cgls_SQ_stat(MPI_Comm m, arecImage i, float *a, arecImage *x, float l, int it, float t) { return arecgb_cyl_cgls_SQ_stat(m, i, a, x, l, it, t); }
int init_weights(MPI_Comm m, arecImage p, arecImage *w) { return arecgb_init_weights(m, p, w); }
int arecCCImages(MPI_Comm m, arecImage a, arecImage b, float *sx, float *sy) { return arecgb_arecCCImages(m, a, b, sx, sy); }
void ccorr2d(int nx, int ny, float *x, float *y, float *c) { arecgb_ccorr2d(nx, ny, x, y, c); }
void speak(int nx, int ny, float *d, float *xt, float *yt) { arecgb_speak(nx, ny, d, xt, yt); }
void fshift2d(int nx, int ny, float *in, float *out, float sx, float sy) { arecgb_fshift2d(nx, ny, in, out, sx, sy); }
int arecRotCCImages(MPI_Comm m, arecImage a, arecImage b, int r2, float *ang) { return arecgb_arecRotCCImages(m, a, b, r2, ang); }
void arecRotateImages(arecImage *i, float *ang) { arecgb_arecRotateImages(i, ang); }
void arecRotateImages_skew(arecImage *i, float *ang) { arecgb_arecRotateImages_skew(i, ang); }
void arecRotateImages_skew_safe(arecImage *i, arecImage *r, float *ang) { arecgb_arecRotateImages_skew_safe(i, r, ang); }
void arecImageTakeLog(arecImage i) { arecgb_arecImageTakeLog(i); }
void periodicDecomposition(arecImage i) { arecgb_periodicDecomposition(i); }
void makePeriodicSlice(int nx, int ny, float *d, float *o) { arecgb_makePeriodicSlice(nx, ny, d, o); }
