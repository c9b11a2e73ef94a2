// Geometry plans: cylinder support, ray/row/column tables and per-angle
// constants, built on the host and uploaded once per (weighting, radius,
// slices, angles).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>

#include "arec_internal.cuh"

namespace arecgb {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error() { return g_last_error.c_str(); }

static std::atomic<long long> g_launches{0};
void count_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int cuda_status(cudaError_t e) {
    if (e == cudaErrorMemoryAllocation) return ARECGB_ERR_NOMEM;
    return ARECGB_ERR_CUDA_BASE - (int)e;
}

// Cylinder support of arecAllocateCylImage (AREC3D/AREC3D/arecImage.cpp:29-86):
// nx = round(2r+1); pixel (ix, iz) is inside when (int)(ix-r)^2 + (int)(iz-r)^2
// <= (int)(r*r), the int conversions truncating toward zero.  Rays are listed
// iz-major, ix-minor.
static int cyl_nx(double radius) { return (int)std::round(2 * radius + 1); }

static void cyl_scan(double radius, std::vector<int> &cord) {
    int nx = cyl_nx(radius);
    int r2 = (int)(radius * radius);
    cord.clear();
    for (int iz = 0; iz < nx; iz++) {
        int zs = (int)(iz - radius);
        int zz = zs * zs;
        for (int ix = 0; ix < nx; ix++) {
            int xs = (int)(ix - radius);
            if (zz + xs * xs <= r2) {
                cord.push_back(ix);
                cord.push_back(iz);
            }
        }
    }
}

static void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

size_t vol_floats(const Plan *p) { return (size_t)p->nrays * p->ys; }
size_t sin_floats(const Plan *p) { return (size_t)p->na * p->nx * p->ys; }

static int choose_vec(int ys) {
    if (ys >= 256) return 8;
    if (ys >= 128) return 4;
    if (ys >= 64) return 2;
    return 1;
}

int plan_create(Plan **out, int weighting, double radius, int ny, int nangles,
                const float *angles_host, bool tables) {
    *out = nullptr;
    if (weighting < ARECGB_LIN || weighting > ARECGB_SQ) {
        set_error("plan_create: weighting must be 1 (LIN), 2 (KB) or 3 (SQ)");
        return ARECGB_ERR_ARG;
    }
    if (!(radius >= 0.0) || radius > 8192.0 || ny < 1 || nangles < 1 || !angles_host) {
        set_error("plan_create: need 0 <= radius <= 8192, ny >= 1, nangles >= 1, angles");
        return ARECGB_ERR_ARG;
    }
    Plan *p = new Plan();
    p->weighting = weighting;
    p->radius = radius;
    p->nx = cyl_nx(radius);
    p->ny = ny;
    p->ys = (ny + 7) & ~7;
    p->na = nangles;
    p->angles.assign(angles_host, angles_host + nangles);
    p->vec = choose_vec(p->ys);
    cudaGetDevice(&p->device);

    std::vector<int> cord;
    cyl_scan(radius, cord);
    p->nrays = (int)(cord.size() / 2);
    if (p->nrays < 1) {
        delete p;
        set_error("plan_create: empty cylinder");
        return ARECGB_ERR_ARG;
    }
    const int nx = p->nx, nr = p->nrays;

    // Ray offsets from the centre as float pairs.
    std::vector<float4> ray(nr);
    if (weighting == ARECGB_LIN) {
        // pmethod=1 reads ray k's coordinates at cord[2k+3], cord[2k+4] through
        // the 2-argument cord macro with a 1-based ray loop (arecproject.cpp:75-78,
        // arecImage.h:20), i.e. (iz of ray k+1, ix of ray k+2), about the integer
        // centre (int)radius + 1.  The last two rays read past the table; those
        // entries are taken as zero.
        int xcent = (int)radius + 1;
        auto at = [&](size_t j) { return j < cord.size() ? cord[j] : 0; };
        for (int k = 0; k < nr; k++) {
            ray[k] = make_float4((float)(at(2 * (size_t)k + 3) - xcent),
                                 (float)(at(2 * (size_t)k + 4) - xcent), 0.f, 0.f);
        }
        p->r_hi = (float)xcent;
        p->r_lo = 0.f;
    } else {
        for (int k = 0; k < nr; k++) {
            float xh, xl, zh, zl;
            split(cord[2 * k] - radius, xh, xl);
            split(cord[2 * k + 1] - radius, zh, zl);
            ray[k] = make_float4(xh, zh, xl, zl);
        }
        split(radius, p->r_hi, p->r_lo);
    }

    // Row and column extents (rows are contiguous in ix, columns in iz).
    std::vector<RowInfo> rows(nx);
    std::vector<ColInfo> cols(nx);
    for (int i = 0; i < nx; i++) {
        rows[i] = RowInfo{0, nx, -1, 0};
        cols[i] = ColInfo{nx, -1, 0, 0};
    }
    for (int k = nr - 1; k >= 0; k--) {
        int ix = cord[2 * k], iz = cord[2 * k + 1];
        rows[iz].start = k;
        rows[iz].lo = std::min(rows[iz].lo, ix);
        rows[iz].hi = std::max(rows[iz].hi, ix);
        cols[ix].lo = std::min(cols[ix].lo, iz);
        cols[ix].hi = std::max(cols[ix].hi, iz);
    }
    // column-major ray order (the forward projector's column sweeps read
    // consecutive pixels of a column as consecutive rays of a gathered copy)
    std::vector<int> kinv(nr);
    {
        int cs = 0;
        for (int ix = 0; ix < nx; ix++) {
            cols[ix].start = cs;
            if (cols[ix].hi >= cols[ix].lo) cs += cols[ix].hi - cols[ix].lo + 1;
        }
        for (int k = 0; k < nr; k++) {
            const int ix = cord[2 * k], iz = cord[2 * k + 1];
            kinv[cols[ix].start + iz - cols[ix].lo] = k;
        }
    }

    // Per-angle constants.  The reference evaluates the ray position with
    // cos(angles[ia]) on a float, which C++ resolves to the float overload
    // (arecproject.cpp:599-600): cosf/sinf here give the same exact floats.
    // The square-pixel footprint takes the angle as a double (sqpoints,
    // arecproject.h:11-22).
    std::vector<AngleParams> ang(nangles);
    for (int a = 0; a < nangles; a++) {
        float phi = angles_host[a];
        AngleParams &q = ang[a];
        memset(&q, 0, sizeof(q));
        q.c = std::cos(phi);  // float overload
        q.s = std::sin(phi);
        double cd = std::cos((double)phi), sd = std::sin((double)phi);
        double cms = std::fabs(0.5 * (cd - sd)), cps = std::fabs(0.5 * (cd + sd));
        double a_ = (cps < cms) ? cps : cms;
        double b_ = ((cms < cps) ? cps : cms) + 1e-6;
        double ymax = 1 / (((b_ - a_) + 2 * a_));
        q.sq_a = (float)a_;
        q.sq_b = (float)b_;
        q.sq_aeps = (float)(a_ + 1e-3);
        q.sq_ymax = (float)ymax;
        q.sq_c2 = (float)(0.5 * ymax * (b_ + a_));
        q.sq_k1 = (float)(0.5 * ymax / (b_ - a_));
        q.orient = std::fabs(q.c) >= std::fabs(q.s) ? 0 : 1;
    }

    // Forward-projection angle groups: runs of consecutive angles sharing a
    // sweep orientation, at most kGroupAngles each, whose strips stay within a
    // few pixels of each other on every line of the disk (so the union of their
    // candidate pixels per line fits the kernel's 32-pixel stage).
    std::vector<int4> groups;
    const double Rg = radius + 2.0;
    for (int a = 0; a < nangles;) {
        int o = ang[a].orient, n = 1;
        while (a + n < nangles && n < kGroupAngles && ang[a + n].orient == o) {
            const double spread = Rg * (std::fabs((double)ang[a + n].c - ang[a].c) +
                                        std::fabs((double)ang[a + n].s - ang[a].s));
            if (spread / 0.7071 > 10.0) break;
            n++;
        }
        groups.push_back(make_int4(a, n, o, 0));
        a += n;
    }
    // orientation 0 first (band launches take one orientation at a time)
    std::stable_sort(groups.begin(), groups.end(),
                     [](const int4 &a, const int4 &b) { return a.z < b.z; });
    p->ngroups = (int)groups.size();
    p->ngroups_o[0] = (int)std::count_if(groups.begin(), groups.end(),
                                         [](const int4 &g) { return g.z == 0; });
    p->ngroups_o[1] = p->ngroups - p->ngroups_o[0];

    // Back-projection tiles of kTileX x kTileZ pixels holding at least one ray.
    std::vector<int2> tiles;
    for (int iz0 = 0; iz0 < nx; iz0 += kTileZ)
        for (int ix0 = 0; ix0 < nx; ix0 += kTileX) {
            bool any = false;
            for (int iz = iz0; iz < std::min(nx, iz0 + kTileZ) && !any; iz++)
                any = rows[iz].lo <= std::min(nx - 1, ix0 + kTileX - 1) && rows[iz].hi >= ix0 &&
                      rows[iz].hi >= rows[iz].lo;
            if (any) tiles.push_back(make_int2(ix0, iz0));
        }
    p->ntiles = (int)tiles.size();

    // Upload.
    cudaError_t e = cudaSuccess;
    e = cudaMalloc(&p->d_groups, sizeof(int4) * groups.size());
    if (e == cudaSuccess) e = cudaMalloc(&p->d_tiles, sizeof(int2) * tiles.size());
    if (e == cudaSuccess) e = cudaMalloc(&p->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->d_err, 0, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_groups, groups.data(), sizeof(int4) * groups.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_tiles, tiles.data(), sizeof(int2) * tiles.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_ray, sizeof(float4) * nr);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_ang, sizeof(AngleParams) * nangles);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_rows, sizeof(RowInfo) * nx);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_cols, sizeof(ColInfo) * nx);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_kinv, sizeof(int) * std::max(nr, 1));
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_ray, ray.data(), sizeof(float4) * nr, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_ang, ang.data(), sizeof(AngleParams) * nangles,
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_rows, rows.data(), sizeof(RowInfo) * nx, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_cols, cols.data(), sizeof(ColInfo) * nx, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nr)
        e = cudaMemcpy(p->d_kinv, kinv.data(), sizeof(int) * nr, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        // room for the back projector's grid with one slice chunk per block
        // at half the vector width (the autotuner may choose it):
        // ntiles x ceil(ys / (32 max(1, vec / 2))) blocks
        const int hv = std::max(1, p->vec / 2);
        const int bp_max = p->ntiles * ((p->ys + 32 * hv - 1) / (32 * hv));
        p->n_partials = std::max(std::max(fp_grid_blocks(p), bp_grid_blocks(p)), bp_max);
        e = cudaMalloc(&p->d_partials, sizeof(double) * (size_t)p->n_partials);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_error(std::string("plan_create: ") + cudaGetErrorString(e));
        plan_destroy(p);
        return cuda_status(e);
    }
    if (int rc = tables ? plan_build_tables(p) : 0) {
        plan_destroy(p);
        return rc;
    }
    *out = p;
    return ARECGB_OK;
}

void plan_destroy(Plan *p) {
    if (!p) return;
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != p->device) cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    cudaFree(p->d_ray);
    cudaFree(p->d_ang);
    cudaFree(p->d_rows);
    cudaFree(p->d_cols);
    for (cudaEvent_t e : p->ev_fp) cudaEventDestroy(e);
    for (cudaEvent_t e : p->ev_bp) cudaEventDestroy(e);
    cudaFree(p->d_w);
    cudaFree(p->d_groups);
    cudaFree(p->d_tiles);
    cudaFree(p->d_ramp);
    cudaFree(p->d_taps);
    cudaFree(p->d_kinv);
    cudaFree(p->d_lin_off);
    cudaFree(p->d_lin_list);
    cudaFree(p->d_xT);
    cudaFree(p->d_bpw);
    cudaFree(p->d_bpf);
    cudaFree(p->d_err);
    cudaFree(p->d_partials);
    for (auto &v : p->d_vol) cudaFree(v);
    for (auto &v : p->d_sin) cudaFree(v);
    cudaFree(p->d_stage);
    for (auto &v : p->d_img) cudaFree(v);
    if (p->h_pinned) cudaFreeHost(p->h_pinned);
    if (p->stream) cudaStreamDestroy(p->stream);
    if (p->solve_stream) cudaStreamSynchronize(p->solve_stream);
    for (cudaStream_t x : p->solve_bs) cudaStreamDestroy(x);
    if (p->solve_stream) cudaStreamDestroy(p->solve_stream);
    for (cudaEvent_t x : p->solve_ev) cudaEventDestroy(x);
    cudaFree(p->d_sred);
    if (p->h_sred) cudaFreeHost(p->h_sred);
    cudaFree(p->d_cstate);
    if (p->h_cstate) cudaFreeHost(p->h_cstate);
    cudaFree(p->d_chist);
    if (cur != p->device) cudaSetDevice(cur);
    delete p;
}

}  // namespace arecgb
