// A C++ caller of the library written against the reference's declarations
// (include/arec_compat.h declares the reference's C++ entry points with their
// own names and signatures).  It re-checks, through those entry points, the
// known answers of the reference's Catch suite
// (AREC3D/AREC3D_test/AREC3D_test.cpp): the cylinder tables (:8-70), the cube
// indexing (:72-95), one-voxel projection and back projection (:97-189),
// bitwise A == A^T on unit vectors for the square-pixel and Kaiser-Bessel
// pairs (:191-324) and the cylinder <-> cube round trip (:326-363); then it
// calls one solver of each family under its C++ name.
//
// Built and run by tests/test_gpu_dropin.py (from the repository root):
//   g++ -std=c++14 -I include tests/dropin/catch_cases.cpp
//       -L arec3d_gb300 -larec_gb300 -Wl,-rpath,arec3d_gb300 -o catch_cases
// Exit status 0 and a final "all <n> checks passed" line mean success.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "arec_compat.h"

static int g_checks = 0, g_failed = 0;

#define CHECK(cond)                                                                     \
    do {                                                                                \
        ++g_checks;                                                                     \
        if (!(cond)) {                                                                  \
            ++g_failed;                                                                 \
            fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #cond);    \
        }                                                                               \
    } while (0)

// Catch's Approx: |a - b| <= 100 * FLT_EPSILON * (1 + max(|a|, |b|)).
static bool approx(double a, double b) {
    const double eps = 1.1920928955078125e-07 * 100.0;
    return fabs(a - b) <= eps * (1.0 + fmax(fabs(a), fabs(b)));
}

static int cord_at(const arecImage &c, int i, int ray) { return c.cord[2 * ray + i]; }

static void cylinder_tables() {
    arecImage c;
    memset(&c, 0, sizeof(c));
    arecgb_arecAllocateCylImage(&c, 1.0, 2);
    CHECK(c.nrays == 5 && c.nnz == 10);
    const int odd[5][2] = {{1, 0}, {0, 1}, {1, 1}, {2, 1}, {1, 2}};
    for (int k = 0; k < 5; k++) {
        CHECK(cord_at(c, 0, k) == odd[k][0]);
        CHECK(cord_at(c, 1, k) == odd[k][1]);
    }
    arecgb_arecImageFree(&c);

    arecgb_arecAllocateCylImage(&c, 0.5, 3);
    CHECK(c.nrays == 4 && c.nnz == 12);
    const int even[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
    for (int k = 0; k < 4; k++) {
        CHECK(cord_at(c, 0, k) == even[k][0]);
        CHECK(cord_at(c, 1, k) == even[k][1]);
    }
    arecgb_arecImageFree(&c);
}

static void cube_indexing() {
    arecImage p;
    memset(&p, 0, sizeof(p));
    arecgb_arecAllocateCBImage(&p, 1, 2, 3);
    for (int i = 0; i < 6; i++) p.data[i] = (float)i;
    const int nx = p.nx, ny = p.ny;
    for (int k = 0; k < 3; k++)
        for (int j = 0; j < 2; j++) CHECK(approx(p.data[(k * ny + j) * nx + 0], 2.0 * k + j));
    arecgb_arecImageFree(&p);
}

static void one_voxel_pair() {
    arecImage c, p;
    memset(&c, 0, sizeof(c));
    memset(&p, 0, sizeof(p));
    arecgb_arecAllocateCylImage(&c, 1.0, 2);
    arecgb_arecAllocateCBImage(&p, 3, 2, 1);
    c.data[4] = 1.0f;
    c.data[5] = 2.0f;
    float angle = 0.0f;
    CHECK(arecProject2D_SQ(c, &angle, 1, &p) == 0);
    double sv = 0, sp = 0;
    for (int i = 0; i < c.nnz; i++) sv += c.data[i];
    for (int i = 0; i < 6; i++) sp += p.data[i];
    CHECK(approx(sv, 3.0));
    CHECK(approx(sp, 3.0));
    CHECK(approx(p.data[1], 1.0));
    CHECK(approx(p.data[4], 2.0));

    arecgb_reset(&c);
    arecgb_reset(&p);
    p.data[1] = 1.0f;
    p.data[4] = 2.0f;
    CHECK(arecBackProject2D_SQ(p, &angle, 1, &c) == 0);
    sv = sp = 0;
    for (int i = 0; i < c.nnz; i++) sv += c.data[i];
    for (int i = 0; i < 6; i++) sp += p.data[i];
    CHECK(approx(sv, 9.0));
    CHECK(approx(sp, 3.0));
    arecgb_arecImageFree(&c);
    arecgb_arecImageFree(&p);
}

typedef int (*op_fn)(arecImage, float *, int, arecImage *);

// Coefficient A[b][a] (forward projection of unit voxel a, read at bin b) and
// A^T[a][b] (back projection of unit bin b, read at voxel a) must be equal
// floats for every pair sampled with the given stride.
static void exact_adjoint(op_fn fwd, op_fn bwd, double radius, int ny, const float *ang_in,
                          int na, int step) {
    arecImage c, p;
    memset(&c, 0, sizeof(c));
    memset(&p, 0, sizeof(p));
    arecgb_arecAllocateCylImage(&c, radius, ny);
    arecgb_arecAllocateCBImage(&p, c.nx, ny, na);
    float *ang = (float *)malloc(sizeof(float) * na);
    memcpy(ang, ang_in, sizeof(float) * na);
    const int nv = c.nnz, ns = p.nx * p.ny * p.nz;
    float *A = (float *)calloc((size_t)nv * ns, sizeof(float));
    for (int a = 0; a < nv; a += step) {
        arecgb_reset(&c);
        arecgb_reset(&p);
        c.data[a] = 1.0f;
        CHECK(fwd(c, ang, na, &p) == 0);
        for (int b = 0; b < ns; b += step) A[(size_t)a * ns + b] = p.data[b];
    }
    for (int b = 0; b < ns; b += step) {
        arecgb_reset(&c);
        arecgb_reset(&p);
        p.data[b] = 1.0f;
        CHECK(bwd(p, ang, na, &c) == 0);
        for (int a = 0; a < nv; a += step) CHECK(A[(size_t)a * ns + b] == c.data[a]);
    }
    free(A);
    free(ang);
    arecgb_arecImageFree(&c);
    arecgb_arecImageFree(&p);
}

static void cylinder_cube_round_trip() {
    arecImage c, cb, c2;
    memset(&c, 0, sizeof(c));
    memset(&cb, 0, sizeof(cb));
    memset(&c2, 0, sizeof(c2));
    arecgb_arecAllocateCylImage(&c, 1.0, 2);
    double s_cyl = 0;
    for (int i = 0; i < c.nnz; i++) {
        c.data[i] = (float)i;
        s_cyl += c.data[i];
    }
    arecgb_arecAllocateCBImage(&cb, c.nx, c.ny, c.nz);
    CHECK(arecgb_ImageCyl2CB(c, cb, c.nx, c.ny, c.nz) == 0);
    double s_cube = 0;
    for (int i = 0; i < cb.nx * cb.ny * cb.nz; i++) s_cube += cb.data[i];
    CHECK(s_cube == s_cyl);
    arecgb_arecAllocateCylImage(&c2, 1.0, 2);
    CHECK(arecgb_ImageCB2Cyl(cb, c2, 2, 2, 2, 2) == 0);
    for (int i = 0; i < c.nnz; i++) CHECK(c.data[i] == c2.data[i]);
    arecgb_arecImageFree(&c);
    arecgb_arecImageFree(&cb);
    arecgb_arecImageFree(&c2);
}

// One solver of each family under its C++ name: the library allocates *xvol
// (data == NULL on entry), and the Kaiser-Bessel CGLS refuses an even width
// with the reference's status -1.
static void solvers() {
    const int nx = 33, ny = 2, na = 12;
    arecImage b;
    memset(&b, 0, sizeof(b));
    arecgb_arecAllocateCBImage(&b, nx, ny, na);
    arecImage x;
    memset(&x, 0, sizeof(x));
    arecgb_arecAllocateCylImage(&x, 0.5 * (nx - 1), ny);
    for (int i = 0; i < x.nnz; i++) x.data[i] = (float)((i * 37) % 11) * 0.1f;
    float ang[na];
    for (int i = 0; i < na; i++) ang[i] = (float)(i * 3.14159265358979 / na);
    CHECK(arecProject2D_SQ(x, ang, na, &b) == 0);

    arecImage xs;
    memset(&xs, 0, sizeof(xs));
    CHECK(cyl_sirt_SQ(0, b, ang, &xs, 1e-3f, 5, 0.0f) == 0);
    CHECK(xs.data != NULL && xs.nrays == x.nrays && xs.nnz == x.nnz && xs.is_cyl == 1);
    arecImage xc;
    memset(&xc, 0, sizeof(xc));
    CHECK(cyl_cgls_SQ(0, b, ang, &xc, 0.0f, 30, 1e-4f) == 0);
    CHECK(xc.data != NULL);
    // noise-free data from x: CGLS must bring the data misfit well below |b|
    arecImage q;
    memset(&q, 0, sizeof(q));
    arecgb_arecAllocateCBImage(&q, nx, ny, na);
    CHECK(arecProject2D_SQ(xc, ang, na, &q) == 0);
    double r = 0, bn = 0;
    for (int i = 0; i < nx * ny * na; i++) {
        r += (double)(q.data[i] - b.data[i]) * (q.data[i] - b.data[i]);
        bn += (double)b.data[i] * b.data[i];
    }
    CHECK(sqrt(r / bn) < 1e-2);

    arecImage b_even;
    memset(&b_even, 0, sizeof(b_even));
    arecgb_arecAllocateCBImage(&b_even, 32, ny, na);
    arecImage xk;
    memset(&xk, 0, sizeof(xk));
    CHECK(cyl_cgls_KB(0, b_even, ang, &xk, 0.0f, 3, 1e-4f) == -1);
    if (xk.data) arecgb_arecImageFree(&xk);
    arecgb_arecImageFree(&b_even);
    arecgb_arecImageFree(&q);
    arecgb_arecImageFree(&xs);
    arecgb_arecImageFree(&xc);
    arecgb_arecImageFree(&x);
    arecgb_arecImageFree(&b);
}

int main() {
    cylinder_tables();
    cube_indexing();
    one_voxel_pair();
    {
        const float ang[3] = {1.475f, 21.123f, 2.123f};
        exact_adjoint(arecProject2D_SQ, arecBackProject2D_SQ, 1.0, 2, ang, 3, 1);
    }
    {
        const float ang[2] = {0.698132f, 1.22173f};
        exact_adjoint(arecProject2D_SQ, arecBackProject2D_SQ, 1.5, 2, ang, 2, 3);
        exact_adjoint(arecProject2D_KB, arecBackProject2D_KB, 0.5, 2, ang, 2, 3);
    }
    cylinder_cube_round_trip();
    solvers();
    if (g_failed) {
        printf("%d of %d checks failed\n", g_failed, g_checks);
        return 1;
    }
    printf("all %d checks passed\n", g_checks);
    return 0;
}
