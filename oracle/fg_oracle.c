/*
 * CPU oracle for the generalised geodesic distance raster scan.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C with OpenMP, the
 * CPU path of masadcv/FastGeodis 1.0.5 so that the CUDA product can be
 * checked against it and so that a CPU baseline can be timed on hosts where
 * the reference sources are not available.  Nothing in the shipped package
 * links or calls it.
 *
 * Parity is pinned: tests/golden/ holds input/output vectors produced by the
 * reference's own CPU build (oracle/build_oracle.py:build_reference), and the
 * CPU test-suite checks this restatement against them bit for bit.
 *
 * What is restated (reference file:line, paths inside the reference project):
 *   - per-row sweep, 3-neighbour stencil, cost
 *       D[t][x] = min(D[t][x], min_k D[t-1][x+k] + l_eucl*ld[k] + l_grad*L1)
 *     FastGeodis/fastgeodis_cpu.cpp:53-162 (geodesic_updown_pass_cpu)
 *   - 2D pass order per iteration: rows down/up, then columns (the reference
 *     transposes and re-runs the row pass)  fastgeodis_cpu.cpp:164-201
 *   - per-plane sweep, 9-neighbour stencil, ld[3i+j] = sqrt(s0 + |i-1| s1 +
 *     |j-1| s2) on squared spacings        fastgeodis_cpu.cpp:203-340
 *   - 3D pass order and spacing permutations {s0,s1,s2}, {s1,s0,s2},
 *     {s2,s1,s0}                              fastgeodis_cpu.cpp:342-407
 *   - L1 channel distance                    fastgeodis_cpu.cpp:38-41
 *   - initial distance v * mask (all mask channels, channel 0 swept)
 *                                             fastgeodis_cpu.cpp:173-174
 *   - signed transform D(M) - D(1-M)         FastGeodis/fastgeodis.cpp:241-258
 *   - GSF composition                        FastGeodis/fastgeodis.cpp:319-343
 *   - Toivanen's sequential raster scan (2D and 3D, plain / signed / GSF)
 *                                             FastGeodis/geodis_toivanen.cpp:35-348,
 *                                             FastGeodis/fastgeodis.cpp:260-277, 345-369
 *
 * The transposes of the reference are replaced by index arithmetic: the
 * value computed for every cell is the same expression on the same operands,
 * so the results are identical; only the memory walk differs.
 *
 * Floating point: every operation is rounded separately, in the reference's
 * order ((D + l_eucl*ld) + l_grad*L1), and the minimum keeps the current
 * value unless the candidate is strictly smaller (std::min).  Build with
 * -ffp-contract=off (oracle/build_oracle.py does).  A double-precision copy
 * of the same scan is provided for error reporting.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FGO_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* float32 scan, exact reference arithmetic                            */
/* ------------------------------------------------------------------ */

/* One forward+backward pair along an axis whose cross-section is one
 * dimension (2D images).  Step t lives at offset t*sstr, cross index x at
 * x*xstr; channels are cstr apart.  fastgeodis_cpu.cpp:53-162. */
static void pair1_f32(const float *img, int C, int64_t cstr, float *D, int L,
                      int64_t sstr, int N, int64_t xstr, float lg, float le,
                      int nthreads)
{
    const float ld[3] = {(float)sqrt(2.0), 1.0f, (float)sqrt(2.0)};
    for (int dir = 0; dir < 2; dir++) {
        int t0 = dir == 0 ? 1 : L - 2, dt = dir == 0 ? 1 : -1;
        for (int t = t0; t >= 0 && t < L; t += dt) {
            int tp = t - dt;
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (int x = 0; x < N; x++) {
                float nd = D[t * sstr + x * xstr];
                for (int k = 0; k < 3; k++) {
                    int xi = x + k - 1;
                    if (xi < 0 || xi >= N)
                        continue;
                    float l1 = 0.0f;
                    if (C == 1) {
                        l1 = fabsf(img[t * sstr + x * xstr] - img[tp * sstr + xi * xstr]);
                    } else {
                        for (int c = 0; c < C; c++)
                            l1 += fabsf(img[c * cstr + t * sstr + x * xstr] -
                                        img[c * cstr + tp * sstr + xi * xstr]);
                    }
                    float cur = D[tp * sstr + xi * xstr] + le * ld[k] + lg * l1;
                    nd = cur < nd ? cur : nd;
                }
                D[t * sstr + x * xstr] = nd;
            }
        }
    }
}

/* Step-length table of one 3D pass, fastgeodis_cpu.cpp:220-231: sp[] are
 * squared spacings already permuted for the swept axis; index 3*i+j with i
 * the offset along cross axis A and j along cross axis B. */
static void table3(const float sp[3], float ld[9])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            float v = sp[0];
            v += (float)abs(i - 1) * sp[1];
            v += (float)abs(j - 1) * sp[2];
            ld[i * 3 + j] = sqrtf(v);
        }
}

/* One forward+backward pair along an axis whose cross-section has two
 * dimensions: A (extent NA, stride astr) and B (extent NB, stride bstr).
 * fastgeodis_cpu.cpp:203-340 after the reference's transposes. */
static void pair2_f32(const float *img, int C, int64_t cstr, float *D, int L,
                      int64_t sstr, int NA, int64_t astr, int NB, int64_t bstr,
                      const float ld[9], float lg, float le, int nthreads)
{
    for (int dir = 0; dir < 2; dir++) {
        int t0 = dir == 0 ? 1 : L - 2, dt = dir == 0 ? 1 : -1;
        for (int t = t0; t >= 0 && t < L; t += dt) {
            int tp = t - dt;
#pragma omp parallel for collapse(2) num_threads(nthreads) schedule(static)
            for (int a = 0; a < NA; a++) {
                for (int b = 0; b < NB; b++) {
                    int64_t here = t * sstr + a * astr + b * bstr;
                    float nd = D[here];
                    for (int i = 0; i < 3; i++) {
                        for (int j = 0; j < 3; j++) {
                            int ai = a + i - 1, bj = b + j - 1;
                            if (bj < 0 || bj >= NB || ai < 0 || ai >= NA)
                                continue;
                            int64_t prev = tp * sstr + ai * astr + bj * bstr;
                            float l1 = 0.0f;
                            if (C == 1) {
                                l1 = fabsf(img[here] - img[prev]);
                            } else {
                                for (int c = 0; c < C; c++)
                                    l1 += fabsf(img[c * cstr + here] - img[c * cstr + prev]);
                            }
                            float cur = D[prev] + le * ld[i * 3 + j] + lg * l1;
                            nd = cur < nd ? cur : nd;
                        }
                    }
                    D[here] = nd;
                }
            }
        }
    }
}

/* out[Cm][H][W] = v * mask, then channel 0 swept.  fastgeodis_cpu.cpp:164-201 */
FGO_API void fgo_geodesic2d(const float *img, int C, int H, int W,
                            const float *mask, int Cm, float *out, float v,
                            float lg, float le, int iters, int nthreads)
{
    int64_t P = (int64_t)H * W;
    for (int64_t i = 0; i < (int64_t)Cm * P; i++)
        out[i] = v * mask[i];
    for (int it = 0; it < iters; it++) {
        pair1_f32(img, C, P, out, H, W, W, 1, lg, le, nthreads);  /* along H */
        pair1_f32(img, C, P, out, W, 1, H, W, lg, le, nthreads);  /* along W */
    }
}

/* fastgeodis_cpu.cpp:342-407 */
FGO_API void fgo_geodesic3d(const float *img, int C, int Dd, int H, int W,
                            const float *mask, int Cm, const float *spacing,
                            float *out, float v, float lg, float le, int iters,
                            int nthreads)
{
    int64_t P = (int64_t)Dd * H * W, HW = (int64_t)H * W;
    float s[3] = {spacing[0] * spacing[0], spacing[1] * spacing[1], spacing[2] * spacing[2]};
    float ldD[9], ldH[9], ldW[9];
    float spD[3] = {s[0], s[1], s[2]}, spH[3] = {s[1], s[0], s[2]}, spW[3] = {s[2], s[1], s[0]};
    table3(spD, ldD);
    table3(spH, ldH);
    table3(spW, ldW);
    for (int64_t i = 0; i < (int64_t)Cm * P; i++)
        out[i] = v * mask[i];
    for (int it = 0; it < iters; it++) {
        /* along D: A = H, B = W */
        pair2_f32(img, C, P, out, Dd, HW, H, W, W, 1, ldD, lg, le, nthreads);
        /* along H: the reference's tensor is [H, D, W]: A = D, B = W */
        pair2_f32(img, C, P, out, H, W, Dd, HW, W, 1, ldH, lg, le, nthreads);
        /* along W: the reference's tensor is [W, H, D]: A = H, B = D */
        pair2_f32(img, C, P, out, W, 1, H, W, Dd, HW, ldW, lg, le, nthreads);
    }
}

/* fastgeodis.cpp:241-249: D(M) - D(1-M), elementwise in float. */
FGO_API void fgo_signed2d(const float *img, int C, int H, int W, const float *mask,
                          int Cm, float *out, float v, float lg, float le,
                          int iters, int nthreads)
{
    int64_t n = (int64_t)Cm * H * W;
    float *inv = (float *)malloc(n * sizeof(float));
    float *db = (float *)malloc(n * sizeof(float));
    for (int64_t i = 0; i < n; i++)
        inv[i] = 1.0f - mask[i];
    fgo_geodesic2d(img, C, H, W, mask, Cm, out, v, lg, le, iters, nthreads);
    fgo_geodesic2d(img, C, H, W, inv, Cm, db, v, lg, le, iters, nthreads);
    for (int64_t i = 0; i < n; i++)
        out[i] = out[i] - db[i];
    free(inv);
    free(db);
}

FGO_API void fgo_signed3d(const float *img, int C, int Dd, int H, int W,
                          const float *mask, int Cm, const float *spacing,
                          float *out, float v, float lg, float le, int iters,
                          int nthreads)
{
    int64_t n = (int64_t)Cm * Dd * H * W;
    float *inv = (float *)malloc(n * sizeof(float));
    float *db = (float *)malloc(n * sizeof(float));
    for (int64_t i = 0; i < n; i++)
        inv[i] = 1.0f - mask[i];
    fgo_geodesic3d(img, C, Dd, H, W, mask, Cm, spacing, out, v, lg, le, iters, nthreads);
    fgo_geodesic3d(img, C, Dd, H, W, inv, Cm, spacing, db, v, lg, le, iters, nthreads);
    for (int64_t i = 0; i < n; i++)
        out[i] = out[i] - db[i];
    free(inv);
    free(db);
}

/* fastgeodis.cpp:319-330.  lambda arrives as float; 1 - lambda is computed
 * in float as the reference does. */
static void gsf_common(int is3d, const float *img, int C, int Dd, int H, int W,
                       const float *mask, int Cm, const float *spacing,
                       float theta, float *out, float v, float lambda, int iters,
                       int nthreads)
{
    int64_t n = (int64_t)Cm * Dd * H * W;
    float le = 1.0f - lambda;
    float *ds = (float *)malloc(n * sizeof(float));
    float *a = (float *)malloc(n * sizeof(float));
    float *s1 = (float *)malloc(n * sizeof(float));
    float *s2 = (float *)malloc(n * sizeof(float));
#define FGO_SIGNED(m, o)                                                             \
    do {                                                                             \
        if (is3d)                                                                    \
            fgo_signed3d(img, C, Dd, H, W, m, Cm, spacing, o, v, lambda, le, iters,  \
                         nthreads);                                                  \
        else                                                                         \
            fgo_signed2d(img, C, H, W, m, Cm, o, v, lambda, le, iters, nthreads);    \
    } while (0)
    FGO_SIGNED(mask, ds);
    /* Md = (Ds > theta); signed(1 - Md) */
    for (int64_t i = 0; i < n; i++)
        a[i] = 1.0f - (ds[i] > theta ? 1.0f : 0.0f);
    FGO_SIGNED(a, s1);
    /* Me = (Ds > -theta); signed(Me) */
    for (int64_t i = 0; i < n; i++)
        a[i] = ds[i] > -theta ? 1.0f : 0.0f;
    FGO_SIGNED(a, s2);
#undef FGO_SIGNED
    for (int64_t i = 0; i < n; i++)
        out[i] = -s1[i] + s2[i];
    free(ds);
    free(a);
    free(s1);
    free(s2);
}

FGO_API void fgo_gsf2d(const float *img, int C, int H, int W, const float *mask,
                       int Cm, float theta, float *out, float v, float lambda,
                       int iters, int nthreads)
{
    gsf_common(0, img, C, 1, H, W, mask, Cm, NULL, theta, out, v, lambda, iters, nthreads);
}

FGO_API void fgo_gsf3d(const float *img, int C, int Dd, int H, int W,
                       const float *mask, int Cm, float theta,
                       const float *spacing, float *out, float v, float lambda,
                       int iters, int nthreads)
{
    gsf_common(1, img, C, Dd, H, W, mask, Cm, spacing, theta, out, v, lambda, iters, nthreads);
}

/* ------------------------------------------------------------------ */
/* Toivanen's raster scan, float32, exact reference arithmetic         */
/* ------------------------------------------------------------------ */
/*
 * FastGeodis/geodis_toivanen.cpp: L1 distance :35-38; 2D forward/backward
 * pair :40-146 and driver :148-164; 3D pair :166-329 and driver :331-348.
 * A forward pass visits every cell in memory order (depth, rows, columns)
 * and replaces it by the minimum of itself and the candidates of its causal
 * neighbours, which already hold this pass's values where they come earlier
 * in the order (the 3D set also reads four cells of the next plane, which
 * still hold the previous pass's values); the backward pass runs in reverse
 * order with the mirrored set.  The reference runs it on one thread; so
 * does this restatement.
 */
static float toiv_l1(const float *img, int C, int64_t cstr, int64_t a, int64_t b)
{
    if (C == 1)
        return fabsf(img[a] - img[b]);
    float s = 0.0f;
    for (int c = 0; c < C; c++)
        s += fabsf(img[c * cstr + a] - img[c * cstr + b]);
    return s;
}

static void toiv_pass(const float *img, int C, int Dd, int H, int W, float *D, int n,
                      const int *dz, const int *dh, const int *dw, const float *ld,
                      int backward, float lg, float le)
{
    int64_t P = (int64_t)Dd * H * W, HW = (int64_t)H * W;
    for (int64_t k = 0; k < P; k++) {
        int64_t i = backward ? P - 1 - k : k;
        int z = (int)(i / HW), h = (int)((i / W) % H), w = (int)(i % W);
        float nd = D[i];
        for (int j = 0; j < n; j++) {
            int zi = z + dz[j], hi = h + dh[j], wi = w + dw[j];
            if (zi < 0 || zi >= Dd || hi < 0 || hi >= H || wi < 0 || wi >= W)
                continue;
            int64_t q = ((int64_t)zi * H + hi) * W + wi;
            float cur = D[q] + le * ld[j] + lg * toiv_l1(img, C, P, i, q);
            if (cur < nd) /* std::min(new_dist, cur_dist) */
                nd = cur;
        }
        D[i] = nd;
    }
}

/* geodis_toivanen.cpp:56-57, 101-102 */
static const int T2_DZ[4] = {0, 0, 0, 0};
static const int T2F_DH[4] = {-1, -1, -1, 0}, T2F_DW[4] = {-1, 0, 1, -1};
static const int T2B_DH[4] = {0, 1, 1, 1}, T2B_DW[4] = {1, -1, 0, 1};
/* geodis_toivanen.cpp:182-184, 209-211 */
static const int T3F_DZ[13] = {-1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1};
static const int T3F_DH[13] = {-1, -1, -1, 0, 0, -1, -1, -1, 0, -1, -1, -1, 0};
static const int T3F_DW[13] = {-1, 0, 1, -1, 0, -1, 0, 1, -1, -1, 0, 1, -1};
static const int T3B_DZ[13] = {-1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 1};
static const int T3B_DH[13] = {0, 1, 1, 1, 0, 1, 1, 1, 0, 0, 1, 1, 1};
static const int T3B_DW[13] = {1, -1, 0, 1, 1, -1, 0, 1, 0, 1, -1, 0, 1};

FGO_API void fgo_toivanen2d(const float *img, int C, int H, int W, const float *mask,
                            int Cm, float *out, float v, float lg, float le, int iters)
{
    int64_t P = (int64_t)H * W;
    const float r2 = sqrtf(2.0f);
    const float ldf[4] = {r2, 1.0f, r2, 1.0f}, ldb[4] = {1.0f, r2, 1.0f, r2};
    for (int64_t i = 0; i < (int64_t)Cm * P; i++)
        out[i] = v * mask[i];
    for (int it = 0; it < iters; it++) {
        toiv_pass(img, C, 1, H, W, out, 4, T2_DZ, T2F_DH, T2F_DW, ldf, 0, lg, le);
        toiv_pass(img, C, 1, H, W, out, 4, T2_DZ, T2B_DH, T2B_DW, ldb, 1, lg, le);
    }
}

/* geodis_toivanen.cpp:186-207, 213-234: sqrt of the summed squared spacings
 * of the axes a neighbour moves along, summed in axis order */
static void toiv_table(const float *sp, const int *dz, const int *dh, const int *dw, float *ld)
{
    for (int i = 0; i < 13; i++) {
        float v = 0.0f;
        if (dz[i] != 0) v += sp[0] * sp[0];
        if (dh[i] != 0) v += sp[1] * sp[1];
        if (dw[i] != 0) v += sp[2] * sp[2];
        ld[i] = sqrtf(v);
    }
}

FGO_API void fgo_toivanen3d(const float *img, int C, int Dd, int H, int W,
                            const float *mask, int Cm, const float *spacing,
                            float *out, float v, float lg, float le, int iters)
{
    int64_t P = (int64_t)Dd * H * W;
    float ldf[13], ldb[13];
    toiv_table(spacing, T3F_DZ, T3F_DH, T3F_DW, ldf);
    toiv_table(spacing, T3B_DZ, T3B_DH, T3B_DW, ldb);
    for (int64_t i = 0; i < (int64_t)Cm * P; i++)
        out[i] = v * mask[i];
    for (int it = 0; it < iters; it++) {
        toiv_pass(img, C, Dd, H, W, out, 13, T3F_DZ, T3F_DH, T3F_DW, ldf, 0, lg, le);
        toiv_pass(img, C, Dd, H, W, out, 13, T3B_DZ, T3B_DH, T3B_DW, ldb, 1, lg, le);
    }
}

/* Signed and GSF compositions of the Toivanen transform: FastGeodis/fastgeodis.cpp
 * :260-277 (D(M) - D(1-M)) and :345-369 (GSF), the same as the raster ones. */
static void toiv_signed(int is3d, const float *img, int C, int Dd, int H, int W,
                        const float *mask, int Cm, const float *spacing, float *out,
                        float v, float lg, float le, int iters)
{
    int64_t n = (int64_t)Cm * Dd * H * W;
    float *inv = (float *)malloc(n * sizeof(float));
    float *db = (float *)malloc(n * sizeof(float));
    for (int64_t i = 0; i < n; i++)
        inv[i] = 1.0f - mask[i];
    if (is3d) {
        fgo_toivanen3d(img, C, Dd, H, W, mask, Cm, spacing, out, v, lg, le, iters);
        fgo_toivanen3d(img, C, Dd, H, W, inv, Cm, spacing, db, v, lg, le, iters);
    } else {
        fgo_toivanen2d(img, C, H, W, mask, Cm, out, v, lg, le, iters);
        fgo_toivanen2d(img, C, H, W, inv, Cm, db, v, lg, le, iters);
    }
    for (int64_t i = 0; i < n; i++)
        out[i] = out[i] - db[i];
    free(inv);
    free(db);
}

FGO_API void fgo_signed_toivanen2d(const float *img, int C, int H, int W, const float *mask,
                                   int Cm, float *out, float v, float lg, float le, int iters)
{
    toiv_signed(0, img, C, 1, H, W, mask, Cm, NULL, out, v, lg, le, iters);
}

FGO_API void fgo_signed_toivanen3d(const float *img, int C, int Dd, int H, int W,
                                   const float *mask, int Cm, const float *spacing,
                                   float *out, float v, float lg, float le, int iters)
{
    toiv_signed(1, img, C, Dd, H, W, mask, Cm, spacing, out, v, lg, le, iters);
}

static void toiv_gsf(int is3d, const float *img, int C, int Dd, int H, int W,
                     const float *mask, int Cm, const float *spacing, float theta,
                     float *out, float v, float lambda, int iters)
{
    int64_t n = (int64_t)Cm * Dd * H * W;
    float le = 1.0f - lambda;
    float *ds = (float *)malloc(n * sizeof(float));
    float *a = (float *)malloc(n * sizeof(float));
    float *s1 = (float *)malloc(n * sizeof(float));
    float *s2 = (float *)malloc(n * sizeof(float));
    toiv_signed(is3d, img, C, Dd, H, W, mask, Cm, spacing, ds, v, lambda, le, iters);
    for (int64_t i = 0; i < n; i++)
        a[i] = 1.0f - (ds[i] > theta ? 1.0f : 0.0f);
    toiv_signed(is3d, img, C, Dd, H, W, a, Cm, spacing, s1, v, lambda, le, iters);
    for (int64_t i = 0; i < n; i++)
        a[i] = ds[i] > -theta ? 1.0f : 0.0f;
    toiv_signed(is3d, img, C, Dd, H, W, a, Cm, spacing, s2, v, lambda, le, iters);
    for (int64_t i = 0; i < n; i++)
        out[i] = -s1[i] + s2[i];
    free(ds);
    free(a);
    free(s1);
    free(s2);
}

FGO_API void fgo_gsf_toivanen2d(const float *img, int C, int H, int W, const float *mask,
                                int Cm, float theta, float *out, float v, float lambda, int iters)
{
    toiv_gsf(0, img, C, 1, H, W, mask, Cm, NULL, theta, out, v, lambda, iters);
}

FGO_API void fgo_gsf_toivanen3d(const float *img, int C, int Dd, int H, int W,
                                const float *mask, int Cm, float theta, const float *spacing,
                                float *out, float v, float lambda, int iters)
{
    toiv_gsf(1, img, C, Dd, H, W, mask, Cm, spacing, theta, out, v, lambda, iters);
}

/* ------------------------------------------------------------------ */
/* float64 copy of the same scan (error reporting only)                */
/* ------------------------------------------------------------------ */

static void pair1_f64(const double *img, int C, int64_t cstr, double *D, int L,
                      int64_t sstr, int N, int64_t xstr, double lg, double le,
                      int nthreads)
{
    const double ld[3] = {sqrt(2.0), 1.0, sqrt(2.0)};
    for (int dir = 0; dir < 2; dir++) {
        int t0 = dir == 0 ? 1 : L - 2, dt = dir == 0 ? 1 : -1;
        for (int t = t0; t >= 0 && t < L; t += dt) {
            int tp = t - dt;
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (int x = 0; x < N; x++) {
                double nd = D[t * sstr + x * xstr];
                for (int k = 0; k < 3; k++) {
                    int xi = x + k - 1;
                    if (xi < 0 || xi >= N)
                        continue;
                    double l1 = 0.0;
                    for (int c = 0; c < C; c++)
                        l1 += fabs(img[c * cstr + t * sstr + x * xstr] -
                                   img[c * cstr + tp * sstr + xi * xstr]);
                    double cur = D[tp * sstr + xi * xstr] + le * ld[k] + lg * l1;
                    nd = cur < nd ? cur : nd;
                }
                D[t * sstr + x * xstr] = nd;
            }
        }
    }
}

static void pair2_f64(const double *img, int C, int64_t cstr, double *D, int L,
                      int64_t sstr, int NA, int64_t astr, int NB, int64_t bstr,
                      const double ld[9], double lg, double le, int nthreads)
{
    for (int dir = 0; dir < 2; dir++) {
        int t0 = dir == 0 ? 1 : L - 2, dt = dir == 0 ? 1 : -1;
        for (int t = t0; t >= 0 && t < L; t += dt) {
            int tp = t - dt;
#pragma omp parallel for collapse(2) num_threads(nthreads) schedule(static)
            for (int a = 0; a < NA; a++) {
                for (int b = 0; b < NB; b++) {
                    int64_t here = t * sstr + a * astr + b * bstr;
                    double nd = D[here];
                    for (int i = 0; i < 3; i++) {
                        for (int j = 0; j < 3; j++) {
                            int ai = a + i - 1, bj = b + j - 1;
                            if (bj < 0 || bj >= NB || ai < 0 || ai >= NA)
                                continue;
                            int64_t prev = tp * sstr + ai * astr + bj * bstr;
                            double l1 = 0.0;
                            for (int c = 0; c < C; c++)
                                l1 += fabs(img[c * cstr + here] - img[c * cstr + prev]);
                            double cur = D[prev] + le * ld[i * 3 + j] + lg * l1;
                            nd = cur < nd ? cur : nd;
                        }
                    }
                    D[here] = nd;
                }
            }
        }
    }
}

FGO_API void fgo_geodesic2d_f64(const double *img, int C, int H, int W,
                                const double *mask, int Cm, double *out, double v,
                                double lg, double le, int iters, int nthreads)
{
    int64_t P = (int64_t)H * W;
    for (int64_t i = 0; i < (int64_t)Cm * P; i++)
        out[i] = v * mask[i];
    for (int it = 0; it < iters; it++) {
        pair1_f64(img, C, P, out, H, W, W, 1, lg, le, nthreads);
        pair1_f64(img, C, P, out, W, 1, H, W, lg, le, nthreads);
    }
}

FGO_API void fgo_geodesic3d_f64(const double *img, int C, int Dd, int H, int W,
                                const double *mask, int Cm, const double *spacing,
                                double *out, double v, double lg, double le,
                                int iters, int nthreads)
{
    int64_t P = (int64_t)Dd * H * W, HW = (int64_t)H * W;
    double s[3] = {spacing[0] * spacing[0], spacing[1] * spacing[1], spacing[2] * spacing[2]};
    double perm[3][3] = {{s[0], s[1], s[2]}, {s[1], s[0], s[2]}, {s[2], s[1], s[0]}};
    double ld[3][9];
    for (int a = 0; a < 3; a++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                ld[a][i * 3 + j] = sqrt(perm[a][0] + abs(i - 1) * perm[a][1] + abs(j - 1) * perm[a][2]);
    for (int64_t i = 0; i < (int64_t)Cm * P; i++)
        out[i] = v * mask[i];
    for (int it = 0; it < iters; it++) {
        pair2_f64(img, C, P, out, Dd, HW, H, W, W, 1, ld[0], lg, le, nthreads);
        pair2_f64(img, C, P, out, H, W, Dd, HW, W, 1, ld[1], lg, le, nthreads);
        pair2_f64(img, C, P, out, W, 1, H, W, Dd, HW, ld[2], lg, le, nthreads);
    }
}

FGO_API int fgo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
