/*
 * NLM oracle: a CPU restatement of the reference's non-local-means arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, the smoke check and the bench's CPU-baseline
 * leg load this library as the checker; the product (the CUDA library behind
 * include/nlm.h) never links, calls or falls back to it.
 *
 * Parity pin: the reference ships no CPU NLM, no tests and no golden outputs.
 * The restatement follows its generic kernels (3DNLM/main.cu:28-238,
 * 2D NLM/11x11/main.cu:383-468); it is pinned against outputs of the
 * reference's own generic CUDA kernels, compiled from the reference sources and
 * run on a GB300, committed under tests/golden/ together with the script that
 * generated them.
 *
 * Forms:
 *   direct     - per voxel, per offset, the patch sum in the reference's loop
 *                order (3DNLM/main.cu:52-111); FP32 or FP64.
 *   separable  - per offset, x box, y box, z ring; FP32 or FP64; OpenMP.  The
 *                FP32 separable form is the timed CPU baseline.
 * Borders: BORDER_REFLECT_101 (gfedcb|abcdefgh|gfedcba), the padding the
 * reference's host driver applies with OpenCV (3DNLM/nlm.cpp:36-41,
 * 2D NLM/11x11/nlm.cpp:15-19), applied here on every axis.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline float rexpf32(float x) { return expf(x); }
static inline double rexpf64(double x) { return exp(x); }

/* Inside the body FN(name) appends the suffix: FN(rexp) is rexpf32 / rexpf64. */
#define REAL float
#define SUFFIX f32
#include "nlm_oracle_body.h"
#undef REAL
#undef SUFFIX

#define REAL double
#define SUFFIX f64
#include "nlm_oracle_body.h"
#undef REAL
#undef SUFFIX

/* OpenCV BORDER_REFLECT_101 index map for any offset (repeated reflection). */
long oracle_reflect101(long i, long n)
{
    if (n <= 1) return 0;
    const long period = 2 * n - 2;
    i %= period;
    if (i < 0) i += period;
    return i < n ? i : period - i;
}

#define DEFINE_PAD(T, name)                                                                  \
    static T* name(const T* v, int X, int Y, int Z, int H, long* Xp, long* Yp)               \
    {                                                                                        \
        long xp = X + 2L * H, yp = Y + 2L * H, zp = Z + 2L * H;                              \
        T* out = (T*)malloc(sizeof(T) * xp * yp * zp);                                       \
        for (long z = 0; z < zp; ++z) {                                                      \
            long sz = oracle_reflect101(z - H, Z);                                           \
            for (long y = 0; y < yp; ++y) {                                                  \
                long sy = oracle_reflect101(y - H, Y);                                       \
                const T* row = v + (sz * Y + sy) * X;                                        \
                T* dst = out + (z * yp + y) * xp;                                            \
                for (long x = 0; x < xp; ++x) dst[x] = row[oracle_reflect101(x - H, X)];     \
            }                                                                                \
        }                                                                                    \
        *Xp = xp;                                                                            \
        *Yp = yp;                                                                            \
        return out;                                                                          \
    }
DEFINE_PAD(float, pad3_f32)
DEFINE_PAD(double, pad3_f64)

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* form: 0 = direct, 1 = separable.  zsum may be NULL. */
void oracle_nlm3d_f32(const float* v, int X, int Y, int Z, int sr, int pr, float h,
                      float* out, float* zsum, int form)
{
    long Xp, Yp;
    float* vp = pad3_f32(v, X, Y, Z, sr + pr, &Xp, &Yp);
    if (form == 0)
        core3d_directf32(vp, Xp, Yp, X, Y, Z, sr, pr, h, out, zsum);
    else
        core3d_sepf32(vp, Xp, Yp, X, Y, Z, sr, pr, h, out, zsum, 4);
    free(vp);
}

void oracle_nlm3d_f64(const double* v, int X, int Y, int Z, int sr, int pr, double h,
                      double* out, double* zsum, int form)
{
    long Xp, Yp;
    double* vp = pad3_f64(v, X, Y, Z, sr + pr, &Xp, &Yp);
    if (form == 0)
        core3d_directf64(vp, Xp, Yp, X, Y, Z, sr, pr, h, out, zsum);
    else
        core3d_sepf64(vp, Xp, Yp, X, Y, Z, sr, pr, h, out, zsum, 4);
    free(vp);
}

void oracle_nlm2d_f32(const float* v, int X, int Y, int sr, int pr, float h, float* out,
                      float* zsum, int form)
{
    long Xp, Yp;
    float* vp = pad3_f32(v, X, Y, 1, sr + pr, &Xp, &Yp);
    /* the 3D pad also padded z; plane H of the padded volume is the image */
    const float* plane = vp + (long)(sr + pr) * Xp * Yp;
    if (form == 0)
        core2d_directf32(plane, Xp, X, Y, sr, pr, h, out, zsum);
    else
        core2d_sepf32(plane, Xp, X, Y, sr, pr, h, out, zsum, 16);
    free(vp);
}

void oracle_nlm2d_f64(const double* v, int X, int Y, int sr, int pr, double h, double* out,
                      double* zsum, int form)
{
    long Xp, Yp;
    double* vp = pad3_f64(v, X, Y, 1, sr + pr, &Xp, &Yp);
    const double* plane = vp + (long)(sr + pr) * Xp * Yp;
    if (form == 0)
        core2d_directf64(plane, Xp, X, Y, sr, pr, h, out, zsum);
    else
        core2d_sepf64(plane, Xp, X, Y, sr, pr, h, out, zsum, 16);
    free(vp);
}

/*
 * Direct form restricted to the box [x0, x0+nx) x [y0, y0+ny) x [z0, z0+nz) of a
 * full volume (borders still reflected at the full volume's edges).  Lets tests
 * spot-check full-size outputs at any location in seconds.  out is nz*ny*nx.
 */
#define DEFINE_REGION(T, SUF, EXPF)                                                            \
    void oracle_nlm3d_region_##SUF(const T* v, int X, int Y, int Z, int sr, int pr, T h,      \
                                   int x0, int y0, int z0, int nx, int ny, int nz, T* out)    \
    {                                                                                          \
        const int m = sr, n = pr;                                                              \
        const long P = (long)(2 * n + 1) * (2 * n + 1) * (2 * n + 1);                           \
        _Pragma("omp parallel for schedule(dynamic, 1)")                                       \
        for (int k = 0; k < nz; ++k)                                                           \
            for (int j = 0; j < ny; ++j)                                                       \
                for (int i = 0; i < nx; ++i) {                                                 \
                    const int x = x0 + i, y = y0 + j, z = z0 + k;                              \
                    T num = 0, zs = 0;                                                         \
                    for (int oz = -m; oz <= m; ++oz)                                           \
                        for (int oy = -m; oy <= m; ++oy)                                       \
                            for (int ox = -m; ox <= m; ++ox) {                                 \
                                T D = 0;                                                       \
                                for (int tz = -n; tz <= n; ++tz)                               \
                                    for (int ty = -n; ty <= n; ++ty)                           \
                                        for (int tx = -n; tx <= n; ++tx) {                     \
                                            T a = v[(oracle_reflect101(z + tz, Z) * Y +         \
                                                     oracle_reflect101(y + ty, Y)) * (long)X +  \
                                                    oracle_reflect101(x + tx, X)];              \
                                            T b = v[(oracle_reflect101(z + oz + tz, Z) * Y +    \
                                                     oracle_reflect101(y + oy + ty, Y)) *       \
                                                        (long)X +                               \
                                                    oracle_reflect101(x + ox + tx, X)];         \
                                            T d = a - b;                                       \
                                            D += d * d;                                        \
                                        }                                                      \
                                T w = EXPF(-(D / (T)P) / (h * h));                             \
                                zs += w;                                                       \
                                num += w * v[(oracle_reflect101(z + oz, Z) * Y +                \
                                              oracle_reflect101(y + oy, Y)) * (long)X +         \
                                             oracle_reflect101(x + ox, X)];                     \
                            }                                                                  \
                    out[((long)k * ny + j) * nx + i] = num / zs;                               \
                }                                                                              \
    }
DEFINE_REGION(float, f32, expf)
DEFINE_REGION(double, f64, exp)

/*
 * Separable form on many boxes of one full volume, each nx x ny x nz with its origin
 * (x, y, z) at origins[3 b .. 3 b + 2]; out holds the boxes one after another.  Each
 * box plus its halo H = sr + pr is gathered from the volume through the REFLECT_101
 * map and the separable core runs on that padded block: an output depends only on
 * inputs within H of it, so the box equals the full-volume separable result.  The
 * per-(voxel, offset) cost is O(patch width) instead of the direct form's O(patch
 * volume), which makes FP64 checks of patch-17^3 outputs affordable.  OpenMP over
 * boxes (the core runs single-threaded inside).
 */
#define DEFINE_BLOCKS_SEP(T, SUF)                                                              \
    void oracle_nlm3d_blocks_sep_##SUF(const T* v, int X, int Y, int Z, int sr, int pr, T h,  \
                                       int nblk, const int* origins, int nx, int ny, int nz,  \
                                       T* out)                                                \
    {                                                                                          \
        const long H = sr + pr;                                                                \
        const long xp = nx + 2 * H, yp = ny + 2 * H, zp = nz + 2 * H;                          \
        _Pragma("omp parallel for schedule(dynamic, 1)")                                       \
        for (int b = 0; b < nblk; ++b) {                                                       \
            const long x0 = origins[3 * b], y0 = origins[3 * b + 1], z0 = origins[3 * b + 2];  \
            T* blk = (T*)malloc(sizeof(T) * xp * yp * zp);                                     \
            for (long zz = 0; zz < zp; ++zz) {                                                 \
                const long sz = oracle_reflect101(z0 + zz - H, Z);                             \
                for (long yy = 0; yy < yp; ++yy) {                                             \
                    const long sy = oracle_reflect101(y0 + yy - H, Y);                         \
                    const T* row = v + (sz * Y + sy) * (long)X;                                \
                    T* dst = blk + (zz * yp + yy) * xp;                                        \
                    for (long xx = 0; xx < xp; ++xx)                                           \
                        dst[xx] = row[oracle_reflect101(x0 + xx - H, X)];                      \
                }                                                                              \
            }                                                                                  \
            core3d_sep##SUF(blk, xp, yp, nx, ny, nz, sr, pr, h,                                \
                            out + (long)b * nx * ny * nz, NULL, nz);                           \
            free(blk);                                                                         \
        }                                                                                      \
    }
DEFINE_BLOCKS_SEP(float, f32)
DEFINE_BLOCKS_SEP(double, f64)

/*
 * Legacy layout (3DNLM/main.h:6, 3DNLM/main.cu:7607-7680): the input is already
 * padded by the caller, unsigned char [Z+SS+NS-2][Y+SS+NS-2][X+SS+NS-2];
 * output float [Z][Y][X]; h on the 0..255 scale (PARAMETER).
 */
void oracle_nlm3d_padded_u8(const unsigned char* in, int X, int Y, int Z, int SS, int NS,
                            float h, float* out, int form)
{
    const int m = (SS - 1) / 2, n = (NS - 1) / 2;
    const long Xp = X + SS + NS - 2, Yp = Y + SS + NS - 2, Zp = Z + SS + NS - 2;
    float* vp = (float*)malloc(sizeof(float) * Xp * Yp * Zp);
    for (long i = 0; i < Xp * Yp * Zp; ++i) vp[i] = (float)in[i];
    if (form == 0)
        core3d_directf32(vp, Xp, Yp, X, Y, Z, m, n, h, out, NULL);
    else
        core3d_sepf32(vp, Xp, Yp, X, Y, Z, m, n, h, out, NULL, 4);
    free(vp);
}

/* Legacy 2D layout (2D NLM/11x11/main.h:6): padded uchar [Y+sr+nb-2][X+sr+nb-2]. */
void oracle_nlm2d_padded_u8(const unsigned char* in, int X, int Y, int sr_size, int nb_size,
                            float h, float* out, int form)
{
    const int m = (sr_size - 1) / 2, n = (nb_size - 1) / 2;
    const long Xp = X + sr_size + nb_size - 2, Yp = Y + sr_size + nb_size - 2;
    float* vp = (float*)malloc(sizeof(float) * Xp * Yp);
    for (long i = 0; i < Xp * Yp; ++i) vp[i] = (float)in[i];
    if (form == 0)
        core2d_directf32(vp, Xp, X, Y, m, n, h, out, NULL);
    else
        core2d_sepf32(vp, Xp, X, Y, m, n, h, out, NULL, 16);
    free(vp);
}

/*
 * FP64 adjoint of the 3D forward (no counterpart in the reference), direct form.
 * With D_p(o) = sum_t (v[p+t] - v[p+o+t])^2, w = exp(-D/(P h^2)),
 * Z_p = sum_o w, out_p = sum_o w v[p+o] / Z_p and upstream gradient g:
 *   a_p(o)   = -g_p (v[p+o] - out_p) w / (Z_p P h^2)          (dL/dD_p(o))
 *   dL/dv    : g_p w / Z_p at p+o; +2 a diff at p+t; -2 a diff at p+o+t
 *   dL/dh    = sum_p sum_o g_p (v[p+o] - out_p) w 2 D / (Z_p P h^3)
 * Gradients on padded (reflected) voxels are folded back onto their sources.
 * Accumulation is per thread then reduced in thread order (deterministic for a
 * fixed thread count).
 */
void oracle_nlm3d_adjoint_f64(const double* v, int X, int Y, int Z, int sr, int pr, double h,
                              const double* g, double* gin, double* gh, double* out_opt)
{
    const int m = sr, n = pr;
    const long H = m + n;
    long Xp, Yp;
    double* vp = pad3_f64(v, X, Y, Z, (int)H, &Xp, &Yp);
    const long Zp = Z + 2 * H;
    const long sxy = Xp * Yp;
    const long NP = sxy * Zp;
    const double P = (double)(2 * n + 1) * (2 * n + 1) * (2 * n + 1);
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    double* gpad_all = (double*)calloc((size_t)nt * NP, sizeof(double));
    double* gh_t = (double*)calloc((size_t)nt, sizeof(double));
    const int S1 = 2 * m + 1;
    const int S = S1 * S1 * S1;
#pragma omp parallel
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* gpad = gpad_all + (size_t)tid * NP;
        double* Dv = (double*)malloc(sizeof(double) * S);
        double* wv = (double*)malloc(sizeof(double) * S);
        double ghl = 0;
#pragma omp for schedule(static)
        for (int z = 0; z < Z; ++z)
            for (int y = 0; y < Y; ++y)
                for (int x = 0; x < X; ++x) {
                    const long p = (z + H) * sxy + (y + H) * Xp + (x + H);
                    double Zs = 0, num = 0;
                    int k = 0;
                    for (int oz = -m; oz <= m; ++oz)
                        for (int oy = -m; oy <= m; ++oy)
                            for (int ox = -m; ox <= m; ++ox, ++k) {
                                const long q = p + oz * sxy + oy * Xp + ox;
                                double D = 0;
                                for (int tz = -n; tz <= n; ++tz)
                                    for (int ty = -n; ty <= n; ++ty)
                                        for (int tx = -n; tx <= n; ++tx) {
                                            const long t = tz * sxy + ty * Xp + tx;
                                            double d = vp[p + t] - vp[q + t];
                                            D += d * d;
                                        }
                                Dv[k] = D;
                                wv[k] = exp(-D / (P * h * h));
                                Zs += wv[k];
                                num += wv[k] * vp[q];
                            }
                    const double outp = num / Zs;
                    const long oidx = ((long)z * Y + y) * X + x;
                    if (out_opt) out_opt[oidx] = outp;
                    const double gp = g[oidx];
                    k = 0;
                    for (int oz = -m; oz <= m; ++oz)
                        for (int oy = -m; oy <= m; ++oy)
                            for (int ox = -m; ox <= m; ++ox, ++k) {
                                const long q = p + oz * sxy + oy * Xp + ox;
                                const double dv = vp[q] - outp;
                                gpad[q] += gp * wv[k] / Zs;
                                const double a = -gp * dv * wv[k] / (Zs * P * h * h);
                                ghl += gp * dv * wv[k] * 2.0 * Dv[k] / (Zs * P * h * h * h);
                                for (int tz = -n; tz <= n; ++tz)
                                    for (int ty = -n; ty <= n; ++ty)
                                        for (int tx = -n; tx <= n; ++tx) {
                                            const long t = tz * sxy + ty * Xp + tx;
                                            const double d = vp[p + t] - vp[q + t];
                                            gpad[p + t] += 2.0 * a * d;
                                            gpad[q + t] -= 2.0 * a * d;
                                        }
                            }
                }
        gh_t[tid] = ghl;
        free(Dv);
        free(wv);
    }
    memset(gin, 0, sizeof(double) * (size_t)X * Y * Z);
    double ghs = 0;
    for (int t = 0; t < nt; ++t) {
        const double* gpad = gpad_all + (size_t)t * NP;
        for (long zz = 0; zz < Zp; ++zz) {
            long sz = oracle_reflect101(zz - H, Z);
            for (long yy = 0; yy < Yp; ++yy) {
                long sy = oracle_reflect101(yy - H, Y);
                for (long xx = 0; xx < Xp; ++xx) {
                    long sx = oracle_reflect101(xx - H, X);
                    gin[(sz * Y + sy) * X + sx] += gpad[zz * sxy + yy * Xp + xx];
                }
            }
        }
        ghs += gh_t[t];
    }
    *gh = ghs;
    free(gpad_all);
    free(gh_t);
    free(vp);
}

/*
 * FP64 central finite differences of L(v) = sum_p g_p out_p(v) with respect to n
 * chosen voxels (test infrastructure for the adjoint; no counterpart in the
 * reference).  For voxel i at idx[3 i .. 3 i + 2] = (x, y, z):
 *   fd[i] = (L(v + eps e_i) - L(v - eps e_i)) / (2 eps),
 * where only the outputs within H = sr + pr of the voxel on every axis change (the
 * REFLECT_101 images of a voxel within H of a face fall inside that box), so L is
 * summed over that box with the direct form.  OpenMP over voxels; each thread
 * perturbs a private copy of the volume.
 */
static double fd_box_loss(const double* v, int X, int Y, int Z, int m, int n, double h,
                          const double* g, int bx0, int by0, int bz0, int bx1, int by1, int bz1)
{
    const double P = (double)(2 * n + 1) * (2 * n + 1) * (2 * n + 1);
    double L = 0;
    for (int z = bz0; z <= bz1; ++z)
        for (int y = by0; y <= by1; ++y)
            for (int x = bx0; x <= bx1; ++x) {
                double num = 0, zs = 0;
                for (int oz = -m; oz <= m; ++oz)
                    for (int oy = -m; oy <= m; ++oy)
                        for (int ox = -m; ox <= m; ++ox) {
                            double D = 0;
                            for (int tz = -n; tz <= n; ++tz)
                                for (int ty = -n; ty <= n; ++ty)
                                    for (int tx = -n; tx <= n; ++tx) {
                                        const double a =
                                            v[(oracle_reflect101(z + tz, Z) * Y +
                                               oracle_reflect101(y + ty, Y)) * (long)X +
                                              oracle_reflect101(x + tx, X)];
                                        const double b =
                                            v[(oracle_reflect101(z + oz + tz, Z) * Y +
                                               oracle_reflect101(y + oy + ty, Y)) * (long)X +
                                              oracle_reflect101(x + ox + tx, X)];
                                        D += (a - b) * (a - b);
                                    }
                            const double w = exp(-(D / P) / (h * h));
                            zs += w;
                            num += w * v[(oracle_reflect101(z + oz, Z) * Y +
                                          oracle_reflect101(y + oy, Y)) * (long)X +
                                         oracle_reflect101(x + ox, X)];
                        }
                L += g[((long)z * Y + y) * X + x] * (num / zs);
            }
    return L;
}

void oracle_nlm3d_fd_grad_f64(const double* v, int X, int Y, int Z, int sr, int pr, double h,
                              const double* g, int nvox, const int* idx, double eps,
                              double* fd)
{
    const int H = sr + pr;
    const size_t N = (size_t)X * Y * Z;
#pragma omp parallel
    {
        double* w = (double*)malloc(sizeof(double) * N);
        memcpy(w, v, sizeof(double) * N);
#pragma omp for schedule(dynamic, 1)
        for (int i = 0; i < nvox; ++i) {
            const int x = idx[3 * i], y = idx[3 * i + 1], z = idx[3 * i + 2];
            const int bx0 = x - H > 0 ? x - H : 0, bx1 = x + H < X - 1 ? x + H : X - 1;
            const int by0 = y - H > 0 ? y - H : 0, by1 = y + H < Y - 1 ? y + H : Y - 1;
            const int bz0 = z - H > 0 ? z - H : 0, bz1 = z + H < Z - 1 ? z + H : Z - 1;
            const long k = ((long)z * Y + y) * X + x;
            w[k] = v[k] + eps;
            const double Lp = fd_box_loss(w, X, Y, Z, sr, pr, h, g, bx0, by0, bz0, bx1, by1, bz1);
            w[k] = v[k] - eps;
            const double Lm = fd_box_loss(w, X, Y, Z, sr, pr, h, g, bx0, by0, bz0, bx1, by1, bz1);
            w[k] = v[k];
            fd[i] = (Lp - Lm) / (2 * eps);
        }
        free(w);
    }
}
