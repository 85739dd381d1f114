/*
 * Type-generic body of the NLM oracle.  Included twice by nlm_oracle.c, once
 * with REAL=float (suffix f32) and once with REAL=double (suffix f64).
 *
 * TEST INFRASTRUCTURE ONLY: the product never links or calls this code.
 *
 * Arithmetic restated from the reference's generic kernels:
 *   3DNLM/main.cu:58-103      squared differences of (reference patch, candidate
 *                             patch), summed over the NS x NS x NS patch
 *   3DNLM/main.cu:108-111     w = exp(-(D / NS^3) / PARAMETER^2); centre offset
 *                             included; num += w * v(candidate centre); Z += w
 *   3DNLM/main.cu:125         out = num / Z
 *   2D NLM/11x11/main.cu:404-422  the same in 2D (patch NS x NS)
 * The reference addresses a padded buffer with halo H = m + n on every side:
 * reference patch origin at padded x + m, candidate origin at padded x + k,
 * k in [0, SS) (3DNLM/main.cu:59); the candidate centre is at padded
 * x + n + k (3DNLM/main.cu:111).  Here o = k - m in [-m, m].
 * The reference's y sliding-window second-slice error (3DNLM/main.cu:140-141)
 * is NOT reproduced: this is the mathematically intended NLM.
 */
#ifndef REAL
#error "define REAL before including nlm_oracle_body.h"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/* Direct form on a padded volume: for every voxel and offset, sum the patch
 * directly, in the reference's loop order (plane, row, column). */
static void FN(core3d_direct)(const REAL* vp, long Xp, long Yp, int X, int Y, int Z,
                             int m, int n, REAL h, REAL* out, REAL* zsum)
{
    const long P = (long)(2 * n + 1) * (2 * n + 1) * (2 * n + 1);
    const long H = m + n;
    const long sxy = Xp * Yp;
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < Z; ++z) {
        for (int y = 0; y < Y; ++y) {
            for (int x = 0; x < X; ++x) {
                REAL num = 0, zs = 0;
                for (int oz = -m; oz <= m; ++oz)
                    for (int oy = -m; oy <= m; ++oy)
                        for (int ox = -m; ox <= m; ++ox) {
                            REAL D = 0;
                            for (int tz = -n; tz <= n; ++tz)
                                for (int ty = -n; ty <= n; ++ty)
                                    for (int tx = -n; tx <= n; ++tx) {
                                        long pa = (z + H + tz) * sxy + (y + H + ty) * Xp + (x + H + tx);
                                        long pb = pa + oz * sxy + oy * Xp + ox;
                                        REAL d = vp[pa] - vp[pb];
                                        D += d * d;
                                    }
                            REAL w = FN(rexp)(-(D / (REAL)P) / (h * h));
                            zs += w;
                            num += w * vp[(z + H + oz) * sxy + (y + H + oy) * Xp + (x + H + ox)];
                        }
                long o = ((long)z * Y + y) * X + x;
                out[o] = num / zs;
                if (zsum) zsum[o] = zs;
            }
        }
    }
}

/* Separable form: per output plane chunk and per offset, the squared-difference
 * field is box-summed along x, then y, then z (ring of 2n+1 planes).  This is
 * the timed CPU baseline; OpenMP over z chunks. */
static void FN(core3d_sep)(const REAL* vp, long Xp, long Yp, int X, int Y, int Z,
                          int m, int n, REAL h, REAL* out, REAL* zsum, int chunk)
{
    const long P = (long)(2 * n + 1) * (2 * n + 1) * (2 * n + 1);
    const long H = m + n;
    const long sxy = Xp * Yp;
    const REAL scale = (REAL)1 / ((REAL)P * h * h);
    const int K = 2 * n + 1;
    const int nchunks = (Z + chunk - 1) / chunk;
#pragma omp parallel
    {
        const long XE = X + 2 * n, YE = Y + 2 * n;
        REAL* d = (REAL*)malloc(sizeof(REAL) * XE * YE);
        REAL* ex = (REAL*)malloc(sizeof(REAL) * X * YE);
        REAL* ring = (REAL*)malloc(sizeof(REAL) * K * X * Y);
        REAL* num = (REAL*)malloc(sizeof(REAL) * chunk * X * Y);
        REAL* zs = (REAL*)malloc(sizeof(REAL) * chunk * X * Y);
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < nchunks; ++c) {
            const int z0 = c * chunk;
            const int z1 = z0 + chunk < Z ? z0 + chunk : Z;
            const int nz = z1 - z0;
            memset(num, 0, sizeof(REAL) * nz * X * Y);
            memset(zs, 0, sizeof(REAL) * nz * X * Y);
            for (int oz = -m; oz <= m; ++oz)
                for (int oy = -m; oy <= m; ++oy)
                    for (int ox = -m; ox <= m; ++ox) {
                        const long off = oz * sxy + oy * Xp + ox;
                        for (int pz = z0 - n; pz < z1 + n; ++pz) {
                            /* squared differences over the plane + patch halo */
                            const REAL* base = vp + (pz + H) * sxy;
                            for (long yy = 0; yy < YE; ++yy) {
                                const REAL* a = base + (yy + m) * Xp + m;
                                const REAL* b = a + off;
                                REAL* dr = d + yy * XE;
                                for (long xx = 0; xx < XE; ++xx) {
                                    REAL t = a[xx] - b[xx];
                                    dr[xx] = t * t;
                                }
                            }
                            /* x box */
                            for (long yy = 0; yy < YE; ++yy) {
                                const REAL* dr = d + yy * XE;
                                REAL* er = ex + yy * X;
                                for (long x = 0; x < X; ++x) {
                                    REAL s = 0;
                                    for (int t = 0; t < K; ++t) s += dr[x + t];
                                    er[x] = s;
                                }
                            }
                            /* y box into the ring slot of this plane */
                            REAL* slot = ring + (long)((pz - z0 + n) % K) * X * Y;
                            for (long y = 0; y < Y; ++y) {
                                REAL* sr = slot + y * X;
                                for (long x = 0; x < X; ++x) sr[x] = 0;
                                for (int t = 0; t < K; ++t) {
                                    const REAL* er = ex + (y + t) * X;
                                    for (long x = 0; x < X; ++x) sr[x] += er[x];
                                }
                            }
                            /* z box once 2n+1 planes are present: output plane pz - n */
                            const int zo = pz - n;
                            if (zo < z0) continue;
                            REAL* nm = num + (long)(zo - z0) * X * Y;
                            REAL* zz = zs + (long)(zo - z0) * X * Y;
                            const REAL* cand = vp + (zo + H + oz) * sxy;
                            for (long y = 0; y < Y; ++y) {
                                const REAL* cr = cand + (y + H + oy) * Xp + H + ox;
                                for (long x = 0; x < X; ++x) {
                                    REAL D = 0;
                                    for (int t = 0; t < K; ++t) D += ring[(long)t * X * Y + y * X + x];
                                    REAL w = FN(rexp)(-D * scale);
                                    zz[y * X + x] += w;
                                    nm[y * X + x] += w * cr[x];
                                }
                            }
                        }
                    }
            for (long i = 0; i < (long)nz * X * Y; ++i) {
                long o = (long)z0 * X * Y + i;
                out[o] = num[i] / zs[i];
                if (zsum) zsum[o] = zs[i];
            }
        }
        free(d); free(ex); free(ring); free(num); free(zs);
    }
}

/* 2D direct form on a padded image (reference 2D NLM/11x11/main.cu:383-422). */
static void FN(core2d_direct)(const REAL* vp, long Xp, int X, int Y, int m, int n, REAL h,
                             REAL* out, REAL* zsum)
{
    const long P = (long)(2 * n + 1) * (2 * n + 1);
    const long H = m + n;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < Y; ++y) {
        for (int x = 0; x < X; ++x) {
            REAL num = 0, zs = 0;
            for (int oy = -m; oy <= m; ++oy)
                for (int ox = -m; ox <= m; ++ox) {
                    REAL D = 0;
                    for (int ty = -n; ty <= n; ++ty)
                        for (int tx = -n; tx <= n; ++tx) {
                            long pa = (y + H + ty) * Xp + (x + H + tx);
                            REAL d = vp[pa] - vp[pa + oy * Xp + ox];
                            D += d * d;
                        }
                    REAL w = FN(rexp)(-(D / (REAL)P) / (h * h));
                    zs += w;
                    num += w * vp[(y + H + oy) * Xp + (x + H + ox)];
                }
            out[(long)y * X + x] = num / zs;
            if (zsum) zsum[(long)y * X + x] = zs;
        }
    }
}

/* 2D separable form (x box then y box), OpenMP over row chunks. */
static void FN(core2d_sep)(const REAL* vp, long Xp, int X, int Y, int m, int n, REAL h,
                          REAL* out, REAL* zsum, int chunk)
{
    const long P = (long)(2 * n + 1) * (2 * n + 1);
    const long H = m + n;
    const REAL scale = (REAL)1 / ((REAL)P * h * h);
    const int K = 2 * n + 1;
    const int nchunks = (Y + chunk - 1) / chunk;
#pragma omp parallel
    {
        const long XE = X + 2 * n;
        REAL* d = (REAL*)malloc(sizeof(REAL) * XE * (chunk + 2 * n));
        REAL* ex = (REAL*)malloc(sizeof(REAL) * X * (chunk + 2 * n));
        REAL* num = (REAL*)malloc(sizeof(REAL) * chunk * X);
        REAL* zs = (REAL*)malloc(sizeof(REAL) * chunk * X);
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < nchunks; ++c) {
            const int y0 = c * chunk;
            const int y1 = y0 + chunk < Y ? y0 + chunk : Y;
            const int ny = y1 - y0;
            memset(num, 0, sizeof(REAL) * ny * X);
            memset(zs, 0, sizeof(REAL) * ny * X);
            for (int oy = -m; oy <= m; ++oy)
                for (int ox = -m; ox <= m; ++ox) {
                    const long off = oy * Xp + ox;
                    for (int r = 0; r < ny + 2 * n; ++r) {
                        const REAL* a = vp + (y0 + r + m) * Xp + m;
                        const REAL* b = a + off;
                        REAL* dr = d + (long)r * XE;
                        for (long xx = 0; xx < XE; ++xx) {
                            REAL t = a[xx] - b[xx];
                            dr[xx] = t * t;
                        }
                        REAL* er = ex + (long)r * X;
                        for (long x = 0; x < X; ++x) {
                            REAL s = 0;
                            for (int t = 0; t < K; ++t) s += dr[x + t];
                            er[x] = s;
                        }
                    }
                    for (int r = 0; r < ny; ++r) {
                        const REAL* cr = vp + (y0 + r + H + oy) * Xp + H + ox;
                        for (long x = 0; x < X; ++x) {
                            REAL D = 0;
                            for (int t = 0; t < K; ++t) D += ex[(long)(r + t) * X + x];
                            REAL w = FN(rexp)(-D * scale);
                            zs[(long)r * X + x] += w;
                            num[(long)r * X + x] += w * cr[x];
                        }
                    }
                }
            for (long i = 0; i < (long)ny * X; ++i) {
                out[(long)y0 * X + i] = num[i] / zs[i];
                if (zsum) zsum[(long)y0 * X + i] = zs[i];
            }
        }
        free(d); free(ex); free(num); free(zs);
    }
}

#undef FN
#undef CAT
#undef CAT_
