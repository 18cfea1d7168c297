/*
 * Oracle (test infrastructure, not the product): an FP64 C restatement of
 * mripy's Gaussian-gridding loops, used only as the checker in tests/, by
 * __graft_entry__.smoke() and as the timed CPU baseline in bench.py.
 *
 * Each function follows one numba loop of the reference, fft/nufft_func.py:
 *   orc_spread{1,2,3}d   build_grid_1d1_fast  :306-325
 *                        build_grid_2d1_fast  :550-582
 *                        build_grid_3d1_fast  :863-911 (array form :931-937)
 *   orc_interp{1,2,3}d   build_grid_1d2_fast  :342-361
 *                        build_grid_2d2_fast  :607-639
 *                        build_grid_3d2_fast  :985-1032 (array form :1034-1038)
 *   orc_normal{1,2,3}d   build_grid_1d21      :364-385
 *                        build_grid_2d21      :642-672
 *                        build_grid_3d21      :1058-1107 (dcf weighting :1094)
 * Layout: coordinates are float64 (M,); sample values are complex128 stored
 * coil-first as (nt, M); grids are complex128 coil-first (nt, nf1[, nf2[, nf3]]).
 * The reference keeps coils last and loops over them with numba.prange
 * (nufft_func.py:935); the coil-first layout gives each OpenMP thread a
 * contiguous grid of its own, which is the same parallel structure.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#include <complex.h>

typedef double _Complex cplx;

static const double TWO_PI = 2.0 * 3.14159265358979323846;
static const double PI_D = 3.14159265358979323846;

/* Python float semantics of `a % b` and `a // b` for b > 0
 * (CPython Objects/floatobject.c, float_rem / float_floor_div). */
static double py_mod(double a, double b) {
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0) != (m < 0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}

static double py_floordiv(double a, double b) {
    double m = fmod(a, b);
    double div = (a - m) / b;
    if (m != 0.0) {
        if ((b < 0) != (m < 0)) div -= 1.0;
    }
    double fd;
    if (div != 0.0) {
        fd = floor(div);
        if (div - fd > 0.5) fd += 1.0;
    } else {
        fd = copysign(0.0, a / b);
    }
    return fd;
}

static inline int64_t wrapi(int64_t i, int64_t n) {
    int64_t r = i % n;
    return r < 0 ? r + n : r;
}

/* ------------------------------------------------------------------ 1-D */

void orc_spread1d(const double *x, const cplx *c, int64_t M, int nt, double tau, int ns,
                  int64_t nf1, cplx *ftau) {
    double hx = TWO_PI / nf1;
    double *E3 = (double *)malloc(sizeof(double) * (ns + 1));
    for (int j = 0; j <= ns; j++) E3[j] = exp(-pow(PI_D * j / nf1, 2) / tau);
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *ct = c + (int64_t)t * M;
        cplx *ft = ftau + (int64_t)t * nf1;
        memset(ft, 0, sizeof(cplx) * nf1);
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI);
            int64_t m = 1 + (int64_t)py_floordiv(xi, hx);
            xi = xi - hx * m;
            double E1 = exp(-0.25 * xi * xi / tau);
            double E2 = exp((xi * PI_D) / (nf1 * tau));
            double E2mm = 1.0;
            for (int mm = 0; mm < ns; mm++) {
                ft[wrapi(m + mm, nf1)] += ct[i] * E1 * E2mm * E3[mm];
                E2mm *= E2;
                ft[wrapi(m - mm - 1, nf1)] += ct[i] * E1 / E2mm * E3[mm + 1];
            }
        }
    }
    free(E3);
}

void orc_interp1d(const double *x, const cplx *fntau, int64_t M, int nt, double tau, int ns,
                  int64_t nf1, cplx *c) {
    double hx = TWO_PI / nf1;
    double *E3 = (double *)malloc(sizeof(double) * (ns + 1));
    for (int j = 0; j <= ns; j++) E3[j] = exp(-pow(PI_D * j / nf1, 2) / tau);
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *ft = fntau + (int64_t)t * nf1;
        cplx *ct = c + (int64_t)t * M;
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI);
            int64_t m = 1 + (int64_t)py_floordiv(xi, hx);
            xi = xi - hx * m;
            double E1 = exp(-0.25 * xi * xi / tau);
            double E2 = exp((xi * PI_D) / (nf1 * tau));
            double E2mm = 1.0;
            cplx acc = 0;
            for (int mm = 0; mm < ns; mm++) {
                acc += ft[wrapi(m + mm, nf1)] * E1 * E2mm * E3[mm];
                E2mm *= E2;
                acc += ft[wrapi(m - mm - 1, nf1)] * E1 / E2mm * E3[mm + 1];
            }
            ct[i] = acc / (double)nf1;
        }
    }
    free(E3);
}

void orc_normal1d(const double *x, const double *dcf, const cplx *fntau, int64_t M, int nt,
                  double tau, int ns, int64_t nf1, cplx *ftau) {
    double hx = TWO_PI / nf1;
    int W = 2 * ns;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *fin = fntau + (int64_t)t * nf1;
        cplx *fout = ftau + (int64_t)t * nf1;
        double *Em = (double *)malloc(sizeof(double) * W);
        memset(fout, 0, sizeof(cplx) * nf1);
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI);
            int64_t m1 = 1 + (int64_t)py_floordiv(xi, hx);
            cplx cc = 0;
            for (int mm = -ns; mm < ns; mm++) {
                double d = xi - hx * (m1 + mm);
                Em[mm + ns] = exp(-0.25 * d * d / tau);
                cc += fin[wrapi(m1 + mm, nf1)] * Em[mm + ns];
            }
            cc = cc / (double)nf1;
            if (dcf) cc *= dcf[i];
            for (int mm = -ns; mm < ns; mm++) fout[wrapi(m1 + mm, nf1)] += cc * Em[mm + ns];
        }
        free(Em);
    }
}

/* ------------------------------------------------------------------ 2-D */

static double *e3_table2(int ns, int64_t nf1, int64_t nf2, double tau) {
    double *E3 = (double *)malloc(sizeof(double) * (ns + 1) * (ns + 1));
    for (int l = 0; l <= ns; l++)
        for (int j = 0; j <= ns; j++)
            E3[j * (ns + 1) + l] = exp(-(pow(PI_D * j / nf1, 2) + pow(PI_D * l / nf2, 2)) / tau);
    return E3;
}

void orc_spread2d(const double *x, const double *y, const cplx *c, int64_t M, int nt, double tau,
                  int ns, int64_t nf1, int64_t nf2, cplx *ftau) {
    double hx = TWO_PI / nf1, hy = TWO_PI / nf2;
    double *E3 = e3_table2(ns, nf1, nf2, tau);
    int S = ns + 1;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *ct = c + (int64_t)t * M;
        cplx *ft = ftau + (int64_t)t * nf1 * nf2;
        memset(ft, 0, sizeof(cplx) * nf1 * nf2);
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI), yi = py_mod(y[i], TWO_PI);
            int64_t mx = 1 + (int64_t)py_floordiv(xi, hx);
            int64_t my = 1 + (int64_t)py_floordiv(yi, hy);
            xi = xi - hx * mx;
            yi = yi - hy * my;
            double E1 = exp(-0.25 * (xi * xi + yi * yi) / tau);
            double E2x = exp((xi * PI_D) / (nf1 * tau));
            double E2y = exp((yi * PI_D) / (nf2 * tau));
            cplx V0 = ct[i] * E1;
            double E2mmx = 1.0;
            for (int mmx = 0; mmx < ns; mmx++) {
                double E2mmy = 1.0;
                int64_t ip = wrapi(mx + mmx, nf1) * nf2, in = wrapi(mx - mmx - 1, nf1) * nf2;
                for (int mmy = 0; mmy < ns; mmy++) {
                    int64_t jp = wrapi(my + mmy, nf2), jn = wrapi(my - mmy - 1, nf2);
                    ft[ip + jp] += V0 * E2mmx * E2mmy * E3[mmx * S + mmy];
                    ft[ip + jn] += V0 * E2mmx / (E2mmy * E2y) * E3[mmx * S + mmy + 1];
                    ft[in + jp] += V0 / (E2mmx * E2x) * E2mmy * E3[(mmx + 1) * S + mmy];
                    ft[in + jn] += V0 / (E2mmx * E2x) / (E2mmy * E2y) * E3[(mmx + 1) * S + mmy + 1];
                    E2mmy *= E2y;
                }
                E2mmx *= E2x;
            }
        }
    }
    free(E3);
}

void orc_interp2d(const double *x, const double *y, const cplx *fntau, int64_t M, int nt,
                  double tau, int ns, int64_t nf1, int64_t nf2, cplx *c) {
    double hx = TWO_PI / nf1, hy = TWO_PI / nf2;
    double *E3 = e3_table2(ns, nf1, nf2, tau);
    int S = ns + 1;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *ft = fntau + (int64_t)t * nf1 * nf2;
        cplx *ct = c + (int64_t)t * M;
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI), yi = py_mod(y[i], TWO_PI);
            int64_t mx = 1 + (int64_t)py_floordiv(xi, hx);
            int64_t my = 1 + (int64_t)py_floordiv(yi, hy);
            xi = xi - hx * mx;
            yi = yi - hy * my;
            double E1 = exp(-0.25 * (xi * xi + yi * yi) / tau);
            double E2x = exp((xi * PI_D) / (nf1 * tau));
            double E2y = exp((yi * PI_D) / (nf2 * tau));
            double E2mmx = 1.0;
            cplx acc = 0;
            for (int mmx = 0; mmx < ns; mmx++) {
                double E2mmy = 1.0;
                int64_t ip = wrapi(mx + mmx, nf1) * nf2, in = wrapi(mx - mmx - 1, nf1) * nf2;
                for (int mmy = 0; mmy < ns; mmy++) {
                    int64_t jp = wrapi(my + mmy, nf2), jn = wrapi(my - mmy - 1, nf2);
                    acc += ft[ip + jp] * E1 * E2mmx * E2mmy * E3[mmx * S + mmy];
                    acc += ft[ip + jn] * E1 * E2mmx / (E2mmy * E2y) * E3[mmx * S + mmy + 1];
                    acc += ft[in + jp] * E1 / (E2mmx * E2x) * E2mmy * E3[(mmx + 1) * S + mmy];
                    acc += ft[in + jn] * E1 / (E2mmx * E2x) / (E2mmy * E2y) * E3[(mmx + 1) * S + mmy + 1];
                    E2mmy *= E2y;
                }
                E2mmx *= E2x;
            }
            ct[i] = acc / (double)(nf1 * nf2);
        }
    }
    free(E3);
}

void orc_normal2d(const double *x, const double *y, const double *dcf, const cplx *fntau, int64_t M,
                  int nt, double tau, int ns, int64_t nf1, int64_t nf2, cplx *ftau) {
    double hx = TWO_PI / nf1, hy = TWO_PI / nf2;
    int W = 2 * ns;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *fin = fntau + (int64_t)t * nf1 * nf2;
        cplx *fout = ftau + (int64_t)t * nf1 * nf2;
        double *Em = (double *)malloc(sizeof(double) * W * W);
        memset(fout, 0, sizeof(cplx) * nf1 * nf2);
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI), yi = py_mod(y[i], TWO_PI);
            int64_t m1 = 1 + (int64_t)py_floordiv(xi, hx);
            int64_t m2 = 1 + (int64_t)py_floordiv(yi, hy);
            cplx cc = 0;
            for (int a = -ns; a < ns; a++) {
                double dx = xi - hx * (m1 + a);
                int64_t ia = wrapi(m1 + a, nf1) * nf2;
                for (int b = -ns; b < ns; b++) {
                    double dy = yi - hy * (m2 + b);
                    double e = exp(-0.25 * (dx * dx + dy * dy) / tau);
                    Em[(a + ns) * W + b + ns] = e;
                    cc += fin[ia + wrapi(m2 + b, nf2)] * e;
                }
            }
            cc = cc / (double)(nf1 * nf2);
            if (dcf) cc *= dcf[i];
            for (int a = -ns; a < ns; a++) {
                int64_t ia = wrapi(m1 + a, nf1) * nf2;
                for (int b = -ns; b < ns; b++) fout[ia + wrapi(m2 + b, nf2)] += cc * Em[(a + ns) * W + b + ns];
            }
        }
        free(Em);
    }
}

/* ------------------------------------------------------------------ 3-D */

static double *e3_table3(int ns, int64_t nf1, int64_t nf2, int64_t nf3, double tau) {
    int S = ns + 1;
    double *E3 = (double *)malloc(sizeof(double) * S * S * S);
    for (int p = 0; p < S; p++)
        for (int l = 0; l < S; l++)
            for (int j = 0; j < S; j++)
                E3[(j * S + l) * S + p] =
                    exp(-(pow(PI_D * j / nf1, 2) + pow(PI_D * l / nf2, 2) + pow(PI_D * p / nf3, 2)) / tau);
    return E3;
}

void orc_spread3d(const double *x, const double *y, const double *z, const cplx *c, int64_t M, int nt,
                  double tau, int ns, int64_t nf1, int64_t nf2, int64_t nf3, cplx *ftau) {
    double hx = TWO_PI / nf1, hy = TWO_PI / nf2, hz = TWO_PI / nf3;
    double *E3 = e3_table3(ns, nf1, nf2, nf3, tau);
    int S = ns + 1;
    int64_t G = nf1 * nf2 * nf3;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *ct = c + (int64_t)t * M;
        cplx *ft = ftau + (int64_t)t * G;
        memset(ft, 0, sizeof(cplx) * G);
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI), yi = py_mod(y[i], TWO_PI), zi = py_mod(z[i], TWO_PI);
            int64_t mx = 1 + (int64_t)py_floordiv(xi, hx);
            int64_t my = 1 + (int64_t)py_floordiv(yi, hy);
            int64_t mz = 1 + (int64_t)py_floordiv(zi, hz);
            xi = xi - hx * mx;
            yi = yi - hy * my;
            zi = zi - hz * mz;
            double E1 = exp(-0.25 * (xi * xi + yi * yi + zi * zi) / tau);
            double E2x = exp((xi * PI_D) / (nf1 * tau));
            double E2y = exp((yi * PI_D) / (nf2 * tau));
            double E2z = exp((zi * PI_D) / (nf3 * tau));
            cplx V0 = ct[i] * E1;
            double E2mmx = 1.0;
            for (int a = 0; a < ns; a++) {
                double E2mmy = 1.0;
                int64_t ip = wrapi(mx + a, nf1) * nf2 * nf3, in = wrapi(mx - a - 1, nf1) * nf2 * nf3;
                double wxp = E2mmx, wxn = 1.0 / (E2mmx * E2x);
                for (int b = 0; b < ns; b++) {
                    int64_t jp = wrapi(my + b, nf2) * nf3, jn = wrapi(my - b - 1, nf2) * nf3;
                    double wyp = E2mmy, wyn = 1.0 / (E2mmy * E2y);
                    double E2mmz = 1.0;
                    for (int q = 0; q < ns; q++) {
                        int64_t kp = wrapi(mz + q, nf3), kn = wrapi(mz - q - 1, nf3);
                        double wzp = E2mmz, wzn = 1.0 / (E2mmz * E2z);
                        ft[ip + jp + kp] += V0 * wxp * wyp * wzp * E3[(a * S + b) * S + q];
                        ft[ip + jn + kp] += V0 * wxp * wyn * wzp * E3[(a * S + b + 1) * S + q];
                        ft[in + jp + kp] += V0 * wxn * wyp * wzp * E3[((a + 1) * S + b) * S + q];
                        ft[in + jn + kp] += V0 * wxn * wyn * wzp * E3[((a + 1) * S + b + 1) * S + q];
                        ft[ip + jp + kn] += V0 * wxp * wyp * wzn * E3[(a * S + b) * S + q + 1];
                        ft[ip + jn + kn] += V0 * wxp * wyn * wzn * E3[(a * S + b + 1) * S + q + 1];
                        ft[in + jp + kn] += V0 * wxn * wyp * wzn * E3[((a + 1) * S + b) * S + q + 1];
                        ft[in + jn + kn] += V0 * wxn * wyn * wzn * E3[((a + 1) * S + b + 1) * S + q + 1];
                        E2mmz *= E2z;
                    }
                    E2mmy *= E2y;
                }
                E2mmx *= E2x;
            }
        }
    }
    free(E3);
}

void orc_interp3d(const double *x, const double *y, const double *z, const cplx *fntau, int64_t M,
                  int nt, double tau, int ns, int64_t nf1, int64_t nf2, int64_t nf3, cplx *c) {
    double hx = TWO_PI / nf1, hy = TWO_PI / nf2, hz = TWO_PI / nf3;
    double *E3 = e3_table3(ns, nf1, nf2, nf3, tau);
    int S = ns + 1;
    int64_t G = nf1 * nf2 * nf3;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *ft = fntau + (int64_t)t * G;
        cplx *ct = c + (int64_t)t * M;
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI), yi = py_mod(y[i], TWO_PI), zi = py_mod(z[i], TWO_PI);
            int64_t mx = 1 + (int64_t)py_floordiv(xi, hx);
            int64_t my = 1 + (int64_t)py_floordiv(yi, hy);
            int64_t mz = 1 + (int64_t)py_floordiv(zi, hz);
            xi = xi - hx * mx;
            yi = yi - hy * my;
            zi = zi - hz * mz;
            double E1 = exp(-0.25 * (xi * xi + yi * yi + zi * zi) / tau);
            double E2x = exp((xi * PI_D) / (nf1 * tau));
            double E2y = exp((yi * PI_D) / (nf2 * tau));
            double E2z = exp((zi * PI_D) / (nf3 * tau));
            cplx acc = 0;
            double E2mmx = 1.0;
            for (int a = 0; a < ns; a++) {
                double E2mmy = 1.0;
                int64_t ip = wrapi(mx + a, nf1) * nf2 * nf3, in = wrapi(mx - a - 1, nf1) * nf2 * nf3;
                double wxp = E2mmx, wxn = 1.0 / (E2mmx * E2x);
                for (int b = 0; b < ns; b++) {
                    int64_t jp = wrapi(my + b, nf2) * nf3, jn = wrapi(my - b - 1, nf2) * nf3;
                    double wyp = E2mmy, wyn = 1.0 / (E2mmy * E2y);
                    double E2mmz = 1.0;
                    for (int q = 0; q < ns; q++) {
                        int64_t kp = wrapi(mz + q, nf3), kn = wrapi(mz - q - 1, nf3);
                        double wzp = E2mmz, wzn = 1.0 / (E2mmz * E2z);
                        acc += ft[ip + jp + kp] * E1 * wxp * wyp * wzp * E3[(a * S + b) * S + q];
                        acc += ft[ip + jn + kp] * E1 * wxp * wyn * wzp * E3[(a * S + b + 1) * S + q];
                        acc += ft[in + jp + kp] * E1 * wxn * wyp * wzp * E3[((a + 1) * S + b) * S + q];
                        acc += ft[in + jn + kp] * E1 * wxn * wyn * wzp * E3[((a + 1) * S + b + 1) * S + q];
                        acc += ft[ip + jp + kn] * E1 * wxp * wyp * wzn * E3[(a * S + b) * S + q + 1];
                        acc += ft[ip + jn + kn] * E1 * wxp * wyn * wzn * E3[(a * S + b + 1) * S + q + 1];
                        acc += ft[in + jp + kn] * E1 * wxn * wyp * wzn * E3[((a + 1) * S + b) * S + q + 1];
                        acc += ft[in + jn + kn] * E1 * wxn * wyn * wzn * E3[((a + 1) * S + b + 1) * S + q + 1];
                        E2mmz *= E2z;
                    }
                    E2mmy *= E2y;
                }
                E2mmx *= E2x;
            }
            ct[i] = acc / (double)G;
        }
    }
    free(E3);
}

void orc_normal3d(const double *x, const double *y, const double *z, const double *dcf,
                  const cplx *fntau, int64_t M, int nt, double tau, int ns, int64_t nf1, int64_t nf2,
                  int64_t nf3, cplx *ftau) {
    double hx = TWO_PI / nf1, hy = TWO_PI / nf2, hz = TWO_PI / nf3;
    int W = 2 * ns;
    int64_t G = nf1 * nf2 * nf3;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; t++) {
        const cplx *fin = fntau + (int64_t)t * G;
        cplx *fout = ftau + (int64_t)t * G;
        double *Em = (double *)malloc(sizeof(double) * W * W * W);
        memset(fout, 0, sizeof(cplx) * G);
        for (int64_t i = 0; i < M; i++) {
            double xi = py_mod(x[i], TWO_PI), yi = py_mod(y[i], TWO_PI), zi = py_mod(z[i], TWO_PI);
            int64_t m1 = 1 + (int64_t)py_floordiv(xi, hx);
            int64_t m2 = 1 + (int64_t)py_floordiv(yi, hy);
            int64_t m3 = 1 + (int64_t)py_floordiv(zi, hz);
            cplx cc = 0;
            for (int a = -ns; a < ns; a++) {
                double dx = xi - hx * (m1 + a);
                int64_t ia = wrapi(m1 + a, nf1) * nf2 * nf3;
                for (int b = -ns; b < ns; b++) {
                    double dy = yi - hy * (m2 + b);
                    int64_t ib = ia + wrapi(m2 + b, nf2) * nf3;
                    for (int q = -ns; q < ns; q++) {
                        double dz = zi - hz * (m3 + q);
                        double e = exp(-0.25 * (dx * dx + dy * dy + dz * dz) / tau);
                        Em[((a + ns) * W + b + ns) * W + q + ns] = e;
                        cc += fin[ib + wrapi(m3 + q, nf3)] * e;
                    }
                }
            }
            cc = (dcf ? dcf[i] : 1.0) * cc / (double)G;
            for (int a = -ns; a < ns; a++) {
                int64_t ia = wrapi(m1 + a, nf1) * nf2 * nf3;
                for (int b = -ns; b < ns; b++) {
                    int64_t ib = ia + wrapi(m2 + b, nf2) * nf3;
                    for (int q = -ns; q < ns; q++)
                        fout[ib + wrapi(m3 + q, nf3)] += cc * Em[((a + ns) * W + b + ns) * W + q + ns];
                }
            }
        }
        free(Em);
    }
}
