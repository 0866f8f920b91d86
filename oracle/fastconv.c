/*
 * Oracle, timed-baseline variant: the fault-fault traction rate of equation.jl:44-61 through a
 * fast Fourier transform, and many independent models integrated in parallel, one per host thread.
 *
 * TEST INFRASTRUCTURE ONLY (the timed CPU baseline; never linked into the product).
 *
 * The reference applies the block-Toeplitz operator by FFTW real transforms of length 2nx-1
 * (equation.jl:44-61, GF.jl:60-67). The checker path of this oracle (orc_dtau_dt in ode.c) keeps
 * that length and evaluates the transforms as direct O(n^2) sums, which is exact to round-off but
 * far slower than FFTW. For timing, this file computes the same linear Toeplitz sum
 *   dtau[i, j] = sum_{k, l} st[|i - k|, j, l] (v[k, l] - vpl)
 * by radix-2 complex FFTs of length P = 2^ceil(log2(2nx - 1)) (zero padding to any length >= 2nx - 1
 * gives the same linear sum): the kernel column h[d] = st[|d|] placed circularly is real and even,
 * so its spectrum is real; two real columns share one complex transform. Results agree with the
 * direct path to round-off (tests/test_oracle_ode.py).
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include "gbc_oracle.h"

/* the convolution table a thread uses inside orc_dtau_dt while it integrates one member */
_Thread_local const orc_fftconv* orc_tl_fastconv = NULL;

typedef struct { int P; double *cs, *sn; int* rev; } fft_plan;
static _Thread_local fft_plan fp_tl = {0, NULL, NULL, NULL};

static const fft_plan* plan_get(int P) {
    fft_plan* p = &fp_tl;
    if (p->P == P) return p;
    free(p->cs); free(p->sn); free(p->rev);
    p->cs = (double*)malloc(sizeof(double) * (P / 2));
    p->sn = (double*)malloc(sizeof(double) * (P / 2));
    p->rev = (int*)malloc(sizeof(int) * P);
    for (int k = 0; k < P / 2; ++k) { p->cs[k] = cos(2.0 * M_PI * k / P); p->sn[k] = sin(2.0 * M_PI * k / P); }
    int bits = 0;
    while ((1 << bits) < P) ++bits;
    for (int i = 0; i < P; ++i) {
        int r = 0;
        for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
        p->rev[i] = r;
    }
    p->P = P;
    return p;
}

/* in-place iterative radix-2 transform of P interleaved complex values; sign -1 forward, +1 inverse
 * (unscaled) */
static void fft(double* z, const fft_plan* p, int sign) {
    const int P = p->P;
    for (int i = 0; i < P; ++i) {
        const int r = p->rev[i];
        if (r > i) {
            double t0 = z[2 * i], t1 = z[2 * i + 1];
            z[2 * i] = z[2 * r]; z[2 * i + 1] = z[2 * r + 1];
            z[2 * r] = t0; z[2 * r + 1] = t1;
        }
    }
    for (int len = 2; len <= P; len <<= 1) {
        const int half = len >> 1, step = P / len;
        for (int s = 0; s < P; s += len)
            for (int k = 0; k < half; ++k) {
                const double wr = p->cs[k * step], wi = sign * p->sn[k * step];
                double* a = z + 2 * (s + k);
                double* b = z + 2 * (s + k + half);
                const double tr = b[0] * wr - b[1] * wi, ti = b[0] * wi + b[1] * wr;
                b[0] = a[0] - tr; b[1] = a[1] - ti;
                a[0] += tr; a[1] += ti;
            }
    }
}

static int pow2_at_least(int n) {
    int P = 1;
    while (P < n) P <<= 1;
    return P;
}

/* real Toeplitz kernel st[d, j, l] (d < nx) from the model's complex rFFT form (length 2nx-1, nx bins) */
static void kernel_from_dft(const orc_model* m, double* st) {
    const int nx = m->nx, nxi = m->nxi, n = 2 * nx - 1;
    double* cs = (double*)malloc(sizeof(double) * n);
    double* sn = (double*)malloc(sizeof(double) * n);
    for (int q = 0; q < n; ++q) { cs[q] = cos(2.0 * M_PI * q / n); sn[q] = sin(2.0 * M_PI * q / n); }
    for (int jl = 0; jl < nxi * nxi; ++jl)
        for (int d = 0; d < nx; ++d) {
            const double* g = m->gf11_dft + 2 * (size_t)nx * jl;
            double acc = g[0];
            int q = 0;  /* k * d mod n, advanced by d per k */
            for (int k = 1; k < nx; ++k) {
                q += d;
                if (q >= n) q -= n;
                acc += 2.0 * (g[2 * k] * cs[q] - g[2 * k + 1] * sn[q]);
            }
            st[d + (size_t)nx * jl] = acc / n;
        }
    free(cs);
    free(sn);
}

int orc_fftconv_init(const orc_model* m, orc_fftconv* c) {
    const int nx = m->nx, nxi = m->nxi, P = pow2_at_least(2 * nx - 1);
    c->P = P;
    c->nx = nx;
    c->nxi = nxi;
    c->H = (double*)malloc(sizeof(double) * (size_t)P * nxi * nxi);
    double* st = (double*)malloc(sizeof(double) * (size_t)nx * nxi * nxi);
    double* z = (double*)malloc(sizeof(double) * 2 * (size_t)P);
    if (!c->H || !st || !z) { free(st); free(z); return -1; }
    kernel_from_dft(m, st);
    const fft_plan* p = plan_get(P);
    for (int j = 0; j < nxi; ++j)
        for (int l = 0; l < nxi; ++l) {
            const double* col = st + (size_t)nx * (j + (size_t)nxi * l);
            memset(z, 0, sizeof(double) * 2 * (size_t)P);
            z[0] = col[0];
            for (int d = 1; d < nx; ++d) z[2 * d] = z[2 * (P - d)] = col[d];
            fft(z, p, -1);
            for (int k = 0; k < P; ++k) c->H[((size_t)k * nxi + j) * nxi + l] = z[2 * k];  /* even kernel: real spectrum */
        }
    free(st);
    free(z);
    return 0;
}

void orc_fftconv_free(orc_fftconv* c) {
    free(c->H);
    c->H = NULL;
}

/* dtau (nx,nxi) from v through the tables of c (single-threaded) */
void orc_dtau_dt_fft(const orc_fftconv* c, const orc_model* m, const double* v, double* dtau) {
    const int nx = c->nx, nxi = c->nxi, P = c->P;
    const fft_plan* p = plan_get(P);
    double* X = (double*)malloc(sizeof(double) * 2 * (size_t)P * nxi);  /* X[k][l] complex */
    double* Y = (double*)malloc(sizeof(double) * 2 * (size_t)P * nxi);
    double* z = (double*)malloc(sizeof(double) * 2 * (size_t)P);
    for (int l = 0; l < nxi; l += 2) {
        const int two = (l + 1 < nxi);
        memset(z, 0, sizeof(double) * 2 * (size_t)P);
        for (int r = 0; r < nx; ++r) {
            z[2 * r] = v[r + (size_t)nx * l] - m->vpl;
            if (two) z[2 * r + 1] = v[r + (size_t)nx * (l + 1)] - m->vpl;
        }
        fft(z, p, -1);
        for (int k = 0; k < P; ++k) {
            const int q = (P - k) & (P - 1);
            const double ar = z[2 * k], ai = z[2 * k + 1], br = z[2 * q], bi = -z[2 * q + 1];  /* Z[k], conj Z[-k] */
            double* xa = X + 2 * ((size_t)k * nxi + l);
            xa[0] = 0.5 * (ar + br);
            xa[1] = 0.5 * (ai + bi);
            if (two) {  /* (Z[k] - conj Z[-k]) / 2i */
                double* xb = X + 2 * ((size_t)k * nxi + l + 1);
                xb[0] = 0.5 * (ai - bi);
                xb[1] = -0.5 * (ar - br);
            }
        }
    }
    for (int k = 0; k < P; ++k) {
        const double* H = c->H + (size_t)k * nxi * nxi;
        const double* x = X + 2 * (size_t)k * nxi;
        double* y = Y + 2 * (size_t)k * nxi;
        for (int j = 0; j < nxi; ++j) {
            double re = 0.0, im = 0.0;
            for (int l = 0; l < nxi; ++l) {
                re += H[j * nxi + l] * x[2 * l];
                im += H[j * nxi + l] * x[2 * l + 1];
            }
            y[2 * j] = re;
            y[2 * j + 1] = im;
        }
    }
    for (int j = 0; j < nxi; j += 2) {
        const int two = (j + 1 < nxi);
        for (int k = 0; k < P; ++k) {  /* W = Y_j + i Y_{j+1}: both inverse transforms are real */
            const double* ya = Y + 2 * ((size_t)k * nxi + j);
            z[2 * k] = ya[0];
            z[2 * k + 1] = ya[1];
            if (two) {
                const double* yb = Y + 2 * ((size_t)k * nxi + j + 1);
                z[2 * k] -= yb[1];
                z[2 * k + 1] += yb[0];
            }
        }
        fft(z, p, +1);
        for (int r = 0; r < nx; ++r) {
            dtau[r + (size_t)nx * j] = z[2 * r] / P;
            if (two) dtau[r + (size_t)nx * (j + 1)] = z[2 * r + 1] / P;
        }
    }
    free(X);
    free(Y);
    free(z);
}

/* Independent models integrated in parallel: one model per host thread at a time (dynamic
 * schedule), each model's right-hand side single-threaded (nested parallel regions inactive),
 * with the FFT convolution when fft != 0. us[i] is model i's flat state, overwritten with u(t1[i]). */
int orc_integrate_many(const orc_model* const* ms, int nm, double* const* us, const double* t0, const double* t1,
                       const orc_solver_opts* o, orc_solver_stats* st, int fft, int nthreads) {
    orc_fftconv* conv = NULL;
    if (fft) {
        conv = (orc_fftconv*)calloc((size_t)nm, sizeof(orc_fftconv));
        if (!conv) return -1;
    }
    const int levels = omp_get_max_active_levels();
    omp_set_max_active_levels(1);
    int bad = 0;
    if (fft) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : bad)
        for (int i = 0; i < nm; ++i) bad |= orc_fftconv_init(ms[i], &conv[i]) != 0;
    }
    if (!bad) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
        for (int i = 0; i < nm; ++i) {
            orc_tl_fastconv = fft ? &conv[i] : NULL;
            orc_integrate(ms[i], us[i], t0[i], t1[i], o, &st[i]);
            orc_tl_fastconv = NULL;
        }
    }
    omp_set_max_active_levels(levels);
    if (fft) {
        for (int i = 0; i < nm; ++i) orc_fftconv_free(&conv[i]);
        free(conv);
    }
    return bad ? -1 : 0;
}
