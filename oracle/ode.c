/*
 * Oracle: the ODE right-hand sides of src/BEM/equation.jl and an adaptive Tsit5 integrator
 * standing in for the reference's OrdinaryDiffEq caller.
 *
 * TEST INFRASTRUCTURE ONLY (the FP64 reference the CUDA path is tested against, and the timed CPU baseline; never
 * linked into the product).
 *
 * The fault-fault traction rate is computed as the reference does it (equation.jl:44-61): a real
 * DFT of the zero-padded v - vpl along strike (length 2nx-1), a per-frequency complex
 * multiply-accumulate with the rFFT'd kernel, and the inverse real DFT truncated to nx rows. The
 * DFT is the direct O(n^2) sum with tabulated twiddles (FFTW is not available here).
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include "gbc_oracle.h"

typedef struct { int n; double *cs, *sn; } twiddle;
static _Thread_local twiddle tw = {0, NULL, NULL};

static void tw_get(int n) {
    if (tw.n == n) return;
    free(tw.cs); free(tw.sn);
    tw.cs = (double*)malloc(sizeof(double) * n);
    tw.sn = (double*)malloc(sizeof(double) * n);
    for (int m = 0; m < n; ++m) { tw.cs[m] = cos(2.0 * M_PI * m / n); tw.sn[m] = sin(2.0 * M_PI * m / n); }
    tw.n = n;
}

/* relative_velocity! + dtau_dt! (equation.jl:35-61): dtau (nx,nxi) from v. A thread integrating
 * under orc_integrate_many with fft on takes the FFT variant of fastconv.c instead. */
void orc_dtau_dt(const orc_model* m, const double* v, double* dtau) {
    if (orc_tl_fastconv) {
        orc_dtau_dt_fft(orc_tl_fastconv, m, v, dtau);
        return;
    }
    const int nx = m->nx, nxi = m->nxi, n = 2 * nx - 1;
    tw_get(n);
    const double* cs = tw.cs;  /* the calling thread's tables (they are thread-local) */
    const double* sn = tw.sn;
    double* X = (double*)malloc(sizeof(double) * 2 * nx * nxi);   /* relv_dft (nx,nxi) complex */
    double* Y = (double*)calloc(2 * (size_t)nx * nxi, sizeof(double)); /* dtau_dft */
    /* every output element is summed by one thread in a fixed order: results do not depend on the
     * thread count */
#pragma omp parallel for schedule(static)
    for (int l = 0; l < nxi; ++l)
        for (int k = 0; k < nx; ++k) {
            double re = 0.0, im = 0.0;
            for (int r = 0; r < nx; ++r) {
                double val = v[r + nx * l] - m->vpl;
                int idx = (int)(((long long)k * r) % n);
                re += val * cs[idx];
                im -= val * sn[idx];
            }
            X[2 * (k + nx * l)] = re;
            X[2 * (k + nx * l) + 1] = im;
        }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nxi; ++j)
        for (int l = 0; l < nxi; ++l)
            for (int k = 0; k < nx; ++k) {
                const double* g = m->gf11_dft + 2 * ((size_t)k + (size_t)nx * (j + (size_t)nxi * l));
                const double* x = X + 2 * (k + nx * l);
                double* y = Y + 2 * (k + nx * j);
                y[0] += g[0] * x[0] - g[1] * x[1];
                y[1] += g[0] * x[1] + g[1] * x[0];
            }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nxi; ++j)
        for (int r = 0; r < nx; ++r) {
            double acc = Y[2 * (nx * j)];
            for (int k = 1; k < nx; ++k) {
                int idx = (int)(((long long)k * r) % n);
                const double* y = Y + 2 * (k + nx * j);
                acc += 2.0 * (y[0] * cs[idx] - y[1] * sn[idx]);
            }
            dtau[r + nx * j] = acc / n;
        }
    free(X);
    free(Y);
}

/* update_fault! with the ageing law (equation.jl:233-246, :279) */
static void update_fault(const orc_model* m, const double* dtau, const double* v, const double* th,
                         double* dv, double* dth, double* ddelta) {
    const int N = m->nx * m->nxi;
    for (int i = 0; i < N; ++i) {
        double psi1 = exp((m->f0 + m->b[i] * log(m->v0 * fmax(0.0, th[i]) / m->L[i])) / m->a[i]) / (2.0 * m->v0);
        double psi2 = m->sigma[i] * psi1 / hypot(1.0, v[i] * psi1);
        double dmu_dv = m->a[i] * psi2;
        double dmu_dth = m->b[i] / th[i] * v[i] * psi2;
        dth[i] = 1.0 - v[i] * th[i] / m->L[i];
        dv[i] = (dtau[i] - dmu_dth * dth[i]) / (dmu_dv + m->eta);
        ddelta[i] = v[i];
    }
}

void orc_ode_fault(const orc_model* m, const double* v, const double* th, double* dv, double* dth,
                   double* ddelta) {
    const int N = m->nx * m->nxi;
    double* dtau = (double*)malloc(sizeof(double) * N);
    orc_dtau_dt(m, v, dtau);
    update_fault(m, dtau, v, th, dv, dth, ddelta);
    free(dtau);
}

/* y (+)= A x for column-major A (rows x cols); rows split across threads */
/* y (+)= A x for a column-major A: row blocks in parallel, each row summing its columns in order
 * (the result does not depend on the blocking). Short matrices (the 1000-row mantle->fault block
 * of a 1000-patch fault) get thinner blocks so that every thread streams a part. */
static void gemv_cm(const double* A, size_t rows, size_t cols, const double* x, double* y, int accumulate) {
    const size_t nt = (size_t)omp_get_max_threads();
    size_t B = 512;  /* 4 KB of a column per block: long contiguous runs for the tall blocks */
    if ((rows + B - 1) / B < nt) {
        B = (rows + nt - 1) / nt;
        B = B < 32 ? 32 : (B + 7) / 8 * 8;
    }
    const long nb = (long)((rows + B - 1) / B);
#pragma omp parallel for schedule(static)
    for (long bi = 0; bi < nb; ++bi) {
        size_t r0 = (size_t)bi * B, r1 = r0 + B < rows ? r0 + B : rows;
        double acc[512];
        for (size_t r = r0; r < r1; ++r) acc[r - r0] = accumulate ? y[r] : 0.0;
        for (size_t c = 0; c < cols; ++c) {
            const double xc = x[c];
            const double* a = A + rows * c;
            for (size_t r = r0; r < r1; ++r) acc[r - r0] += a[r] * xc;
        }
        for (size_t r = r0; r < r1; ++r) y[r] = acc[r - r0];
    }
}

void orc_ode_visco(const orc_model* m, const double* v, const double* th, const double* sig,
                   double* dv, double* dth, double* deps, double* dsig, double* ddelta) {
    const int N = m->nx * m->nxi, ne = m->ne;
    double* dtau = (double*)malloc(sizeof(double) * N);
    double* relv = (double*)malloc(sizeof(double) * N);
    double* reldeps = (double*)malloc(sizeof(double) * 6 * (size_t)ne);
    for (int i = 0; i < N; ++i) relv[i] = v[i] - m->vpl;
    /* update_strain_rate! (equation.jl:207-222) with the power law dϵ = γ σ' τ^n (:285) */
    for (int i = 0; i < ne; ++i) {
        const double* s = sig;
        double skk = (s[i] + s[i + 3 * ne] + s[i + 5 * ne]) / 3.0;
        double sxx = s[i] - skk, syy = s[i + 3 * ne] - skk, szz = s[i + 5 * ne] - skk;
        double sxy = s[i + ne], sxz = s[i + 2 * ne], syz = s[i + 4 * ne];
        double tau = sqrt(sxx * sxx + syy * syy + szz * szz + 2.0 * (sxy * sxy + sxz * sxz + syz * syz));
        /* one law (equation.jl:285) or the sum of a composite's laws (equation.jl:286-292) */
        double f = 0.0;
        const int K = m->nlaws > 1 ? m->nlaws : 1;
        for (int k = 0; k < K; ++k) f += m->gamma[i + (size_t)k * ne] * pow(tau, m->n[i + (size_t)k * ne]);
        deps[i] = f * sxx;
        deps[i + ne] = f * sxy;
        deps[i + 2 * ne] = f * sxz;
        deps[i + 3 * ne] = f * syy;
        deps[i + 4 * ne] = f * syz;
        deps[i + 5 * ne] = f * szz;
    }
    /* relative_strain_rate! (:224-230) */
    for (int k = 0; k < 6; ++k)
        for (int i = 0; i < ne; ++i) reldeps[i + k * ne] = deps[i + k * ne] - m->deps0[k];
    orc_dtau_dt(m, v, dtau);                                        /* :200 */
    gemv_cm(m->gf21, N, 6 * (size_t)ne, reldeps, dtau, 1);          /* :201 */
    gemv_cm(m->gf12, 6 * (size_t)ne, N, relv, dsig, 0);             /* :202 */
    gemv_cm(m->gf22, 6 * (size_t)ne, 6 * (size_t)ne, reldeps, dsig, 1); /* :203 */
    update_fault(m, dtau, v, th, dv, dth, ddelta);                  /* :204 */
    free(dtau); free(relv); free(reldeps);
}

/* update_fault_with_dilatancy! (equation.jl:248-276) with d𝓅_dt (:282) */
void orc_ode_dilatancy(const orc_model* m, const double* v, const double* th, const double* p,
                       double* dv, double* dth, double* ddelta, double* dp) {
    const int N = m->nx * m->nxi;
    double* dtau = (double*)malloc(sizeof(double) * N);
    orc_dtau_dt(m, v, dtau);
    for (int i = 0; i < N; ++i) {
        dth[i] = 1.0 - v[i] * th[i] / m->L[i];
        dp[i] = -(p[i] - m->p0[i]) / m->tp[i] + m->deps[i] / m->beta[i] / th[i] * dth[i];
        const double af = m->a[i] / m->f0, bf = m->b[i] / m->f0;
        const double vf = fmax(0.0, v[i] / m->v0), thf = fmax(0.0, th[i] * m->v0 / m->L[i]);
        const double vfa1 = pow(vf, af - 1.0), thfb1 = pow(thf, bf - 1.0);
        const double vfa = pow(vf, af), thfb = pow(thf, bf);
        dv[i] = (dtau[i] + m->f0 * dp[i] * vfa * thfb -
                 m->f0 * (m->sigma[i] - p[i]) * vfa * thfb1 * bf * m->v0 / m->L[i] * dth[i]) /
                (m->f0 * (m->sigma[i] - p[i]) * vfa1 * thfb * af / m->v0);
        ddelta[i] = v[i];
    }
    free(dtau);
}

long long orc_state_len(const orc_model* m, int mantle) {
    long long N = (long long)m->nx * m->nxi;
    if (mantle == 2) return 4 * N;
    return mantle ? 3 * N + 12LL * m->ne : 3 * N;
}

static void rhs_flat(const orc_model* m, int mantle, const double* u, double* du) {
    const long long N = (long long)m->nx * m->nxi;
    if (mantle == 2) {
        orc_ode_dilatancy(m, u, u + N, u + 3 * N, du, du + N, du + 2 * N, du + 3 * N);
        return;
    }
    if (!mantle) {
        orc_ode_fault(m, u, u + N, du, du + N, du + 2 * N);
    } else {
        const long long E = 6LL * m->ne;
        orc_ode_visco(m, u, u + N, u + 2 * N + E, du, du + N, du + 2 * N, du + 2 * N + E,
                      du + 2 * N + 2 * E);
    }
}

/* Tsitouras (2011) 5(4) tableau (order conditions verified by tests/test_oracle_ode.py). The
 * right-hand side is autonomous, so the stage abscissae c_i are not needed here. */
static const double TA[7][6] = {
    {0},
    {0.161},
    {-0.008480655492356989, 0.335480655492357},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
static const double TE[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                             -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                             0.015151515151515152};

void orc_tsit5_tableau(double a[7][6], double e[7]) {
    memcpy(a, TA, sizeof(TA));
    memcpy(e, TE, sizeof(TE));
}

int orc_integrate(const orc_model* m, double* u, double t0, double t1, const orc_solver_opts* o,
                  orc_solver_stats* stt) {
    return orc_integrate_record(m, u, t0, t1, o, stt, 0, 0, NULL, NULL, NULL);
}

/* VCABM5: variable-coefficient Adams-Bashforth-Moulton in PECE mode, orders 1..5, restated from
 * the published method (Hairer, Norsett & Wanner, Solving ODEs I, sec. III.5, Krogh's modified
 * divided differences; Shampine & Gordon 1975), standing in for OrdinaryDiffEq's VCABM5 used by
 * the reference's example (examples/otf-with-mantle.jl:160-162).
 *
 * With x_{n+1} = x_n + h, psi_i(n) = x_{n+1} - x_{n-i} = h + psi_{i-1}(n-1), beta_0 = 1,
 * beta_i = beta_{i-1} psi_{i-1}(n) / psi_{i-1}(n-1), and the Adams weights g_j = c_j(1) from
 * c_0(q) = 1/q, c_j(q) = c_{j-1}(q) - c_{j-1}(q+1) h / psi_{j-1}(n):
 *   predict  y^p = y_n + h sum_{j<k} g_j beta_j Phi_j(n)                      (order k)
 *   evaluate f^p = f(y^p);  Phi^p_k = f^p - sum_{j<k} beta_j Phi_j(n)
 *   correct  y_{n+1} = y^p + h g_k Phi^p_k                                     (order k+1)
 *   error    h (g_k - g_{k-1}) Phi^p_k, RMS-scaled as for Tsit5
 *   evaluate f_{n+1} = f(y_{n+1}) (accepted steps); Phi_0(n+1) = f_{n+1},
 *            Phi_{j+1}(n+1) = Phi_j(n+1) - beta_j Phi_j(n)
 * The order starts at 1 and rises by one per accepted step up to 5; three rejections in a row
 * restart it at 1. Step factor 0.8 EEst^(-1/(k+1)) within [0.2, 2] (at most 0.8 on rejection). */
#define ABM_KMAX 5
#define ABM_QMAX 2.0     /* step growth per accepted step */
#define ABM_QMIN 0.2
#define ABM_GAM 0.8      /* safety factor (0.9 rejected 24 % of the steps of a 50-year fault run, 0.8 8 %) */
#define ABM_RESTART 3    /* consecutive rejections that restart the order at 1 */
void orc_abm_coefficients(int k, double h, const double* psi_prev, double* psi, double* beta, double* g) {
    psi[0] = h;
    for (int i = 1; i < k; ++i) psi[i] = h + psi_prev[i - 1];
    beta[0] = 1.0;
    for (int i = 1; i < k; ++i) beta[i] = beta[i - 1] * psi[i - 1] / psi_prev[i - 1];
    double c[ABM_KMAX + 3] = {0};
    for (int q = 1; q <= k + 1; ++q) c[q] = 1.0 / q;
    g[0] = c[1];
    for (int j = 1; j <= k; ++j) {
        const double r = h / psi[j - 1];
        for (int q = 1; q <= k + 1 - j; ++q) c[q] = c[q] - c[q + 1] * r;
        g[j] = c[1];
    }
}

static int abm_integrate(const orc_model* m, double* u, double t0, double t1, const orc_solver_opts* o,
                         orc_solver_stats* stt, int stride, long long max_records, double* t_out, double* u_out,
                         long long* nrec) {
    const long long n = orc_state_len(m, o->mantle);
    double* phi[ABM_KMAX + 1];
    for (int j = 0; j <= ABM_KMAX; ++j) phi[j] = (double*)calloc((size_t)n, sizeof(double));
    double* yp = (double*)malloc(sizeof(double) * n);
    double* fp = (double*)malloc(sizeof(double) * n);
    double* sv = (double*)malloc(sizeof(double) * n);
    double* yn = (double*)malloc(sizeof(double) * n);
    const double qmin = ABM_QMIN, qmax = ABM_QMAX, gam = ABM_GAM;
    double psi_prev[ABM_KMAX] = {0}, psi[ABM_KMAX + 1], beta[ABM_KMAX + 1], g[ABM_KMAX + 2];
    int k = 1, fails = 0, status = 0;
    double t = t0, h = o->dt0;
    long long it = 0, rec = 0;
    memset(stt, 0, sizeof(*stt));
    rhs_flat(m, o->mantle, u, phi[0]);
    stt->nrhs = 1;
    if (stride > 0 && rec < max_records) {
        t_out[rec] = t;
        memcpy(u_out + rec * n, u, sizeof(double) * n);
        ++rec;
    }
    while (t < t1) {
        if (it++ >= o->maxiters) { status = -2; break; }
        if (h > o->dtmax) h = o->dtmax;
        if (t + h > t1) h = t1 - t;
        orc_abm_coefficients(k, h, psi_prev, psi, beta, g);
        for (long long i = 0; i < n; ++i) {
            double s = 0.0, acc = 0.0;
            for (int j = 0; j < k; ++j) {
                const double pj = beta[j] * phi[j][i];
                s += pj;
                acc += g[j] * pj;
            }
            sv[i] = s;
            yp[i] = u[i] + h * acc;
        }
        rhs_flat(m, o->mantle, yp, fp);
        stt->nrhs += 1;
        double ss = 0.0;
        int finite = 1;
        const double ce = h * (g[k] - g[k - 1]);
        for (long long i = 0; i < n; ++i) {
            const double pk = fp[i] - sv[i];
            yn[i] = yp[i] + h * g[k] * pk;
            const double sc = o->abstol + o->reltol * fmax(fabs(u[i]), fabs(yn[i]));
            const double r = ce * pk / sc;
            ss += r * r;
            if (!isfinite(yn[i])) finite = 0;
        }
        double EEst = sqrt(ss / (double)n);
        if (!finite || !isfinite(EEst)) EEst = INFINITY;
        const double fac = gam * pow(EEst, -1.0 / (k + 1));
        if (EEst <= 1.0) {
            t += h;
            memcpy(u, yn, sizeof(double) * n);
            rhs_flat(m, o->mantle, u, fp);  /* f_{n+1} */
            stt->nrhs += 1;
            for (long long i = 0; i < n; ++i) {
                double nw = fp[i];
                for (int j = 0; j < k; ++j) {
                    const double old = phi[j][i];
                    phi[j][i] = nw;
                    nw = nw - beta[j] * old;
                }
                phi[k][i] = nw;
            }
            for (int i = 0; i < k; ++i) psi_prev[i] = psi[i];
            h = h * fmin(qmax, fmax(qmin, fac));
            if (k < ABM_KMAX) ++k;
            fails = 0;
            stt->naccept++;
            if (stride > 0 && stt->naccept % stride == 0 && rec < max_records) {
                t_out[rec] = t;
                memcpy(u_out + rec * n, u, sizeof(double) * n);
                ++rec;
            }
        } else {
            h = h * fmax(qmin, fmin(gam, isfinite(fac) ? fac : qmin));
            if (++fails >= ABM_RESTART) k = 1;
            stt->nreject++;
        }
        if (h < o->dtmin) { status = -1; break; }
    }
    stt->t = t;
    stt->dt = h;
    stt->status = status;
    if (nrec) *nrec = rec;
    for (int j = 0; j <= ABM_KMAX; ++j) free(phi[j]);
    free(yp); free(fp); free(sv); free(yn);
    return status;
}

int orc_integrate_record(const orc_model* m, double* u, double t0, double t1, const orc_solver_opts* o,
                         orc_solver_stats* stt, int stride, long long max_records, double* t_out,
                         double* u_out, long long* nrec) {
    if (o->alg == 1) return abm_integrate(m, u, t0, t1, o, stt, stride, max_records, t_out, u_out, nrec);
    const long long n = orc_state_len(m, o->mantle);
    double* k[7];
    for (int s = 0; s < 7; ++s) k[s] = (double*)malloc(sizeof(double) * n);
    double* y = (double*)malloc(sizeof(double) * n);
    double* un = (double*)malloc(sizeof(double) * n);
    /* PI controller parameters for a 5th-order pair: beta2 = 2/(5*5), beta1 = 7*beta2/4 */
    const double beta2 = 0.08, beta1 = 0.14, gam = 0.9, qmin = 0.2, qmax = 10.0;
    double qold = 1e-4;
    double t = t0, dt = o->dt0;
    long long it = 0;
    int status = 0;
    memset(stt, 0, sizeof(*stt));
    rhs_flat(m, o->mantle, u, k[0]);
    stt->nrhs = 1;
    long long rec = 0;
    if (stride > 0 && rec < max_records) {
        t_out[rec] = t;
        memcpy(u_out + rec * n, u, sizeof(double) * n);
        ++rec;
    }
    while (t < t1) {
        if (it++ >= o->maxiters) { status = -2; break; }
        if (dt > o->dtmax) dt = o->dtmax;
        if (t + dt > t1) dt = t1 - t;
        for (int s = 1; s < 7; ++s) {
            for (long long i = 0; i < n; ++i) {
                double acc = 0.0;
                for (int r = 0; r < s; ++r) acc += TA[s][r] * k[r][i];
                y[i] = u[i] + dt * acc;
            }
            if (s == 6) memcpy(un, y, sizeof(double) * n);
            rhs_flat(m, o->mantle, y, k[s]);
        }
        stt->nrhs += 6;
        double ss = 0.0;
        int finite = 1;
        for (long long i = 0; i < n; ++i) {
            double e = 0.0;
            for (int s = 0; s < 7; ++s) e += TE[s] * k[s][i];
            e *= dt;
            double sc = o->abstol + o->reltol * fmax(fabs(u[i]), fabs(un[i]));
            double r = e / sc;
            ss += r * r;
            if (!isfinite(un[i])) finite = 0;
        }
        double EEst = sqrt(ss / (double)n);
        if (!finite || !isfinite(EEst)) EEst = INFINITY;
        double q11 = pow(EEst, beta1);
        if (EEst <= 1.0) {
            double q = q11 / pow(qold, beta2);
            q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gam));
            t += dt;
            memcpy(u, un, sizeof(double) * n);
            double* tmp = k[0]; k[0] = k[6]; k[6] = tmp;   /* FSAL */
            qold = fmax(EEst, 1e-4);
            dt = dt / q;
            stt->naccept++;
            if (stride > 0 && stt->naccept % stride == 0 && rec < max_records) {
                t_out[rec] = t;
                memcpy(u_out + rec * n, u, sizeof(double) * n);
                ++rec;
            }
        } else {
            double q = isfinite(q11) ? fmin(1.0 / qmin, q11 / gam) : 1.0 / qmin;
            dt = dt / q;
            stt->nreject++;
        }
        if (dt < o->dtmin) { status = -1; break; }
    }
    stt->t = t;
    stt->dt = dt;
    stt->status = status;
    if (nrec) *nrec = rec;
    for (int s = 0; s < 7; ++s) free(k[s]);
    free(y); free(un);
    return status;
}
