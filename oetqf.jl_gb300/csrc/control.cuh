// Step control shared by the single-model integrator and the shared-geometry sweep: the Tsit5
// tableau, the PI controller of the 5(4) pair, and the VCABM5 coefficients and controller. Each
// function updates one Ctrl from its error estimate; the per-element stage arithmetic stays in
// the kernels that own the state.
#pragma once
#include <cuda_runtime.h>

#include "integrator.cuh"

namespace gbc {

// Tsitouras (2011) 5(4): stage coefficients a[s][r] and the error weights b - b̂
static __constant__ double c_ta[7][6] = {
    {0},
    {0.161},
    {-0.008480655492356989, 0.335480655492357},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
static __constant__ double c_te[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                                      -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                                      0.015151515151515152};

// Tsit5 accept/reject and next dt from the RMS error norm EEst of the step just taken (c->dt)
__device__ __forceinline__ void tsit5_control(Ctrl* c, double EEst) {
    const double dt = c->dt;
    if (!isfinite(EEst)) EEst = INFINITY;
    // PI controller for a 5th-order pair: beta1 = 7/50, beta2 = 2/25, safety 0.9, q in [1/10, 5]
    const double beta1 = 0.14, beta2 = 0.08, gam = 0.9, qmin = 0.2, qmax = 10.0;
    const double q11 = pow(EEst, beta1);
    c->iters += 1;
    c->nrhs += 6;
    double dtn;
    if (EEst <= 1.0) {
        double q = q11 / pow(c->qold, beta2);
        q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gam));
        const double tn = c->t + dt;
        c->t = (tn >= c->t1) ? c->t1 : tn;
        c->qold = fmax(EEst, 1e-4);
        c->naccept += 1;
        c->accept = 1;
        c->record = (c->stride > 0 && c->naccept % c->stride == 0) ? 1 : 0;
        dtn = dt / q;
    } else {
        const double q = isfinite(q11) ? fmin(1.0 / qmin, q11 / gam) : 1.0 / qmin;
        c->nreject += 1;
        c->accept = 0;
        dtn = dt / q;
    }
    if (c->t >= c->t1) {
        c->done = 1;
        c->status = 0;
    } else if (dtn < c->dtmin || !isfinite(dtn)) {
        c->done = 1;
        c->status = -5;
    } else if (c->iters >= c->maxiters) {
        c->done = 1;
        c->status = -5;
    }
    if (dtn > c->dtmax) dtn = c->dtmax;
    const double rem = c->t1 - c->t;
    if (dtn >= rem) dtn = rem;
    c->dt = dtn;
}

// ---- VCABM5 ---------------------------------------------------------------------------------------
// Krogh's modified divided differences (Hairer, Norsett & Wanner, Solving ODEs I, sec. III.5;
// Shampine & Gordon 1975). With x_{n+1} = x_n + h: psi_i = x_{n+1} - x_{n-i} = h + psi_{i-1}(prev),
// beta_0 = 1, beta_i = beta_{i-1} psi_{i-1} / psi_{i-1}(prev), g_j = c_j(1) from c_0(q) = 1/q,
// c_j(q) = c_{j-1}(q) - c_{j-1}(q+1) h / psi_{j-1}. Predict y^p = y + h sum_{j<k} g_j beta_j Phi_j,
// evaluate f^p, correct y_{n+1} = y^p + h g_k (f^p - sum_{j<k} beta_j Phi_j), error
// h (g_k - g_{k-1}) (f^p - sum beta_j Phi_j); an accepted step evaluates f_{n+1} and updates
// Phi_0 = f_{n+1}, Phi_{j+1} = Phi_j(new) - beta_j Phi_j(old). The order rises by one per accepted
// step up to 5 and restarts at 1 after three rejections in a row.
constexpr int kAbmMax = 5;

// this step's psi, beta and Adams weights g for the current order k and step h = c->dt
__device__ __forceinline__ void abm_coef(Ctrl* c) {
    const int k = c->k;
    const double h = c->dt;
    c->kq = k;
    c->psi[0] = h;
    for (int i = 1; i < k; ++i) c->psi[i] = h + c->psi_prev[i - 1];
    c->beta[0] = 1.0;
    for (int i = 1; i < k; ++i) c->beta[i] = c->beta[i - 1] * c->psi[i - 1] / c->psi_prev[i - 1];
    double cq[kAbmMax + 3] = {0};
    for (int q = 1; q <= k + 1; ++q) cq[q] = 1.0 / q;
    c->g[0] = cq[1];
    for (int j = 1; j <= k; ++j) {
        const double r = h / c->psi[j - 1];
        for (int q = 1; q <= k + 1 - j; ++q) cq[q] = cq[q] - cq[q + 1] * r;
        c->g[j] = cq[1];
    }
}

// VCABM5 accept/reject, order and next dt from the RMS error norm EEst of the step of order kq
__device__ __forceinline__ void abm_control(Ctrl* c, double EEst) {
    const int k = c->kq;
    const double h = c->dt;
    if (!isfinite(EEst)) EEst = INFINITY;
    const double qmin = 0.2, qmax = 2.0, gam = 0.8;
    const double fac = gam * pow(EEst, -1.0 / (k + 1));
    c->iters += 1;
    c->nrhs += 1;
    double dtn;
    if (EEst <= 1.0) {
        const double tn = c->t + h;
        c->t = (tn >= c->t1) ? c->t1 : tn;
        c->accept = 1;
        c->skip2 = 0;
        c->nrhs += 1;
        c->naccept += 1;
        c->record = (c->stride > 0 && c->naccept % c->stride == 0) ? 1 : 0;
        for (int i = 0; i < k; ++i) c->psi_prev[i] = c->psi[i];
        if (c->k < kAbmMax) c->k += 1;
        c->fails = 0;
        dtn = h * fmin(qmax, fmax(qmin, fac));
    } else {
        c->accept = 0;
        c->skip2 = 1;
        c->nreject += 1;
        if (++c->fails >= 3) c->k = 1;
        dtn = h * fmax(qmin, fmin(gam, isfinite(fac) ? fac : qmin));
    }
    if (c->t >= c->t1) {
        c->done = 1;
        c->status = 0;
    } else if (dtn < c->dtmin || !isfinite(dtn) || c->iters >= c->maxiters) {
        c->done = 1;
        c->status = -5;
    }
    if (dtn > c->dtmax) dtn = c->dtmax;
    const double rem = c->t1 - c->t;
    if (dtn >= rem) dtn = rem;
    c->dt = dtn;
}

}  // namespace gbc
