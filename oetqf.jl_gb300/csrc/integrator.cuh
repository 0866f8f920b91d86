// Device-resident adaptive integration of one model: Tsit5 or VCABM5.
#pragma once
#include <cuda_runtime.h>

#include "rhs.cuh"

namespace gbc {

// Solver state kept in device memory so whole steps run without the host.
struct Ctrl {
    double t, dt, t1, qold;
    double reltol, abstol, dtmax, dtmin;
    long long naccept, nreject, nrhs, iters, maxiters;
    int done, status, accept, log_theta;
    unsigned int blocks_done;
    long long th_lo, th_hi;  // θ slot of the state; holds ψ = ln θ when log_theta
    // VCABM5 (alg 1): current order k, order of the step in flight kq, consecutive rejections,
    // psi of the last accepted step, this step's psi / beta / Adams weights g, and skip2 = no
    // evaluation at the corrected point (rejected or finished)
    int alg, k, kq, fails, skip2;
    double psi_prev[5], psi[6], beta[6], g[7];
    // recording (wsolve-style): every stride-th accepted step into a device ring of ring_cap slots
    int stride, record;
    long long nrec, ring_cap;
    double* t_ring;
    double* u_ring;
};

// host side of a recording: records are drained from the ring after each graph launch
struct Recorder {
    int stride = 0;
    long long max_records = 0, drained = 0;
    double* t_out = nullptr;   // host
    double* u_out = nullptr;   // host, max_records x n
};

struct Integrator {
    long long n = 0;
    double* k[7] = {};   // stage derivatives
    double* y = nullptr; // stage state
    double* un = nullptr;
    double* partial = nullptr;  // per-block error partial sums
    Ctrl* ctrl = nullptr;       // device
    Ctrl* ctrl_host = nullptr;  // pinned mirror
    int err_blocks = 0;
    cudaGraphExec_t step_exec = nullptr;  // captured group of steps
    int steps_per_launch = 0;
    long long graph_launches = 0;  // graph launches of the last run
    double* t_ring = nullptr;      // device ring of the recorder (ring_cap slots)
    double* u_ring = nullptr;
    long long ring_cap = 0;
    double* phi[6] = {};  // VCABM: modified divided differences Phi_0..Phi_5 (allocated on first use)
};

// Ctrl at the start of an integration from t0 to t1 (VCABM5 starts at order 1; done when t1 <= t0)
inline Ctrl ctrl_start(int alg, double t0, double t1, double reltol, double abstol, double dt0, double dtmax,
                       double dtmin, long long maxiters) {
    Ctrl h{};
    h.alg = alg;
    h.k = 1;
    h.t = t0;
    h.t1 = t1;
    h.dt = dt0 < dtmax ? dt0 : dtmax;
    if (h.dt > t1 - t0) h.dt = t1 - t0;
    h.qold = 1e-4;
    h.reltol = reltol;
    h.abstol = abstol;
    h.dtmax = dtmax;
    h.dtmin = dtmin;
    h.maxiters = maxiters;
    h.done = (t1 <= t0) ? 1 : 0;
    return h;
}

int integrator_alloc(Integrator& I, long long n);
void integrator_free(Integrator& I);
// Integrates u (device) from t0 to t1 with Tsit5 (alg 0) or VCABM5 (alg 1). Fills the host mirror
// of Ctrl.
int integrator_run(Integrator& I, const RhsArgs& rhs, double* u, double t0, double t1,
                   double reltol, double abstol, double dt0, double dtmax, double dtmin,
                   long long maxiters, cudaStream_t s, Recorder* rec = nullptr, int alg = 0);

}  // namespace gbc
