// Batched fault-only models: the per-model descriptor of the persistent ensemble kernel and the
// helpers the serving loop shares with gbc_ensemble.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace gbc {

struct EnsModel {
    int nx, nxi, N, log_theta;
    int P, logP;       // FFT length (power of two >= 2nx - 1) and its log2
    long long off_n;   // patch offset inside a gbc_ensemble's arrays (host bookkeeping)
    long long off_st;
    // device buffers of this model
    const float* ghat;                       // real spectra of the circulant kernels (nxi, nxi, P/2+1)
    const double *a, *b, *L, *sig, *c1;      // friction (N each); c1 = f0/a + (b/a) ln(v0/L) - ln(2 v0)
    double* u;                               // state (v, θ-or-ψ, δ), 3N
    double* k[7];                            // stage derivatives, 3N each
    double* y;                               // stage state
    double* un;                              // candidate state
    double eta, vpl, f0, v0;
    double t, dt, t1, qold;
    long long naccept, nreject, iters, maxiters;
    int status, done, started, logged;  // logged: θ slot holds ln θ during this integration
};

struct EnsArgs {
    EnsModel* models;
    int nmodels;
    double reltol, abstol, dtmax, dtmin;
    int budget;                      // step cap per launch and model
    unsigned long long budget_ns;    // wall-clock budget per launch (all models stay busy until done)
};


// sizes, FFT length and shared-memory need of one model (descriptor zeroed first)
int ens_prepare_model(EnsModel& m, int nx, int nxi, size_t* smem_bytes);
size_t ens_ghat_floats(const EnsModel& m);
// real spectra of the model's circulant kernels from its real Toeplitz kernel (device)
int ens_ghat(const double* st_dev, const EnsModel& m, float* ghat_dev, cudaStream_t s);
// one persistent launch over n device descriptors, each model runs until done or budget_ns
int ens_run(EnsModel* d_models, int n, double reltol, double abstol, double dtmax, double dtmin,
            unsigned long long budget_ns, int block, size_t smem, cudaStream_t s);
// θ <-> ln θ on the state of every descriptor with `logged` set
int ens_theta(EnsModel* d_models, int n, int to_log, cudaStream_t s);
void count_launches(long long n);

}  // namespace gbc
