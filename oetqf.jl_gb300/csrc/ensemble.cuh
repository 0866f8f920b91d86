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
    const double *boa, *iL;                  // b/a and 1/L per patch (the ln θ friction path)
    double* u;                               // state (v, θ-or-ψ, δ), 3N
    double* k[7];                            // stage derivatives, 3N each
    double* y;                               // stage state
    double* un;                              // candidate state
    double eta, vpl, f0, v0;
    double t, dt, t1, qold;
    long long naccept, nreject, iters, maxiters;
    int status, done, started, logged;  // logged: θ slot holds ln θ during this integration
    int abm_k, abm_fails;                // VCABM5: order (0 = start at 1) and consecutive rejections
    double psi_prev[5];                  // VCABM5: psi of the last accepted step
};

struct EnsArgs {
    EnsModel* models;
    int nmodels;
    const int* order;            // models of this launch, grouped by cluster size: order[first + i]
    int first;
    int alg;                     // 0: Tsit5, 1: VCABM5                    // per model: stop flag of the current step (written by rank 0)
    double reltol, abstol, dtmax, dtmin;
    int budget;                      // step cap per launch and model
    unsigned long long budget_ns;    // wall-clock budget per launch (all models stay busy until done)
    int gsm;                         // 1: each CTA copies its model's spectra into shared memory
};


// sizes, FFT length and shared-memory need of one model (descriptor zeroed first)
int ens_prepare_model(EnsModel& m, int nx, int nxi, size_t* smem_bytes);
size_t ens_ghat_floats(const EnsModel& m);
// real spectra of the model's circulant kernels from its real Toeplitz kernel (device)
int ens_ghat(const double* st_dev, const EnsModel& m, float* ghat_dev, cudaStream_t s);
// cluster sizes 1, 2, 4, 8 and 16 CTAs (16 is a non-portable size, used only where it can launch)
constexpr int kEnsGroups = 5;
// Models are grouped by cluster size (1, 2, 4 or 8 CTAs per model, from the patch count); each
// group is one persistent cluster launch on its own stream, forked from and joined to `main`.
struct EnsLaunch {
    EnsModel* models = nullptr;
    int n = 0, cap = 0;
    const int* order = nullptr;  // device: model indices grouped by cluster size
    int first[kEnsGroups] = {0, 0, 0, 0, 0}, count[kEnsGroups] = {0, 0, 0, 0, 0};
    cudaStream_t aux[kEnsGroups] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[kEnsGroups] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};
// cluster size of a model of N patches: by size, at least `boost`, at most maxc
int ens_csize(int N, int maxc, int boost);
// the cluster size every model may use when nactive models share the SMs (1, 2, ... up to maxb)
int ens_boost(int nactive, int maxb = 8);
double ens_step_us(int N, int c);
void ens_plan(int n, const int* N, const int* done, const double* left, const double cap[kEnsGroups], int* w);
int ens_max_clusters(int csize, int block, size_t smem, int alg);
// whether 16-CTA clusters of the 512-thread ensemble kernel with smem bytes of shared memory each
// can be resident (non-portable cluster size; sets the kernel attribute that allows it)
bool ens_cluster16_ok(size_t smem, int alg);
int ens_launch_create(EnsLaunch& L, int capacity);
void ens_launch_destroy(EnsLaunch& L);
// groups the models of `host` that are not done (uploads their order); want (host, may be null)
// gives each model's cluster size instead of the size rule
int ens_launch_prepare(EnsLaunch& L, EnsModel* d_models, const EnsModel* host, int n, int maxc, int boost,
                       cudaStream_t s, const int* want = nullptr);
// one persistent launch per group: each model runs until done or budget_ns of wall clock
// gbytes > 0: the largest model's spectra in bytes; when every CTA of the grouping gets an SM to
// itself and the spectra fit beside the FFT buffers, the launches stage them in shared memory
// prioritize: 0 default stream priority; 1 larger clusters at higher priority (the ensemble
// alone on the GPU); 2 every group at the greatest priority (a server's batch beside other work)
int ens_run_groups(const EnsLaunch& L, double reltol, double abstol, double dtmax, double dtmin,
                   unsigned long long budget_ns, int block, size_t smem, cudaStream_t main, int alg = 0,
                   size_t gbytes = 0, int prioritize = 0);
// θ <-> ln θ on the state of every descriptor with `logged` set
int ens_theta(EnsModel* d_models, int n, int to_log, cudaStream_t s);
void count_launches(long long n);

}  // namespace gbc
