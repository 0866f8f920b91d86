/*
 * gbcycle -- C ABI of the GB300 earthquake-cycle hot path (libgbcycle.so).
 *
 * The library replaces, behind a plain C boundary, what the reference Oetqf.jl v0.3.6 computes
 * on this path: the stress Green's functions (src/BEM/GF.jl) and the ODE right-hand side that
 * OrdinaryDiffEq calls millions of times (src/BEM/equation.jl), plus an on-device adaptive
 * integrator. Every entry point returns 0 on success or a negative GBC_E* code; the message of
 * the last failure on the calling thread is available from gbc_last_error(). There is no CPU
 * fallback: without a CUDA device every entry point that needs one fails with GBC_ENODEV.
 *
 * Arrays cross the boundary as plain pointers in the reference's Julia (column-major) layouts
 * unless stated otherwise. "_dev" variants take device pointers (same CUDA context as the
 * caller's, e.g. torch tensors on cuda:0) and run on the model's stream.
 */
#ifndef GBCYCLE_H
#define GBCYCLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBC_OK 0
#define GBC_EINVAL -1     /* bad argument (the reference raises AssertionError/ArgumentError) */
#define GBC_ENODEV -2     /* no usable CUDA device */
#define GBC_ECUDA -3      /* CUDA runtime error */
#define GBC_ENOMEM -4     /* device allocation failed or HBM budget exceeded */
#define GBC_ESOLVER -5    /* integration failed (dt below dtmin, maxiters, non-finite state) */
#define GBC_ESTATE -6     /* model not ready (missing Green's functions or properties) */

#define GBC_STRIKE_SLIP 0 /* StrikeSlip() (src/BEM/GF.jl:4) */
#define GBC_DIP_SLIP 1    /* DipSlip()    (src/BEM/GF.jl:5) */

/* RectOkadaMesh (src/BEM/mesh.jl:5-21). ax is (nx,2) and axi is (nxi,2), row-major (lo, hi). */
typedef struct gbc_fault_mesh {
    int nx, nxi;
    const double *x, *xi, *y, *z;
    const double *ax, *axi;
    double dx, dxi, dep, dip;
} gbc_fault_mesh;

/* BEMHex8Mesh (src/BEM/mesh.jl:58-72); the rotation field is unused by the reference's GFs. */
typedef struct gbc_hex_mesh {
    int ne;
    const double *cx, *cy, *cz, *qx, *qy, *qz, *dx, *dy, *dz;
} gbc_hex_mesh;

/* ---- Green's functions ------------------------------------------------------------------- */

/* stress_greens_function(mesh::RectOkadaMesh, λ, μ; ftype, fourier, nrept, buffer_ratio)
 * (src/BEM/GF.jl:31-71). out: real (nx,nxi,nxi) when fourier == 0, else complex interleaved
 * (re,im) (nx,nxi,nxi) -- the rFFT of the circulant embedding (GF.jl:60-67). Host pointer. */
int gbc_stress_gf_ff(const gbc_fault_mesh* mf, double lambda, double mu, int ftype, int fourier,
                     int nrept, double buffer_ratio, double* out);

/* stress_greens_function(mf, ma, λ, μ; ftype, qtype, nrept, buffer_ratio) (GF.jl:123-174).
 * qcoords: 3*nq local coordinates in [-1,1]^3, qweights: nq normalised weights ("Gauss1" is
 * one point at 0 with weight 1). out: (6ne, nx*nxi) column-major. Host pointer. */
int gbc_stress_gf_fm(const gbc_fault_mesh* mf, const gbc_hex_mesh* ma, double lambda, double mu,
                     int ftype, const double* qcoords, const double* qweights, int nq, int nrept,
                     double buffer_ratio, double* out);

/* stress_greens_function(ma, mf, λ, μ; ftype) (GF.jl:194-227). out: (nx*nxi, 6ne) col-major. */
int gbc_stress_gf_mf(const gbc_hex_mesh* ma, const gbc_fault_mesh* mf, double lambda, double mu,
                     int ftype, double* out);

/* stress_greens_function(ma, λ, μ; qtype) (GF.jl:250-290, without the eigvals print).
 * out: (6ne, 6ne) column-major. */
int gbc_stress_gf_mm(const gbc_hex_mesh* ma, double lambda, double mu, const double* qcoords,
                     const double* qweights, int nq, double* out);
/* No reference counterpart: whether a mantle mesh is a complete grid of equal cells (centres on
 * uniform x and y grids spaced by the cell size, any set of depths, equal source-corner offsets),
 * which the mantle-mantle assembly evaluates once per (horizontal offset, layer pair) instead of
 * once per cell pair. Returns 1 (and the grid size in nX, nY, nZ) or 0; host-only, no device use. */
int gbc_hex_mesh_grid(const gbc_hex_mesh* ma, int* nX, int* nY, int* nZ);

/* ---- Models: the ODEProblem parameter tuple of assemble (src/BEM/equation.jl:81-89,141-154) -- */

typedef struct gbc_model gbc_model;

#define GBC_PREC_F64 0    /* Green's functions stored and applied in FP64 */
#define GBC_PREC_BF16 1   /* block-scaled BF16 storage (128x128 FP32 scales), FP32 accumulate */
#define GBC_PREC_F16 2    /* block-scaled FP16 storage (128x128 FP32 scales), FP32 accumulate */
#define GBC_PREC_DF64 3   /* FP64-accurate double-float: each entry as an FP32 pair hi + lo, compensated
                             FP32 products and sums (relative error ~1e-14), FP64 results */

/* A model with nx*nxi fault patches and ne mantle cells (ne = 0: fault-only, equation.jl:156-166;
 * ne > 0: viscoelastic, equation.jl:185-205). Allocates device buffers; owns one CUDA stream. */
int gbc_model_create(int nx, int nxi, int ne, gbc_model** out);
void gbc_model_destroy(gbc_model* m);

/* RateStateQuasiDynamicProperty (src/BEM/property.jl:10-25); a, b, L, sigma are (nx,nxi). */
int gbc_model_set_fault_props(gbc_model* m, const double* a, const double* b, const double* L,
                              const double* sigma, double eta, double vpl, double f0, double v0);
/* PowerLawViscosityProperty (src/BEM/property.jl:34-41): gamma, n (= power - 1) of length ne and
 * deps0 of length 6 (xx, xy, xz, yy, yz, zz). */
int gbc_model_set_mantle_props(gbc_model* m, const double* gamma, const double* n,
                               const double* deps0);
/* CompositePowerLawViscosityProperty (src/BEM/property.jl:43-48, equation.jl:286-292): nlaws
 * power laws summed; gamma and n are (ne, nlaws) column-major (law k at offset k*ne). */
int gbc_model_set_mantle_props_composite(gbc_model* m, int nlaws, const double* gamma,
                                         const double* n, const double* deps0);
/* DilatancyProperty (src/BEM/property.jl:27-32) for a fault-only model: the ode becomes
 * equation.jl:168-183 with update_fault_with_dilatancy! (:248-276) and d𝓅_dt (:282); the state is
 * (v, θ, δ, 𝓅), four (nx,nxi) parts. tp, eps, beta, p0 are (nx,nxi). FP64 path. */
int gbc_model_set_dilatancy(gbc_model* m, const double* tp, const double* eps, const double* beta,
                            const double* p0);

#define GBC_GF11_REAL 0   /* (nx,nxi,nxi) real Toeplitz kernel */
#define GBC_GF11_DFT 1    /* (nx,nxi,nxi) complex interleaved, the reference's fourier=true form */
#define GBC_GF12 2        /* (6ne, N) fault -> mantle */
#define GBC_GF21 3        /* (N, 6ne) mantle -> fault */
#define GBC_GF22 4        /* (6ne, 6ne) mantle -> mantle */

/* Upload a Green's function from host memory in the reference layout (the gf₁₁..gf₂₂ arguments
 * of assemble, equation.jl:141-149). */
int gbc_model_set_gf(gbc_model* m, int which, const double* host);
/* Assemble every Green's function of the model directly on the device (no host round trip).
 * ma may be NULL for a fault-only model. */
int gbc_model_assemble(gbc_model* m, const gbc_fault_mesh* mf, const gbc_hex_mesh* ma,
                       double lambda, double mu, int ftype, int nrept, double buffer_ratio,
                       const double* qcoords, const double* qweights, int nq);
/* Copy a Green's function back to host memory in the reference layout (parity checks). */
int gbc_model_export_gf(gbc_model* m, int which, double* host);
/* Copy chosen rows of GBC_GF12, GBC_GF21 or GBC_GF22 to host memory: rows[k] is a row of the
 * reference layout (k*ne + j for stress component k at cell j; patch i for GF21), and host receives
 * nrows x (number of columns) doubles, row by row. For checking entries of large models (the
 * full 6ne x 6ne block of an 8000-cell mantle is 18 GB) without a full export. */
int gbc_model_export_gf_rows(gbc_model* m, int which, int nrows, const int* rows, double* host);
/* Storage precision of the mantle Green's functions (GBC_PREC_*); FP64 by default. BF16/FP16
 * store [G12|G22] and G21 as one 16-bit matrix with an FP32 scale per 128x128 block and
 * accumulate in FP32; the fault-fault kernel runs in FP32 and friction stays FP64. The 16-bit
 * copy is rebuilt from the FP64 Green's functions whenever they change. DF64 stores the same
 * rows as FP32 pairs (hi = fl32(g), lo = fl32(g - hi): the same 8 bytes per entry as FP64) and
 * runs the dot products on the FP32 pipe with error-free transformations (TwoProduct by FMA,
 * TwoSum), so the result keeps ~48 significant bits; the fault-fault sum and friction stay FP64.
 * Entries and rates must lie inside FP32's normal range (1e-38 .. 3e38) for the full accuracy. */
int gbc_model_set_precision(gbc_model* m, int mode);
/* Integrate ψ = ln θ instead of θ inside gbc_integrate* (the caller's state keeps θ). */
int gbc_model_set_log_theta(gbc_model* m, int on);
/* Device error word of the model's bounded waits (0 = none); nonzero means a TMA pipeline wait
 * timed out and the last right-hand side is not valid. */
int gbc_model_error_word(gbc_model* m);
/* Resets the error word to 0 (after the caller has handled a timeout). */
int gbc_model_clear_error_word(gbc_model* m);

/* ode(du, u, p, t) (equation.jl:156-166 / 168-183 / 185-205) on host buffers in ArrayPartition
 * order: nparts = 3: (v, θ, δ), each (nx,nxi); 4 with dilatancy: (v, θ, δ, 𝓅);
 * 5: (v, θ, ϵ, σ, δ), ϵ and σ (ne,6). */
int gbc_rhs(gbc_model* m, double t, const double* const* u_parts, double* const* du_parts,
            int nparts);
/* Same on device memory: u and du are the flat concatenation of the parts (length
 * gbc_model_state_len). Runs on the model's stream and does not synchronise. */
int gbc_rhs_dev(gbc_model* m, double t, const double* u, double* du);
long long gbc_model_state_len(const gbc_model* m);

/* ---- On-device adaptive integration (stands in for OrdinaryDiffEq's solve, src/io.jl:125-130) */

#define GBC_ALG_TSIT5 0   /* Tsitouras 5(4), PI step control (the reference's tests) */
#define GBC_ALG_VCABM5 1  /* variable-coefficient Adams-Bashforth-Moulton, PECE, orders 1-5 (the
                             reference's example, examples/otf-with-mantle.jl:160-162) */

typedef struct gbc_solver_opts {
    double reltol, abstol;   /* error norm: RMS of err / (abstol + reltol * max(|u|, |u_new|)) */
    double dt0, dtmax, dtmin;
    long long maxiters;
    int alg;                 /* GBC_ALG_TSIT5 (0) or GBC_ALG_VCABM5 (1), for every integrating call */
} gbc_solver_opts;

typedef struct gbc_solver_stats {
    long long naccept, nreject, nrhs;
    double t, dt;
    int status;              /* 0 = reached t1, GBC_ESOLVER otherwise */
} gbc_solver_stats;

/* Tsit5 with PI step control or VCABM5 (opts->alg) from t0 to t1; u (flat, host) is overwritten
 * with u(t1). */
int gbc_integrate(gbc_model* m, double* u, double t0, double t1, const gbc_solver_opts* opts,
                  gbc_solver_stats* stats);
/* gbc_integrate that also records the state history like the reference's wsolve callback
 * (src/io.jl:51-58, :118-133): record 0 is (t0, u0), then (t, u) after every stride-th accepted
 * step, up to max_records (t_out: max_records, u_out: max_records x state_len, host). The device
 * keeps a small ring of recent records that the host drains after each group of steps. */
int gbc_integrate_record(gbc_model* m, double* u, double t0, double t1, const gbc_solver_opts* opts,
                         int stride, long long max_records, double* t_out, double* u_out,
                         long long* nrec, gbc_solver_stats* stats);
/* Same with the state already on the device; does not synchronise the stats until it returns. */
int gbc_integrate_dev(gbc_model* m, double* u_dev, double t0, double t1,
                      const gbc_solver_opts* opts, gbc_solver_stats* stats);

/* Viscoelastic ode(du, u, p, t) (equation.jl:185-205) that allocates no device memory. No
 * counterpart in the reference: it is for callers that cannot call cudaMalloc when they evaluate
 * the right-hand side -- code running while another library captures the stream into a CUDA
 * graph (allocation is not permitted during capture), processes whose device memory is owned by
 * their own pool, and bindings that only pass raw device pointers. Every input and output is the
 * caller's device memory (deps0 excepted: 6 doubles in host memory):
 *   st (nx,nxi,nxi) real Toeplitz kernel, column-major;
 *   gm row-major (6ne rows, leading dim ldm >= npad + 6ne, even): columns [0,N) hold G12,
 *      [N,npad) zeros and [npad, npad+6ne) G22, with N = nx*nxi and npad = N rounded up to 32;
 *   g21 row-major (N rows, leading dim ld21 >= 6ne, even);
 *   gm and g21 start on 16-byte boundaries (rows are read as pairs of doubles; GBC_EINVAL
 *      otherwise, e.g. for a view that starts one double into a larger buffer);
 *   a, b, L, sigma (N), gamma, n (ne); u, du flat states of length 3N + 12ne.
 * The one scratch vector lives in a fixed 8 MiB device array inside the library, so the model
 * must satisfy npad + 6ne <= 1048576 (GBC_EINVAL otherwise). The first call on each device looks
 * the array up (and may load the library's device code): make it before any stream capture.
 * The looked-up address is kept for the life of the process, so do not call this entry point
 * again on a device after cudaDeviceReset on it. All calls share the array: calls whose work
 * overlaps on the GPU race. stream may be NULL. */
int gbc_rhs_visco_noalloc(int nx, int nxi, int ne, const double* st, const double* gm, size_t ldm,
                          const double* g21, size_t ld21, const double* a, const double* b,
                          const double* L, const double* sigma, double eta, double vpl, double f0,
                          double v0, const double* gamma, const double* n, const double* deps0,
                          const double* u, double* du, void* stream);

/* The model's CUDA stream (a cudaStream_t), so callers can order their own work or record
 * CUDA events around the library's launches. */
void* gbc_model_stream(gbc_model* m);

/* ---- Batched ensembles (many independent fault-only models in one persistent launch) -------- */

typedef struct gbc_ensemble gbc_ensemble;

/* nmodels fault-only models of sizes nx[i] x nxi[i] (each model's ODE is equation.jl:156-166).
 * Each model runs on one CTA with its Toeplitz kernel in shared memory (FP32) and its own Tsit5
 * step control; the state, friction and error norm are FP64. nx*nxi*nxi + nx*nxi floats of the
 * largest model must fit in 200 KB. */
int gbc_ensemble_create(int nmodels, const int* nx, const int* nxi, gbc_ensemble** out);
void gbc_ensemble_destroy(gbc_ensemble* e);
/* Per model, as for a single model: the reference's fourier or real fault-fault kernel
 * (GBC_GF11_DFT / GBC_GF11_REAL, src/BEM/GF.jl:31-71), or assembled on the device. */
int gbc_ensemble_set_gf(gbc_ensemble* e, int model, int which, const double* host);
int gbc_ensemble_assemble(gbc_ensemble* e, int model, const gbc_fault_mesh* mf, double lambda,
                          double mu, int ftype, int nrept, double buffer_ratio);
int gbc_ensemble_set_fault_props(gbc_ensemble* e, int model, const double* a, const double* b,
                                 const double* L, const double* sigma, double eta, double vpl,
                                 double f0, double v0);
/* Threads per model CTA (128, 256 or 512; picked by the autotuner in the host package). */
int gbc_ensemble_set_block(gbc_ensemble* e, int threads);
/* Integrate ψ = ln θ internally (default on; the caller's state keeps θ). */
int gbc_ensemble_set_log_theta(gbc_ensemble* e, int on);
/* Largest thread-block cluster per model (1, 2, 4, 8 or 16; default 16). A model on a cluster of
 * CTAs is split over them: each CTA owns a slice of the patches for the friction update, the
 * stages and the error norm, and the CTAs exchange slip rates and error-norm sums through
 * distributed shared memory. 16-CTA clusters are used where that non-portable size can be
 * resident. A model's trajectory does not depend on its cluster or block size (its error norm is
 * summed over fixed 32-patch chunks in a fixed order). */
int gbc_ensemble_set_max_cluster(gbc_ensemble* e, int ctas);
/* Regrouping (default on). Before the first launch and after every launch (about 0.2 s), the
 * models still running are planned onto cluster sizes (gbc_ensemble_plan_clusters, with the
 * occupancy the GPU reports for each size), so that all their CTAs are resident together; the
 * larger clusters launch first, at a higher stream priority. Off: the size rule by patch count
 * (one CTA up to 600 patches, 2 up to 1200, 4 up to 2400, 8 beyond). */
int gbc_ensemble_set_regroup(gbc_ensemble* e, int on);
/* The regrouping plan (host only, no GPU): sizes[i] = the cluster size (1, 2, 4, 8 or 16) for n
 * models of npatch[i] patches, done[i] != 0 for finished ones (size 1), steps_left[i] = the steps
 * left at the current step size (ties only). capacity[g] = how many clusters of 2^g CTAs the GPU
 * holds at once (g = 0..4; 0: that size is not available). Every model starts on one CTA; then,
 * repeatedly, the model with the largest predicted step latency moves to the next size when that
 * saves at least 3 % and the sum over running models of 1 / capacity[log2 size] stays at most 1. */
int gbc_ensemble_plan_clusters(int n, const int* npatch, const int* done, const double* steps_left,
                               const int* capacity, int* sizes);
/* The flat state is the concatenation over models of (v, θ, δ); model i starts at
 * gbc_ensemble_state_offset(e, i). Each model integrates from t0[i] to t1[i]; stats has one entry
 * per model. The _dev variant takes a device pointer. */
long long gbc_ensemble_state_len(const gbc_ensemble* e);
long long gbc_ensemble_state_offset(const gbc_ensemble* e, int model);
int gbc_ensemble_integrate(gbc_ensemble* e, double* u, const double* t0, const double* t1,
                           const gbc_solver_opts* opts, gbc_solver_stats* stats);
int gbc_ensemble_integrate_dev(gbc_ensemble* e, double* u_dev, const double* t0, const double* t1,
                               const gbc_solver_opts* opts, gbc_solver_stats* stats);
void* gbc_ensemble_stream(gbc_ensemble* e);

/* ---- Parameter sweeps on one geometry (tensor-core batched right-hand side) ------------------ */

typedef struct gbc_sweep gbc_sweep;

#define GBC_SWEEP_SIMT 0  /* product on the FP32 pipe, each variant's sums in the single model's order */
#define GBC_SWEEP_UMMA 1  /* product on the tensor cores (tcgen05, BF16 x BF16 -> FP32), the default */

/* nvariants (1..64) copies of a viscoelastic model's ODE (equation.jl:185-205) that share the base
 * model's Green's functions and differ in properties and state -- the reference's way of rerunning
 * one assembled model with other properties (examples/otf-with-mantle.jl:44-56, 140-162) batched on
 * the device. The base model must use GBC_PREC_BF16 with its Green's functions and properties set;
 * each variant starts with the base's properties. One right-hand side applies the block-scaled
 * mantle rows to every variant's state at once: a product with nvariants columns that reads the
 * matrix once. The base must outlive the sweep and keep its Green's functions and precision (the
 * sweep fails with GBC_ESTATE otherwise); the fault must satisfy N + nx*nxi <= 40960. */
int gbc_sweep_create(gbc_model* base, int nvariants, gbc_sweep** out);
void gbc_sweep_destroy(gbc_sweep* s);
/* Properties of variant k (same meaning as gbc_model_set_fault_props / _mantle_props; gamma and n
 * have the base's number of power laws, law-major). */
int gbc_sweep_set_fault_props(gbc_sweep* s, int k, const double* a, const double* b, const double* L,
                              const double* sigma, double eta, double vpl, double f0, double v0);
int gbc_sweep_set_mantle_props(gbc_sweep* s, int k, const double* gamma, const double* n,
                               const double* deps0);
/* GBC_SWEEP_UMMA (default) or GBC_SWEEP_SIMT. */
int gbc_sweep_set_engine(gbc_sweep* s, int engine);
/* Fault rows on the tensor cores too (GBC_SWEEP_UMMA only; default off): the dense fault-fault
 * block is built once as three BF16 planes hi + mid + lo (exact for the FP32 Toeplitz entries,
 * 6 N^2 bytes with N rounded up to 128) and applied to all variants in the tensor-core product,
 * leaving only the FP64 friction per variant. Off: the per-variant FP32 Toeplitz rows. */
int gbc_sweep_set_fault_product(gbc_sweep* s, int on);
/* State length of one variant; states are variant-major (variant k at k * gbc_sweep_state_len). */
long long gbc_sweep_state_len(const gbc_sweep* s);
/* ode(du, u, p, t) for every variant: u, du hold nvariants flat states (host, or device for _dev,
 * which runs on the sweep's stream without synchronising). */
int gbc_sweep_rhs(gbc_sweep* s, const double* u, double* du);
int gbc_sweep_rhs_dev(gbc_sweep* s, const double* u, double* du);
/* Integrates every variant from t0 to t1 with its own step control (opts->alg: Tsit5 or VCABM5);
 * stats has nvariants entries. The variants share each right-hand side evaluation; a variant that
 * reached t1 stops changing while the others continue. */
int gbc_sweep_integrate(gbc_sweep* s, double* u, double t0, double t1, const gbc_solver_opts* opts,
                        gbc_solver_stats* stats);
int gbc_sweep_integrate_dev(gbc_sweep* s, double* u_dev, double t0, double t1,
                            const gbc_solver_opts* opts, gbc_solver_stats* stats);
/* Device error word of the tensor-core pipeline's bounded waits (0 = none). */
int gbc_sweep_error_word(gbc_sweep* s);
void* gbc_sweep_stream(gbc_sweep* s);

/* ---- Serving: continuous batching of cycle-simulation requests on one GPU ------------------ */

typedef struct gbc_server gbc_server;

/* One request: a fault (and optionally a mantle) with its properties, initial state and horizon.
 * Every array is copied at submission. Fault-only requests run in the server's continuous batch
 * with the server's solver options; mantle requests run on their own stream with block-scaled
 * `precision` Green's functions (GBC_PREC_BF16/F16, or F64) and their own options when
 * ne_opts_valid is set. u0 is (v, θ, δ) or (v, θ, ϵ, σ, δ). */
typedef struct gbc_request {
    const gbc_fault_mesh* mf;
    const gbc_hex_mesh* ma;         /* NULL: fault-only */
    double lambda, mu;
    int ftype, nrept;
    double buffer_ratio;
    const double *a, *b, *L, *sigma;
    double eta, vpl, f0, v0;
    const double *gamma, *n, *deps0; /* mantle requests only */
    const double *qcoords, *qweights;
    int nq;
    const double* u0;
    double t0, t1;
    int precision;
    int ne_opts_valid;
    gbc_solver_opts opts;
} gbc_request;

typedef struct gbc_request_result {
    long long id;
    int status;
    double submit_s, admit_s, done_s; /* seconds since the server started */
    gbc_solver_stats stats;
} gbc_request_result;

typedef struct gbc_server_info {
    int queued, batched, mantle;
    double bytes_in_use, peak_bytes;   /* bytes_in_use includes cached Green's functions */
    long long iterations;
    int cache_entries;                 /* assembled geometries resident on the device */
    double cache_bytes;
    long long cache_hits, cache_misses;
} gbc_server_info;

/* A server admitting requests while their estimated device footprint fits hbm_budget_bytes, in
 * arrival order, except that fault-only requests (megabytes) that fit run ahead of a queued
 * request that does not fit yet. A native scheduler thread owns all GPU work. */
int gbc_server_create(double hbm_budget_bytes, const gbc_solver_opts* batch_opts, gbc_server** out);
int gbc_server_submit(gbc_server* s, const gbc_request* req, long long* id);
/* Blocks until request id finishes; writes its final state into u_out (host, may be NULL). */
int gbc_server_wait(gbc_server* s, long long id, double* u_out, gbc_request_result* res);
int gbc_server_query(gbc_server* s, gbc_server_info* out);
/* Green's-function cache across requests (on by default; the serving counterpart of saving and
 * reloading assembled Green's functions, examples/otf-with-mantle.jl:44-56): requests whose mesh,
 * elastic constants, fault type, images, buffer ratio, quadrature and precision equal a cached
 * geometry skip assembly. Idle entries count against the budget and are evicted least recently
 * used first. Turning it off frees the idle entries. */
int gbc_server_set_gf_cache(gbc_server* s, int enabled);
/* Finishes every admitted and queued request, then stops the scheduler. */
void gbc_server_destroy(gbc_server* s);

/* ---- Diagnostics ------------------------------------------------------------------------ */
/* No reference counterpart: failure injection for tests of the bounded waits. mode 1 makes every
 * 16-bit (GBC_PREC_BF16/F16) mantle GEMV launched afterwards on the current device issue no TMA
 * copies and give up each pipeline wait after 1024 polls, so every such right-hand side takes its
 * timeout path: it records the model's error word and returns, with no copy in flight, and its
 * output is not valid. mode 0 (the default) restores normal operation. Not for production use. */
int gbc_debug_pipeline_fault(int mode);
/* No reference counterpart: a throughput probe of the GPU's FP64 FMA pipe, the bound of the FP64
 * row GEMV on this chip. Launches blocks x threads threads (threads a multiple of 32, <= 1024), each
 * running independent FMA chains for iters iterations on `stream`, and writes one double per thread
 * to out_dev (device, blocks*threads doubles). *flops receives the launch's FLOP count (2 per
 * FMA); time the launch with CUDA events on the same stream. Does not synchronise. */
int gbc_probe_fp64_fma(double* out_dev, int blocks, int threads, long long iters, void* stream,
                       double* flops);
int gbc_last_error(char* buf, size_t len);
const char* gbc_version(void);
/* Number of kernels this library launched in this process (used to report GPU launch counts). */
long long gbc_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
