// Device-resident adaptive integrators standing in for the reference's OrdinaryDiffEq caller
// (src/io.jl:125-130): Tsit5 (Tsitouras 2011, 5(4) pair) with a PI step-size controller, as in the
// reference's tests (test/tests.jl:11), and VCABM5 (variable-coefficient Adams-Bashforth-Moulton
// in PECE mode, orders 1..5), as in the reference's example (examples/otf-with-mantle.jl:160-162).
//
// One step = 6 x (stage combination + RHS) + error norm/controller + commit, all on the device:
// the controller kernel reads the error norm, accepts or rejects, and writes the next dt into
// device memory, so steps chain without host round trips. The host captures a group of steps
// into a CUDA graph and relaunches it until the controller reports completion; launches after
// completion see Ctrl::done and return immediately.
#include <cuda_runtime.h>

#include "gbc_internal.cuh"
#include "control.cuh"
#include "integrator.cuh"

namespace gbc {

struct KPtrs {
    const double* k[7];
};

// y = u + dt * sum_{r < s} a[s][r] k_r
__global__ void k_stage(int s, long long n, const double* __restrict__ u, KPtrs K, double* __restrict__ y,
                        const Ctrl* __restrict__ c) {
    if (c->done) return;
    const double dt = c->dt;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int r = 0; r < s; ++r) acc = fma(c_ta[s][r], K.k[r][i], acc);
        y[i] = u[i] + dt * acc;
    }
}

// error norm partials, then the last block to finish runs the controller
__global__ void k_error_control(long long n, const double* __restrict__ u, const double* __restrict__ un,
                                KPtrs K, double* __restrict__ partial, Ctrl* c) {
    if (c->done) return;
    __shared__ double red[32];
    __shared__ int last;
    const double dt = c->dt, rtol = c->reltol, atol = c->abstol;
    double ss = 0.0;
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double e = 0.0;
#pragma unroll
        for (int s = 0; s < 7; ++s) e = fma(c_te[s], K.k[s][i], e);
        e *= dt;
        const double unv = un[i];
        // with ψ = ln θ an absolute ψ error equals a relative θ error: scale it by reltol
        const double sc = (c->log_theta && i >= c->th_lo && i < c->th_hi) ? atol + rtol
                                                                             : atol + rtol * fmax(fabs(u[i]), fabs(unv));
        const double r = e / sc;
        ss = fma(r, r, ss);
        bad |= !isfinite(unv);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = bad ? INFINITY : ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += red[w];
        partial[blockIdx.x] = b;
        __threadfence();
        const unsigned prev = atomicAdd(&c->blocks_done, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double tot = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) tot += ((volatile double*)partial)[b];
    c->blocks_done = 0;
    tsit5_control(c, sqrt(tot / (double)n));
}

// accept: u <- un and the FSAL derivative k0 <- k6; a recorded step also goes to the ring slot
// nrec % ring_cap (θ restored from ψ when integrating ln θ)
__global__ void k_commit(long long n, double* __restrict__ u, const double* __restrict__ un, double* __restrict__ k0,
                         const double* __restrict__ k6, const Ctrl* __restrict__ c) {
    if (!c->accept) return;
    const bool rec = c->record && c->ring_cap > 0;
    double* ur = rec ? c->u_ring + (c->nrec % c->ring_cap) * n : nullptr;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = un[i];
        u[i] = v;
        k0[i] = k6[i];
        if (rec) ur[i] = (c->log_theta && i >= c->th_lo && i < c->th_hi) ? exp(v) : v;
    }
    if (rec && blockIdx.x == 0 && threadIdx.x == 0) c->t_ring[c->nrec % c->ring_cap] = c->t;
}

// the commit above must not run twice for one accepted step: clear the flag for the next step
// (and advance the ring after every block of k_commit has used the same slot)
__global__ void k_clear_accept(Ctrl* c) {
    if (c->accept && c->record && c->ring_cap > 0) c->nrec += 1;
    c->accept = 0;
    c->record = 0;
}

// ---- VCABM5 (coefficients and controller in control.cuh) --------------------------------------
__global__ void k_abm_coef(Ctrl* c) {
    if (c->done) return;
    abm_coef(c);
}

struct PhiPtrs {
    double* p[kAbmMax + 1];
};

// y^p = u + h sum_{j<k} g_j beta_j Phi_j and sv = sum_{j<k} beta_j Phi_j
__global__ void k_abm_predict(long long n, const double* __restrict__ u, PhiPtrs P, double* __restrict__ yp,
                              double* __restrict__ sv, const Ctrl* __restrict__ c) {
    if (c->done) return;
    const int k = c->kq;
    const double h = c->dt;
    double beta[kAbmMax], g[kAbmMax];
#pragma unroll
    for (int j = 0; j < kAbmMax; ++j) {
        beta[j] = c->beta[j];
        g[j] = c->g[j];
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double sacc = 0.0, acc = 0.0;
#pragma unroll
        for (int j = 0; j < kAbmMax; ++j) {
            if (j < k) {
                const double pj = beta[j] * P.p[j][i];
                sacc += pj;
                acc = fma(g[j], pj, acc);
            }
        }
        sv[i] = sacc;
        yp[i] = u[i] + h * acc;
    }
}

// corrector, error norm partials; the last block to finish runs the step controller
__global__ void k_abm_correct_control(long long n, const double* __restrict__ u, const double* __restrict__ yp,
                                      const double* __restrict__ fp, const double* __restrict__ sv,
                                      double* __restrict__ un, double* __restrict__ partial, Ctrl* c) {
    if (c->done) return;
    __shared__ double red[32];
    __shared__ int last;
    const int k = c->kq;
    const double h = c->dt, rtol = c->reltol, atol = c->abstol;
    const double gk = c->g[k], ce = h * (c->g[k] - c->g[k - 1]);
    double ss = 0.0;
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double pk = fp[i] - sv[i];
        const double yn = yp[i] + h * gk * pk;
        un[i] = yn;
        // with ψ = ln θ an absolute ψ error equals a relative θ error: scale it by reltol
        const double sc = (c->log_theta && i >= c->th_lo && i < c->th_hi) ? atol + rtol
                                                                             : atol + rtol * fmax(fabs(u[i]), fabs(yn));
        const double r = ce * pk / sc;
        ss = fma(r, r, ss);
        bad |= !isfinite(yn);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = bad ? INFINITY : ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += red[w];
        partial[blockIdx.x] = b;
        __threadfence();
        const unsigned prev = atomicAdd(&c->blocks_done, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double tot = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) tot += ((volatile double*)partial)[b];
    c->blocks_done = 0;
    abm_control(c, sqrt(tot / (double)n));
}

// accepted step: u <- y_{n+1}, Phi update with f_{n+1} (fn) and this step's beta, ring record
__global__ void k_abm_commit(long long n, double* __restrict__ u, const double* __restrict__ un,
                             const double* __restrict__ fn, PhiPtrs P, const Ctrl* __restrict__ c) {
    if (!c->accept) return;
    const int k = c->kq;
    double beta[kAbmMax];
#pragma unroll
    for (int j = 0; j < kAbmMax; ++j) beta[j] = c->beta[j];
    const bool rec = c->record && c->ring_cap > 0;
    double* ur = rec ? c->u_ring + (c->nrec % c->ring_cap) * n : nullptr;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = un[i];
        u[i] = v;
        double nw = fn[i];
#pragma unroll
        for (int j = 0; j < kAbmMax; ++j) {
            if (j < k) {
                const double old = P.p[j][i];
                P.p[j][i] = nw;
                nw = nw - beta[j] * old;
            }
        }
        P.p[k][i] = nw;
        if (rec) ur[i] = (c->log_theta && i >= c->th_lo && i < c->th_hi) ? exp(v) : v;
    }
    if (rec && blockIdx.x == 0 && threadIdx.x == 0) c->t_ring[c->nrec % c->ring_cap] = c->t;
}

static int enqueue_abm_step(Integrator& I, const RhsArgs& rhs0, double* u, cudaStream_t s) {
    const long long n = I.n;
    const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 4);
    PhiPtrs P;
    for (int j = 0; j <= kAbmMax; ++j) P.p[j] = I.phi[j];
    double* yp = I.y;
    double* fp = I.k[1];
    double* sv = I.k[2];
    double* fn = I.k[3];
    k_abm_coef<<<1, 1, 0, s>>>(I.ctrl);
    GBC_CUDA(cudaGetLastError());
    k_abm_predict<<<g, 256, 0, s>>>(n, u, P, yp, sv, I.ctrl);
    GBC_CUDA(cudaGetLastError());
    RhsArgs rhs = rhs0;
    rhs.skip = &I.ctrl->done;
    if (int rc = launch_rhs(rhs, yp, fp, s)) return rc;
    k_abm_correct_control<<<I.err_blocks, 256, 0, s>>>(n, u, yp, fp, sv, I.un, I.partial, I.ctrl);
    GBC_CUDA(cudaGetLastError());
    rhs.skip = &I.ctrl->skip2;  // the corrected point is evaluated only for accepted steps
    if (int rc = launch_rhs(rhs, I.un, fn, s)) return rc;
    k_abm_commit<<<g, 256, 0, s>>>(n, u, I.un, fn, P, I.ctrl);
    GBC_CUDA(cudaGetLastError());
    k_clear_accept<<<1, 1, 0, s>>>(I.ctrl);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int integrator_alloc(Integrator& I, long long n) {
    if (I.n == n && I.y) return 0;
    integrator_free(I);
    I.n = n;
    for (int s = 0; s < 7; ++s) GBC_CUDA(cudaMalloc(&I.k[s], sizeof(double) * n));
    GBC_CUDA(cudaMalloc(&I.y, sizeof(double) * n));
    GBC_CUDA(cudaMalloc(&I.un, sizeof(double) * n));
    I.err_blocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 2);
    if (I.err_blocks < 1) I.err_blocks = 1;
    GBC_CUDA(cudaMalloc(&I.partial, sizeof(double) * I.err_blocks));
    GBC_CUDA(cudaMalloc(&I.ctrl, sizeof(Ctrl)));
    GBC_CUDA(cudaMallocHost(&I.ctrl_host, sizeof(Ctrl)));
    return 0;
}

void integrator_free(Integrator& I) {
    for (int s = 0; s < 7; ++s) if (I.k[s]) cudaFree(I.k[s]);
    if (I.y) cudaFree(I.y);
    if (I.un) cudaFree(I.un);
    if (I.partial) cudaFree(I.partial);
    if (I.ctrl) cudaFree(I.ctrl);
    if (I.ctrl_host) cudaFreeHost(I.ctrl_host);
    if (I.step_exec) cudaGraphExecDestroy(I.step_exec);
    if (I.t_ring) cudaFree(I.t_ring);
    if (I.u_ring) cudaFree(I.u_ring);
    for (int j = 0; j <= kAbmMax; ++j) if (I.phi[j]) cudaFree(I.phi[j]);
    I = Integrator();
}

static int enqueue_step(Integrator& I, const RhsArgs& rhs0, double* u, cudaStream_t s) {
    const long long n = I.n;
    const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 4);
    RhsArgs rhs = rhs0;
    rhs.skip = &I.ctrl->done;
    KPtrs K;
    for (int r = 0; r < 7; ++r) K.k[r] = I.k[r];
    for (int st = 1; st < 7; ++st) {
        double* dst = (st == 6) ? I.un : I.y;
        k_stage<<<g, 256, 0, s>>>(st, n, u, K, dst, I.ctrl);
        GBC_CUDA(cudaGetLastError());
        if (int rc = launch_rhs(rhs, dst, I.k[st], s)) return rc;
    }
    k_error_control<<<I.err_blocks, 256, 0, s>>>(n, u, I.un, K, I.partial, I.ctrl);
    GBC_CUDA(cudaGetLastError());
    k_commit<<<g, 256, 0, s>>>(n, u, I.un, I.k[0], I.k[6], I.ctrl);
    GBC_CUDA(cudaGetLastError());
    k_clear_accept<<<1, 1, 0, s>>>(I.ctrl);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int integrator_run(Integrator& I, const RhsArgs& rhs0, double* u, double t0, double t1, double reltol,
                   double abstol, double dt0, double dtmax, double dtmin, long long maxiters,
                   cudaStream_t s, Recorder* rec, int alg) {
    if (alg != 0 && alg != 1) return fail(GBC_EINVAL, "unknown integrator (GBC_ALG_TSIT5 or GBC_ALG_VCABM5)");
    if (alg == 1 && !I.phi[0])
        for (int j = 0; j <= kAbmMax; ++j) {
            GBC_CUDA(cudaMalloc(&I.phi[j], sizeof(double) * I.n));
            GBC_CUDA(cudaMemsetAsync(I.phi[j], 0, sizeof(double) * I.n, s));
        }
    Ctrl h = ctrl_start(alg, t0, t1, reltol, abstol, dt0, dtmax, dtmin, maxiters);
    if (rec && rec->stride > 0) {
        const long long cap = 32;  // >= the steps of one graph launch
        if (I.ring_cap != cap) {
            if (I.t_ring) cudaFree(I.t_ring);
            if (I.u_ring) cudaFree(I.u_ring);
            I.t_ring = I.u_ring = nullptr;
            GBC_CUDA(cudaMalloc(&I.t_ring, sizeof(double) * cap));
            GBC_CUDA(cudaMalloc(&I.u_ring, sizeof(double) * cap * I.n));
            I.ring_cap = cap;
        }
        h.stride = rec->stride;
        h.ring_cap = I.ring_cap;
        h.t_ring = I.t_ring;
        h.u_ring = I.u_ring;
    }
    h.log_theta = rhs0.log_theta;
    h.th_lo = rhs0.N;
    h.th_hi = 2LL * rhs0.N;
    *I.ctrl_host = h;
    GBC_CUDA(cudaMemcpyAsync(I.ctrl, I.ctrl_host, sizeof(Ctrl), cudaMemcpyHostToDevice, s));
    RhsArgs rhs = rhs0;
    rhs.skip = nullptr;
    // FSAL seed k0 = f(u0) (Tsit5) or Phi_0 = f(u0) (VCABM5)
    if (int rc = launch_rhs(rhs, u, alg == 1 ? I.phi[0] : I.k[0], s)) return rc;
    // capture a group of steps once per (model, state pointer); relaunch until done
    const int group = (alg == 1) ? 16 : 8;
    if (I.step_exec) {
        cudaGraphExecDestroy(I.step_exec);
        I.step_exec = nullptr;
    }
    cudaGraph_t graph;
    GBC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int k = 0; k < group && rc == 0; ++k) rc = (alg == 1) ? enqueue_abm_step(I, rhs0, u, s) : enqueue_step(I, rhs0, u, s);
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (rc) return rc;
    GBC_CUDA(ce);
    GBC_CUDA(cudaGraphInstantiate(&I.step_exec, graph, 0));
    cudaGraphDestroy(graph);
    I.steps_per_launch = group;
    I.graph_launches = 0;
    for (;;) {
        GBC_CUDA(cudaGraphLaunch(I.step_exec, s));
        ++I.graph_launches;
        GBC_CUDA(cudaMemcpyAsync(I.ctrl_host, I.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        if (rec && rec->stride > 0) {  // drain the ring into the caller's host arrays
            const long long nrec = I.ctrl_host->nrec;
            for (; rec->drained < nrec; ++rec->drained) {
                const long long slot = rec->drained % I.ring_cap, dst = rec->drained + 1;  // slot 0 holds t0
                if (dst >= rec->max_records) continue;
                GBC_CUDA(cudaMemcpyAsync(rec->t_out + dst, I.t_ring + slot, sizeof(double), cudaMemcpyDeviceToHost, s));
                GBC_CUDA(cudaMemcpyAsync(rec->u_out + dst * I.n, I.u_ring + slot * I.n, sizeof(double) * I.n,
                                         cudaMemcpyDeviceToHost, s));
            }
            GBC_CUDA(cudaStreamSynchronize(s));
        }
        if (I.ctrl_host->done) break;
    }
    return I.ctrl_host->status;
}

}  // namespace gbc
