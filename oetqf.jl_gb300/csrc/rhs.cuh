// Right-hand-side kernels (src/BEM/equation.jl:156-166 fault-only, :185-205 viscoelastic).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

#include "gbcycle.h"

namespace gbc {

struct RhsArgs {
    int nx, nxi, ne, N;          // N = nx * nxi
    int npad;                    // column offset of the strain-rate block (N rounded up to 32)
    // fault-fault real Toeplitz kernel st (nx, nxi, nxi), column-major
    const double* st;
    // mantle receiver rows [G12 | 0 | G22], row-major (6ne x (npad + 6ne)), leading dim ldm
    const double* gm;
    size_t ldm;
    // fault receiver rows G21, row-major (N x 6ne), leading dimension ld21
    const double* g21;
    size_t ld21;
    // friction (property.jl:10-25)
    const double *a, *b, *L, *sig;
    double eta, vpl, f0, v0;
    // viscosity (property.jl:34-48): nlaws power laws summed, gamma/nexp are (nlaws x ne) law-major
    const double *gamma, *nexp;
    int nlaws;
    double deps0[6];
    // dilatancy (property.jl:27-32): nonzero -> fault-only state (v, θ, δ, 𝓅)
    int dila;
    const double *tp, *deps_d, *beta_d, *p0;
    // scratch: x = [v - vpl (N); 0 (npad - N); dϵ - dϵ₀ (6ne)]
    double* xm;
    // optional device flag: when non-null and nonzero the launch does nothing (finished solve)
    const int* skip;
    // integrate ln θ instead of θ (the state's θ slot holds ψ = ln θ; dψ/dt = (1 - vθ/L)/θ)
    int log_theta;
    // ---- block-scaled 16-bit storage (GBC_PREC_BF16 / GBC_PREC_F16) --------------------------
    int mode;                    // GBC_PREC_*: 0 FP64 path above; 1 BF16; 2 FP16; 3 double-float pairs
    const void* q;               // (rowsq x ldq) 16-bit: rows [0,M) = [G12|0|G22], [Mpad,Mpad+N) = [0|G21]
    const float* qscale;         // FP32 scale per 128x128 block, (rowsq/128) x (ldq/128)
    long long rowsq, ldq, Mpad;
    const void* tmap;            // host pointer to the CUtensorMap of q (box 256 x 32)
    const float* st32;           // fault-fault Toeplitz kernel in FP32
    float* x32;                  // [v - vpl; 0; dϵ - dϵ₀; 0] in FP32, length ldq (DF64: FP32 pairs, 2 ldq)
    float* y32;                  // G21 part of the fault rows, length N
    int* err;                    // device error word (bounded-wait timeouts)
};

// state offsets in the flat ArrayPartition layout
struct StateLayout {
    long long v, th, eps, sig, delta, p, n;
};
inline StateLayout layout_of(int N, int ne, int dila = 0) {
    StateLayout s;
    const long long E = 6LL * ne;
    s.v = 0;
    s.th = N;
    s.p = -1;
    if (dila) {  // (v, θ, δ, 𝓅), equation.jl:176-177
        s.eps = s.sig = -1;
        s.delta = 2LL * N;
        s.p = 3LL * N;
        s.n = 4LL * N;
        return s;
    }
    if (ne > 0) {
        s.eps = 2LL * N;
        s.sig = 2LL * N + E;
        s.delta = 2LL * N + 2 * E;
        s.n = 3LL * N + 2 * E;
    } else {
        s.eps = s.sig = -1;
        s.delta = 2LL * N;
        s.n = 3LL * N;
    }
    return s;
}

#ifdef __CUDACC__
// update_fault! (equation.jl:233-246) with the ageing law (:279) for patch i, given its traction
// rate dτ: writes dθ (or dψ = dθ/θ when the state holds ψ = ln θ), dv and dδ = v.
__device__ __forceinline__ void fault_friction(const RhsArgs& a, const double* __restrict__ u, double* __restrict__ du,
                                               const StateLayout& L, int i, double dtau) {
    const double vi = u[L.v + i], th = a.log_theta ? exp(u[L.th + i]) : u[L.th + i];
    const double ai = a.a[i], bi = a.b[i], Li = a.L[i];
    const double psi1 = exp((a.f0 + bi * log(a.v0 * fmax(0.0, th) / Li)) / ai) / (2.0 * a.v0);
    const double psi2 = a.sig[i] * psi1 / hypot(1.0, vi * psi1);
    const double dmu_dv = ai * psi2;
    const double dmu_dth = bi / th * vi * psi2;
    const double dth = 1.0 - vi * th / Li;
    du[L.th + i] = a.log_theta ? dth / th : dth;
    du[L.v + i] = (dtau - dmu_dth * dth) / (dmu_dv + a.eta);
    du[L.delta + i] = vi;
}

// Σ_q γ_q τ^{n_q} of cell i (equation.jl:285-292); τ^0 = 1 exactly, as pow returns
__device__ __forceinline__ double viscous_factor(const RhsArgs& a, int i, double tau) {
    double f = 0.0;
    for (int q = 0; q < a.nlaws; ++q) {
        const double n = a.nexp[i + (size_t)q * a.ne];
        f += a.gamma[i + (size_t)q * a.ne] * (n == 0.0 ? 1.0 : pow(tau, n));
    }
    return f;
}

// Power-law strain rates of cell i (equation.jl:285-292): d = f(τ) σ', σ' the deviatoric part of
// the cell's stress (xx, xy, xz, yy, yz, zz) in the (ne, 6) block s and τ its second invariant.
__device__ __forceinline__ void viscous_rates(const RhsArgs& a, const double* __restrict__ s, int i, double (&d)[6]) {
    const int ne = a.ne;
    const double skk = (s[i] + s[i + 3 * ne] + s[i + 5 * ne]) / 3.0;
    const double sxx = s[i] - skk, syy = s[i + 3 * ne] - skk, szz = s[i + 5 * ne] - skk;
    const double sxy = s[i + ne], sxz = s[i + 2 * ne], syz = s[i + 4 * ne];
    const double tau = sqrt(sxx * sxx + syy * syy + szz * szz + 2.0 * (sxy * sxy + sxz * sxz + syz * syz));
    const double f = viscous_factor(a, i, tau);  // equation.jl:285 (one law) or :286-292 (composite)
    d[0] = f * sxx;
    d[1] = f * sxy;
    d[2] = f * sxz;
    d[3] = f * syy;
    d[4] = f * syz;
    d[5] = f * szz;
}
#endif

// Launches the RHS for the flat state u -> du on stream s (1 kernel fault-only, 2 viscoelastic).
int launch_rhs(const RhsArgs& a, const double* u, double* du, cudaStream_t s);
// Number of kernels one launch_rhs enqueues for these arguments.
int rhs_kernel_count(const RhsArgs& a);

// Block-scaled 16-bit path (mixed.cu)
int launch_rhs_mixed(const RhsArgs& a, const double* u, double* du, cudaStream_t s);
// failure-injection hook of the 16-bit GEMV pipeline on the current device (gbc_debug_pipeline_fault)
int set_pipeline_fault(int mode);
// Builds q and qscale from the FP64 rows (gm with ldm, g21 with ld21) on stream s.
int quantize_mantle(int mode, int N, int npad, long long M, long long Mpad, long long rowsq, long long ldq,
                    const double* gm, size_t ldm, const double* g21, size_t ld21, void* q, float* qscale,
                    cudaStream_t s);
// Encodes the TMA descriptor for q (rowsq x ldq 16-bit, box 256 columns x 32 rows).
int encode_qmap(int mode, void* q, long long rowsq, long long ldq, void* tmap_out /* 128 B */);
int fault_f32(const double* st, float* st32, long long n, cudaStream_t s);

// Double-float path (df64.cu): q holds (rowsq x ldq) FP32 pairs of the unified rows, whose fault
// rows carry the dense fault-fault block expanded from the Toeplitz kernel st in columns [0, N).
int split_mantle(int nx, int nxi, int npad, long long M, long long Mpad, long long rowsq, long long ldq,
                 const double* st, const double* gm, size_t ldm, const double* g21, size_t ld21, void* q,
                 cudaStream_t s);
int encode_pairmap(void* q, long long rowsq, long long ldq, void* tmap_out /* 128 B */);
// The double-float GEMV over all unified rows; fault rows finish with the friction update.
int launch_gemv_df64(const RhsArgs& a, const double* u, double* du, cudaStream_t s);
// the path launch_rhs takes: FP64 rows, or the 16-bit / double-float mantle GEMV
inline bool uses_mixed(const RhsArgs& a) { return a.mode != 0 && !a.dila && !(a.mode == GBC_PREC_DF64 && a.ne == 0); }

}  // namespace gbc
