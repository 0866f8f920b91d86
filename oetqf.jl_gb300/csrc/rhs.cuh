// Right-hand-side kernels (src/BEM/equation.jl:156-166 fault-only, :185-205 viscoelastic).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

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
    // viscosity (property.jl:34-41)
    const double *gamma, *nexp;
    double deps0[6];
    // scratch: x = [v - vpl (N); 0 (npad - N); dϵ - dϵ₀ (6ne)]
    double* xm;
    // optional device flag: when non-null and nonzero the launch does nothing (finished solve)
    const int* skip;
};

// state offsets in the flat ArrayPartition layout
struct StateLayout {
    long long v, th, eps, sig, delta, n;
};
inline StateLayout layout_of(int N, int ne) {
    StateLayout s;
    const long long E = 6LL * ne;
    s.v = 0;
    s.th = N;
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

// Launches the RHS for the flat state u -> du on stream s (1 kernel fault-only, 2 viscoelastic).
int launch_rhs(const RhsArgs& a, const double* u, double* du, cudaStream_t s);

}  // namespace gbc
