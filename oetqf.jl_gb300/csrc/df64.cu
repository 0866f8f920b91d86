// FP64-accurate mantle GEMV on the FP32 pipe (GBC_PREC_DF64).
//
// GB300 issues FP64 FMAs at 1/56 of its FP32 rate, so an FP64 GEMV over the mantle rows is bound
// by the FP64 pipe (about 0.6 of HBM bandwidth), not by memory. Here every Green's-function entry
// g is stored as the unevaluated FP32 pair (hi, lo) = (fl32(g), fl32(g - hi)) -- eight bytes, as
// in FP64 -- and x = [v - vpl; 0; dϵ - dϵ₀] likewise. Each product g·x is formed with Dekker's
// TwoProduct (p = fl(gh xh), r = fma(gh, xh, -p): p + r = gh xh exactly) plus the two cross terms,
// and accumulated with Knuth's TwoSum into a (sum, error) pair: the compensated dot product "Dot2"
// of Ogita, Rump & Oishi (SIAM J. Sci. Comput. 26, 2005), applied to double-float operands. The
// result carries ~48 significant bits (representation error 2^-48 per operand, cross terms at
// 2^-48, accumulation error ~n 2^-48 of the sum of |terms| over a lane's n terms), converted to
// FP64 per lane and reduced across the warp in FP64.
//
// The kernel is persistent (two CTAs per SM, tiles dealt round-robin so the 8-row tiles of every
// part of the matrix spread over all SMs). In each CTA one producer warp streams 8-row x
// 256-entry tiles of the pair matrix (TMA, cp.async.bulk.tensor.2d, 16 KB) plus the matching 2 KB
// of x (cp.async.bulk) through a 6-stage mbarrier ring; eight consumer warps take one row each.
// Every wait is bounded; on a timeout the kernel records an error word, the producer waits
// (bounded) for its own copies in flight, and all threads return.
//
// Rows follow the unified layout of the 16-bit path: [0, M) mantle stress rates [G12 | 0 | G22]
// (equation.jl:202-203); [Mpad, Mpad + N) the fault traction rate, here [G11 | 0 | G21] with the
// fault-fault block expanded densely from the Toeplitz kernel (the convolution of :44-61 plus
// :201 as one row; 8 N^2 extra bytes), so a fault row is complete when its warp finishes and the
// same warp runs the FP64 friction update (:233-246) on it: one launch after the prologue.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "gbc_internal.cuh"
#include "rhs.cuh"
#include "tma.cuh"

namespace gbc {

constexpr int DR = 8;                               // rows per tile (one per consumer warp)
constexpr int DC = 256;                             // entries per chunk (2 KB per row)
constexpr int DSTAGES = 6;
constexpr unsigned kDTile = DR * DC * 8;            // 16 KB
constexpr unsigned kDX = DC * 8;                    // 2 KB
constexpr int kDThreads = 32 * (DR + 1);            // 8 consumer warps + 1 producer warp
constexpr int kDCtasPerSM = 2;

size_t df64_smem_bytes() { return DSTAGES * (kDTile + kDX) + 2 * DSTAGES * sizeof(uint64_t); }

// ---- storage ---------------------------------------------------------------------------------
struct PairSrc {
    int nx, nxi, N, npad;
    long long M, Mpad;
    const double* st;
    const double* gm;
    size_t ldm;
    const double* g21;
    size_t ld21;
    __device__ __forceinline__ double at(long long r, long long c) const {
        if (r < M) return (c < npad + M) ? gm[(size_t)r * ldm + c] : 0.0;
        if (r < Mpad || r >= Mpad + N) return 0.0;
        const int i = (int)(r - Mpad);
        if (c < N) {  // fault-fault: st[|i_x - k_x|, i_ξ, k_ξ]
            const int k = (int)c, ii = i % nx, kk = k % nx;
            const int d = ii > kk ? ii - kk : kk - ii;
            return st[(size_t)d + (size_t)nx * (i / nx + (size_t)nxi * (k / nx))];
        }
        if (c >= npad && c < npad + M) return g21[(size_t)i * ld21 + (c - npad)];
        return 0.0;
    }
};

__device__ __forceinline__ float2 split_pair(double v) {
    const float hi = __double2float_rn(v);
    return make_float2(hi, __double2float_rn(v - (double)hi));
}

__global__ void k_split(PairSrc src, long long rowsq, long long ldq, float2* __restrict__ q) {
    const long long total = rowsq * ldq;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x)
        q[t] = split_pair(src.at(t / ldq, t % ldq));
}

int split_mantle(int nx, int nxi, int npad, long long M, long long Mpad, long long rowsq, long long ldq,
                 const double* st, const double* gm, size_t ldm, const double* g21, size_t ld21, void* q,
                 cudaStream_t s) {
    PairSrc src{nx, nxi, nx * nxi, npad, M, Mpad, st, gm, ldm, g21, ld21};
    k_split<<<sm_count() * 8, 256, 0, s>>>(src, rowsq, ldq, static_cast<float2*>(q));
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int encode_pairmap(void* q, long long rowsq, long long ldq, void* tmap_out) {
    // the pair matrix seen as 8-byte elements (one FP32 pair each; TMA only moves the bytes): the
    // inner box is 256 pairs = 2 KB, every tile starts at a multiple of 2 KB (16-byte TMA rule)
    // and the row stride is 8*ldq bytes
    return encode_tmap_2d(q, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, rowsq, ldq, DC, DR, false, tmap_out);
}

// ---- compensated arithmetic -----------------------------------------------------------------
// (s, e) += (gh + gl)(xh + xl). The _rn intrinsics are never contracted into FMAs, which the
// error-free transformations rely on.
__device__ __forceinline__ void dot2_step(float& s, float& e, float gh, float gl, float xh, float xl) {
    const float p = __fmul_rn(gh, xh);
    const float r = __fmaf_rn(gh, xh, -p);                 // TwoProduct: p + r = gh xh
    const float c = __fmaf_rn(gh, xl, __fmul_rn(gl, xh));  // cross terms (gl xl ~ 2^-48 dropped)
    const float t = __fadd_rn(s, p);                       // TwoSum: t + d = s + p
    const float z = __fsub_rn(t, s);
    const float d = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    e = __fadd_rn(e, __fadd_rn(d, __fadd_rn(r, c)));
}

// ---- the GEMV ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(kDThreads, kDCtasPerSM) k_gemv_df64(const __grid_constant__ CUtensorMap tm, RhsArgs a,
                                                                      const double* __restrict__ u,
                                                                      double* __restrict__ du, StateLayout L) {
    if (a.skip && *a.skip) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    float* tiles = reinterpret_cast<float*>(smem);                               // DSTAGES x DR x 2DC
    float* xs = reinterpret_cast<float*>(smem + DSTAGES * kDTile);               // DSTAGES x 2DC
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + DSTAGES * (kDTile + kDX));
    uint64_t* empty = full + DSTAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // tiles blockIdx.x, blockIdx.x + gridDim.x, ...
    const int ntiles = (int)(a.rowsq / DR);
    const int mine = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    const int nch = (int)(a.ldq / DC);
    const long long nitems = (long long)mine * nch;
    if (threadIdx.x == 0) {
        for (int s = 0; s < DSTAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], DR);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == DR) {  // producer warp: one elected lane issues every copy
        if (lane != 0) return;
        // ring position (stage s, its use count n) and matrix position (tile t, chunk c) advance
        // incrementally: no 64-bit division on the issue path
        int s = 0, c = 0, t = (int)blockIdx.x;
        unsigned n = 0;
        long long k = 0;
        bool ok = true;
        for (; k < nitems; ++k) {
            if (n > 0 && !mbar_wait(&empty[s], (n - 1) & 1)) { ok = false; break; }
            mbar_expect_tx(&full[s], kDTile + kDX);
            tma_tile(tiles + (size_t)s * DR * 2 * DC, &tm, c * DC, t * DR, &full[s]);
            bulk_copy(xs + (size_t)s * 2 * DC, a.x32 + (size_t)c * 2 * DC, kDX, &full[s]);
            if (++c == nch) { c = 0; t += gridDim.x; }
            if (++s == DSTAGES) { s = 0; ++n; }
        }
        if (!ok) atomicExch(a.err, 2);
        // the CTA's shared memory must outlive every copy issued: wait for the last ring's worth
        for (long long j = (k > DSTAGES ? k - DSTAGES : 0); j < k; ++j)
            if (!mbar_wait(&full[j % DSTAGES], (unsigned)((j / DSTAGES) & 1))) atomicExch(a.err, 3);
        return;
    }

    float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f;
    int s = 0, c = 0;
    unsigned ph = 0;
    long long row = (long long)blockIdx.x * DR + warp;
    for (long long k = 0; k < nitems; ++k) {
        if (!mbar_wait(&full[s], ph)) {
            atomicExch(a.err, 1);
            return;
        }
        const float4* g = reinterpret_cast<const float4*>(tiles + ((size_t)s * DR + warp) * 2 * DC);
        const float4* x = reinterpret_cast<const float4*>(xs + (size_t)s * 2 * DC);
        float4 gv[4], xv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            gv[q] = g[32 * q + lane];
            xv[q] = x[32 * q + lane];
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
        if (++s == DSTAGES) { s = 0; ph ^= 1u; }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            dot2_step(s0, e0, gv[q].x, gv[q].y, xv[q].x, xv[q].y);
            dot2_step(s1, e1, gv[q].z, gv[q].w, xv[q].z, xv[q].w);
        }
        if (++c == nch) {  // the tile's last chunk: this warp's row is complete
            c = 0;
            double r = ((double)s0 + (double)e0) + ((double)s1 + (double)e1);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
            if (lane == 0) {
                if (row < 6LL * a.ne) du[L.sig + row] = r;
                else if (row >= a.Mpad && row < a.Mpad + a.N) fault_friction(a, u, du, L, (int)(row - a.Mpad), r);
            }
            row += (long long)gridDim.x * DR;
            s0 = e0 = s1 = e1 = 0.f;
        }
    }
}

int launch_gemv_df64(const RhsArgs& a, const double* u, double* du, cudaStream_t s) {
    const size_t smem = df64_smem_bytes();
    if (int rc = set_smem_limit((const void*)k_gemv_df64, (int)smem)) return rc;
    const int ntiles = (int)(a.rowsq / DR);
    const int slots = sm_count() * kDCtasPerSM;
    const int grid = ntiles < slots ? ntiles : slots;
    CUtensorMap tm;
    memcpy(&tm, a.tmap, sizeof(tm));
    k_gemv_df64<<<grid, kDThreads, smem, s>>>(tm, a, u, du, layout_of(a.N, a.ne));
    GBC_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace gbc
