// Block-scaled 16-bit Green's functions (BF16 or FP16 with one FP32 scale per 128x128 block) for
// the mantle interaction rows, FP32 accumulation, FP64 friction. The big GEMV streams the 16-bit
// matrix through shared memory with TMA (cp.async.bulk.tensor.2d) and an mbarrier ring: one
// elected thread issues a 32-row x 256-column tile plus the matching 256 entries of x per stage,
// eight warps consume four rows each. Every mbarrier wait is bounded; on a timeout the kernel
// records an error word, waits (bounded) for its own copies in flight and returns.
//
// Rows of the unified matrix: [0, M) mantle stress rates [G12 | 0 | G22] (equation.jl:202-203);
// [Mpad, Mpad + N) the G21 part of the fault traction rate (equation.jl:201). The fault rows
// then add the FP32 Toeplitz sum (equation.jl:44-61) and run the FP64 friction update
// (equation.jl:233-246) in k_fault_rows_smem (k_fault_rows_mixed for faults too large for its
// shared-memory staging).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "gbc_internal.cuh"
#include "mixed.cuh"
#include "rhs.cuh"
#include "tma.cuh"

namespace gbc {

constexpr int QB = 128;        // scale block edge
constexpr int TR = 32;         // rows per TMA tile
constexpr int TC = 256;        // columns per TMA tile (512 B of 16-bit)
constexpr int STAGES = 4;
constexpr unsigned kTileBytes = TR * TC * 2;
constexpr unsigned kXBytes = TC * 4;

// ---- quantisation --------------------------------------------------------------------------
struct QSrc {
    int N, npad;
    long long M, Mpad;
    const double* gm;
    size_t ldm;
    const double* g21;
    size_t ld21;
    __device__ __forceinline__ double at(long long r, long long c) const {
        if (r < M) return (c < npad + M) ? gm[(size_t)r * ldm + c] : 0.0;
        if (r >= Mpad && r < Mpad + N && c >= npad && c < npad + M) return g21[(size_t)(r - Mpad) * ld21 + (c - npad)];
        return 0.0;
    }
};

__global__ void k_block_scale(QSrc src, long long ncb, int mode, float* __restrict__ qscale) {
    const long long b = blockIdx.x;
    const long long rb = b / ncb, cb = b % ncb;
    double amax = 0.0;
    for (int t = threadIdx.x; t < QB * QB; t += blockDim.x) {
        const long long r = rb * QB + t / QB, c = cb * QB + t % QB;
        amax = fmax(amax, fabs(src.at(r, c)));
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = amax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
        // map the block maximum to 2^15 (inside FP16's 65504; BF16 keeps FP32's range anyway)
        qscale[b] = (m > 0.0) ? (float)(m / 32768.0) : 1.0f;
    }
}

__global__ void k_quantize(QSrc src, long long rowsq, long long ldq, int mode, const float* __restrict__ qscale,
                           uint16_t* __restrict__ q) {
    const long long ncb = ldq / QB;
    const long long total = rowsq * ldq;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long r = t / ldq, c = t % ldq;
        const float s = qscale[(r / QB) * ncb + c / QB];
        const float v = (float)(src.at(r, c) / (double)s);
        uint16_t bits;
        if (mode == GBC_PREC_BF16) {
            __nv_bfloat16 h = __float2bfloat16_rn(v);
            memcpy(&bits, &h, 2);
        } else {
            __half h = __float2half_rn(v);
            memcpy(&bits, &h, 2);
        }
        q[t] = bits;
    }
}

int quantize_mantle(int mode, int N, int npad, long long M, long long Mpad, long long rowsq, long long ldq,
                    const double* gm, size_t ldm, const double* g21, size_t ld21, void* q, float* qscale,
                    cudaStream_t s) {
    QSrc src{N, npad, M, Mpad, gm, ldm, g21, ld21};
    const long long nrb = rowsq / QB, ncb = ldq / QB;
    k_block_scale<<<(unsigned)(nrb * ncb), 256, 0, s>>>(src, ncb, mode, qscale);
    GBC_CUDA(cudaGetLastError());
    k_quantize<<<sm_count() * 8, 256, 0, s>>>(src, rowsq, ldq, mode, qscale, static_cast<uint16_t*>(q));
    GBC_CUDA(cudaGetLastError());
    return 0;
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

int fault_f32(const double* st, float* st32, long long n, cudaStream_t s) {
    k_to_f32<<<sm_count() * 2, 256, 0, s>>>(st, st32, n);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int encode_tmap_2d(void* base, int dtype, int esize, long long rows, long long cols, int box_cols, int box_rows,
                   bool swizzle128, void* tmap_out) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult qr;
        void* fn = nullptr;
        GBC_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr));
        if (qr != cudaDriverEntryPointSuccess || !fn) return fail(GBC_ECUDA, "cuTensorMapEncodeTiled unavailable");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * (cuuint64_t)esize};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(static_cast<CUtensorMap*>(tmap_out), (CUtensorMapDataType)dtype, 2, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GBC_ECUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return 0;
}

int encode_qmap(int mode, void* q, long long rowsq, long long ldq, void* tmap_out) {
    return encode_tmap_2d(q, mode == GBC_PREC_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                          rowsq, ldq, TC, TR, false, tmap_out);
}

// Failure-injection hook for tests (gbc_debug_pipeline_fault): when set, the GEMV's producer
// issues no copies, so no full-barrier phase ever completes, and every pipeline wait gives up after
// kFaultPolls polls. The kernel then takes its timeout path (error word, return) without any copy
// in flight. Zero (the default) leaves the kernel as it is.
__device__ int g_pipeline_fault = 0;
constexpr long long kFaultPolls = 1024;

__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, unsigned parity, long long polls) {
    for (long long i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// y = Q x for one 32-row tile per CTA; mantle rows go to du (FP64), fault rows to y32.
template <int MODE>
__global__ void __launch_bounds__(256) k_gemv_tma(const __grid_constant__ CUtensorMap tm, RhsArgs a,
                                                  double* __restrict__ du_sig) {
    if (a.skip && *a.skip) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* tiles = smem;                                 // STAGES x kTileBytes
    float* xs = reinterpret_cast<float*>(smem + STAGES * kTileBytes);  // STAGES x TC
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * (kTileBytes + kXBytes));
    uint64_t* empty = full + STAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long row0 = (long long)blockIdx.x * TR;
    const int nch = (int)(a.ldq / TC);
    const long long ncb = a.ldq / QB;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 8);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool inject = g_pipeline_fault != 0;
    const long long polls = inject ? kFaultPolls : kWaitLimit;
    const bool producer = (threadIdx.x == 0);
    if (producer && !inject) {
        for (int c = 0; c < STAGES && c < nch; ++c) {
            mbar_expect_tx(&full[c], kTileBytes + kXBytes);
            tma_tile(tiles + c * kTileBytes, &tm, c * TC, (int)row0, &full[c]);
            bulk_copy(xs + c * TC, a.x32 + (size_t)c * TC, kXBytes, &full[c]);
        }
    }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const long long rb = row0 / QB;
    bool ok = true;
    int c = 0;
    for (; c < nch; ++c) {
        const int s = c % STAGES;
        const unsigned ph = (unsigned)((c / STAGES) & 1);
        if (!mbar_wait_n(&full[s], ph, polls)) { ok = false; break; }
        const unsigned char* tile = tiles + s * kTileBytes;
        const float4* xv = reinterpret_cast<const float4*>(xs + s * TC) + 2 * lane;
        const float4 x0 = xv[0], x1 = xv[1];
        const float sc = __ldg(a.qscale + rb * ncb + 2LL * c + (lane >> 4));
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint4 qv = *reinterpret_cast<const uint4*>(tile + (4 * warp + r) * (TC * 2) + 16 * lane);
            float f[8];
            unpack8<MODE>(qv, f);
            float p = f[0] * x0.x;
            p = fmaf(f[1], x0.y, p);
            p = fmaf(f[2], x0.z, p);
            p = fmaf(f[3], x0.w, p);
            p = fmaf(f[4], x1.x, p);
            p = fmaf(f[5], x1.y, p);
            p = fmaf(f[6], x1.z, p);
            p = fmaf(f[7], x1.w, p);
            acc[r] = fmaf(sc, p, acc[r]);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
        if (producer && c + STAGES < nch) {
            if (!mbar_wait_n(&empty[s], ph, polls)) { ok = false; break; }
            mbar_expect_tx(&full[s], kTileBytes + kXBytes);
            tma_tile(tiles + s * kTileBytes, &tm, (c + STAGES) * TC, (int)row0, &full[s]);
            bulk_copy(xs + s * TC, a.x32 + (size_t)(c + STAGES) * TC, kXBytes, &full[s]);
        }
    }
    if (!ok) {
        atomicExch(a.err, 1);
        if (producer && !inject) {  // let our own copies in flight land before the CTA's shared memory goes away
            for (int k = c; k < nch && k < c + STAGES; ++k) mbar_wait(&full[k % STAGES], (unsigned)((k / STAGES) & 1));
        }
        return;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float v = acc[r];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        const long long row = row0 + 4 * warp + r;
        if (lane == 0) {
            if (row < 6LL * a.ne) du_sig[row] = (double)v;
            else if (row >= a.Mpad && row < a.Mpad + a.N) a.y32[row - a.Mpad] = v;
        }
    }
}

// x = [v - vpl; 0; dϵ - dϵ₀] in FP32 (PAIR: as FP32 pairs hi + lo) and dϵ (FP64) -- the
// viscoelastic prologue of the 16-bit and double-float paths
template <bool PAIR>
__device__ __forceinline__ void put_x(float* x, long long i, double v) {
    if (PAIR) {
        const float hi = __double2float_rn(v);
        reinterpret_cast<float2*>(x)[i] = make_float2(hi, __double2float_rn(v - (double)hi));
    } else {
        x[i] = (float)v;
    }
}

template <bool PAIR>
__global__ void k_prologue_mixed(RhsArgs a, const double* __restrict__ u, double* __restrict__ du, StateLayout L) {
    if (a.skip && *a.skip) return;
    const int ne = a.ne, N = a.N;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N + ne; t += gridDim.x * blockDim.x) {
        if (t < N) {
            put_x<PAIR>(a.x32, t, u[L.v + t] - a.vpl);
            continue;
        }
        const int i = t - N;
        double d[6];
        viscous_rates(a, u + L.sig, i, d);
        double* deps = du + L.eps;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            deps[i + k * ne] = d[k];
            put_x<PAIR>(a.x32, a.npad + i + (long long)k * ne, d[k] - a.deps0[k]);
        }
    }
}

// Fault rows: FP32 Toeplitz sum + the G21 part from the GEMV, then FP64 friction (one warp/row).
__global__ void __launch_bounds__(256) k_fault_rows_mixed(RhsArgs a, const double* __restrict__ u,
                                                          double* __restrict__ du, StateLayout L) {
    if (a.skip && *a.skip) return;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int nx = a.nx, nxi = a.nxi, N = a.N;
    const double* v = u + L.v;
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < N; i += warps) {
        const int ii = i % nx, j = i / nx;
        float acc = 0.f;
        for (int l = 0; l < nxi; ++l) {
            const float* stl = a.st32 + (size_t)nx * (j + (size_t)nxi * l);
            const double* vl = v + (size_t)nx * l;
            for (int k = lane; k < nx; k += 32) {
                const int d = ii > k ? ii - k : k - ii;
                acc = fmaf(__ldg(stl + d), (float)(vl[k] - a.vpl), acc);
            }
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) fault_friction(a, u, du, L, i, (double)acc + (a.ne > 0 ? (double)a.y32[i] : 0.0));
    }
}

__global__ void __launch_bounds__(kFR_II * kFR_L) k_fault_rows_smem(RhsArgs a, const double* __restrict__ u,
                                                                 double* __restrict__ du, StateLayout L) {
    if (a.skip && *a.skip) return;
    extern __shared__ float fsm[];
    fault_rows_cta(a, u, du, L, (int)blockIdx.x, fsm);
}

size_t fault_rows_smem_bytes(int N, int nx, int nxi) { return sizeof(float) * ((size_t)N + (size_t)nx * nxi); }

int set_pipeline_fault(int mode) {
    const int v = mode ? 1 : 0;
    GBC_CUDA(cudaMemcpyToSymbol(g_pipeline_fault, &v, sizeof(int)));
    return 0;
}

int launch_rhs_mixed(const RhsArgs& a, const double* u, double* du, cudaStream_t s) {
    const StateLayout L = layout_of(a.N, a.ne);
    const int sms = sm_count();
    const bool pair = (a.mode == GBC_PREC_DF64);
    if (a.ne > 0) {
        const int n = a.N + a.ne;
        int g = (n + 255) / 256;
        if (g > sms * 8) g = sms * 8;
        if (pair) k_prologue_mixed<true><<<g, 256, 0, s>>>(a, u, du, L);
        else k_prologue_mixed<false><<<g, 256, 0, s>>>(a, u, du, L);
        GBC_CUDA(cudaGetLastError());
    }
    if (pair) return launch_gemv_df64(a, u, du, s);  // fault rows and friction included
    if (a.ne > 0) {
        const size_t smem = STAGES * (kTileBytes + kXBytes) + 2 * STAGES * sizeof(uint64_t);
        const unsigned grid = (unsigned)(a.rowsq / TR);
        CUtensorMap tm;
        memcpy(&tm, a.tmap, sizeof(tm));
        if (a.mode == GBC_PREC_BF16) {
            if (int rc = set_smem_limit((const void*)k_gemv_tma<GBC_PREC_BF16>, (int)smem)) return rc;
            k_gemv_tma<GBC_PREC_BF16><<<grid, 256, smem, s>>>(tm, a, du + L.sig);
        } else {
            if (int rc = set_smem_limit((const void*)k_gemv_tma<GBC_PREC_F16>, (int)smem)) return rc;
            k_gemv_tma<GBC_PREC_F16><<<grid, 256, smem, s>>>(tm, a, du + L.sig);
        }
        GBC_CUDA(cudaGetLastError());
    }
    const size_t fsm = fault_rows_smem_bytes(a.N, a.nx, a.nxi);
    if (fsm <= 160 * 1024) {
        if (int rc = set_smem_limit((const void*)k_fault_rows_smem, 160 * 1024)) return rc;
        const int nb = (a.nx + kFR_II - 1) / kFR_II;
        k_fault_rows_smem<<<nb * a.nxi, kFR_II * kFR_L, fsm, s>>>(a, u, du, L);
    } else {  // faults above ~20k patches: one warp per row through L2
        int g = (a.N + 7) / 8;
        if (g > sms * 8) g = sms * 8;
        k_fault_rows_mixed<<<g, 256, 0, s>>>(a, u, du, L);
    }
    GBC_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace gbc
