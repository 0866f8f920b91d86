// Device buffers and the model handle behind gbc_model* (shared by the C ABI and the sweep,
// which borrows a model's block-scaled Green's functions).
#pragma once
#include <cuda_runtime.h>

#include "gbc_internal.cuh"
#include "integrator.cuh"
#include "rhs.cuh"

namespace gbc {

// ---- device buffers --------------------------------------------------------------------------
struct DevBuf {
    double* p = nullptr;
    size_t n = 0;
    int alloc(size_t count) {
        if (p && n == count) return 0;
        release();
        if (count == 0) return 0;
        cudaError_t e = cudaMalloc(&p, sizeof(double) * count);
        if (e != cudaSuccess) { p = nullptr; return cuda_fail(e, "cudaMalloc"); }
        n = count;
        return 0;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
};

struct RawBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int alloc(size_t nbytes) {
        if (p && bytes == nbytes) return 0;
        release();
        if (nbytes == 0) return 0;
        cudaError_t e = cudaMalloc(&p, nbytes);
        if (e != cudaSuccess) { p = nullptr; return cuda_fail(e, "cudaMalloc"); }
        bytes = nbytes;
        return 0;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    ~RawBuf() { release(); }
};

inline int upload(DevBuf& b, const double* h, size_t count, cudaStream_t s) {
    if (int rc = b.alloc(count)) return rc;
    GBC_CUDA(cudaMemcpyAsync(b.p, h, sizeof(double) * count, cudaMemcpyHostToDevice, s));
    return 0;
}

}  // namespace gbc

struct gbc_model {
    int nx = 0, nxi = 0, ne = 0, N = 0, npad = 0;
    long long M = 0;
    size_t ldm = 0, ld21 = 0;
    cudaStream_t stream = nullptr;
    gbc::DevBuf st, gm, g21, a, b, L, sig, gamma, nexp, xm, u, du, tp, deps_d, beta_d, p0;
    int nlaws = 1;
    int dila = 0;
    double eta = 0, vpl = 0, f0 = 0.6, v0 = 1e-6, deps0[6] = {0, 0, 0, 0, 0, 0};
    bool props = false, mprops = false, has_st = false, has_g12 = false, has_g21 = false, has_g22 = false;
    int precision = GBC_PREC_F64;
    int log_theta = 0;
    bool mixed_dirty = true;
    long long rowsq = 0, ldq = 0, Mpad = 0;
    gbc::RawBuf q, qscale, x32, y32, st32, err;
    alignas(128) unsigned char tmap[128];
    gbc::Integrator integ;

    gbc::RhsArgs args() const {
        gbc::RhsArgs r{};
        r.nx = nx; r.nxi = nxi; r.ne = ne; r.N = N; r.npad = npad;
        r.st = st.p; r.gm = gm.p; r.ldm = ldm; r.g21 = g21.p; r.ld21 = ld21;
        r.a = a.p; r.b = b.p; r.L = L.p; r.sig = sig.p;
        r.eta = eta; r.vpl = vpl; r.f0 = f0; r.v0 = v0;
        r.gamma = gamma.p; r.nexp = nexp.p; r.nlaws = nlaws;
        for (int k = 0; k < 6; ++k) r.deps0[k] = deps0[k];
        r.dila = dila;
        r.tp = tp.p; r.deps_d = deps_d.p; r.beta_d = beta_d.p; r.p0 = p0.p;
        r.xm = xm.p;
        r.skip = nullptr;
        r.log_theta = 0;
        r.mode = precision;
        r.q = q.p;
        r.qscale = static_cast<const float*>(qscale.p);
        r.rowsq = rowsq; r.ldq = ldq; r.Mpad = Mpad;
        r.tmap = tmap;
        r.st32 = static_cast<const float*>(st32.p);
        r.x32 = static_cast<float*>(x32.p);
        r.y32 = static_cast<float*>(y32.p);
        r.err = static_cast<int*>(err.p);
        return r;
    }
    // builds the block-scaled 16-bit (or double-float pair) copies when such a mode is on and the
    // GFs changed
    int prepare() {
        if (precision == GBC_PREC_F64 || !mixed_dirty) return 0;
        if (precision == GBC_PREC_DF64) return prepare_pairs();
        if (int rc = ready()) return rc;
        Mpad = (M + 127) / 128 * 128;
        rowsq = Mpad + (N + 127) / 128 * 128;
        ldq = (npad + M + 255) / 256 * 256;
        if (ne == 0) { rowsq = 128; ldq = 256; }
        cudaStream_t s = stream;
        if (int rc = st32.alloc(sizeof(float) * (size_t)nx * nxi * nxi)) return rc;
        if (int rc = gbc::fault_f32(st.p, static_cast<float*>(st32.p), (long long)nx * nxi * nxi, s)) return rc;
        if (int rc = y32.alloc(sizeof(float) * N)) return rc;
        if (int rc = err.alloc(sizeof(int))) return rc;
        GBC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
        if (ne > 0) {
            if (int rc = q.alloc(2 * (size_t)rowsq * ldq)) return rc;
            if (int rc = qscale.alloc(sizeof(float) * (size_t)(rowsq / 128) * (ldq / 128))) return rc;
            if (int rc = x32.alloc(sizeof(float) * (size_t)ldq)) return rc;
            GBC_CUDA(cudaMemsetAsync(x32.p, 0, sizeof(float) * (size_t)ldq, s));
            if (int rc = gbc::quantize_mantle(precision, N, npad, M, Mpad, rowsq, ldq, gm.p, ldm, g21.p, ld21, q.p,
                                         static_cast<float*>(qscale.p), s))
                return rc;
            if (int rc = gbc::encode_qmap(precision, q.p, rowsq, ldq, tmap)) return rc;
        }
        GBC_CUDA(cudaStreamSynchronize(s));
        mixed_dirty = false;
        return 0;
    }
    int prepare_pairs() {
        if (int rc = ready()) return rc;
        cudaStream_t s = stream;
        if (int rc = err.alloc(sizeof(int))) return rc;
        GBC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
        if (ne > 0) {
            Mpad = (M + 127) / 128 * 128;
            rowsq = Mpad + (N + 127) / 128 * 128;
            ldq = (npad + M + 255) / 256 * 256;
            if (int rc = q.alloc(8 * (size_t)rowsq * ldq)) return rc;
            if (int rc = x32.alloc(8 * (size_t)ldq)) return rc;
            GBC_CUDA(cudaMemsetAsync(x32.p, 0, 8 * (size_t)ldq, s));
            if (int rc = gbc::split_mantle(nx, nxi, npad, M, Mpad, rowsq, ldq, st.p, gm.p, ldm, g21.p, ld21, q.p, s))
                return rc;
            if (int rc = gbc::encode_pairmap(q.p, rowsq, ldq, tmap)) return rc;
        }
        GBC_CUDA(cudaStreamSynchronize(s));
        mixed_dirty = false;
        return 0;
    }
    int ready() const {
        if (!props) return gbc::fail(GBC_ESTATE, "fault properties not set (gbc_model_set_fault_props)");
        if (!has_st) return gbc::fail(GBC_ESTATE, "fault-fault Green's function not set");
        if (ne > 0 && (!mprops || !has_g12 || !has_g21 || !has_g22))
            return gbc::fail(GBC_ESTATE, "viscoelastic model needs mantle properties and gf12, gf21, gf22");
        return 0;
    }
    long long state_len() const { return gbc::layout_of(N, ne, dila).n; }
};

