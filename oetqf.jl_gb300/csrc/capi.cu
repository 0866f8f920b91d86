// extern "C" entry points of libgbcycle.so (declared in include/gbcycle.h): argument checks in
// the reference's terms, device buffers behind opaque model handles, one stream per model.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "gbc_internal.cuh"
#include "integrator.cuh"
#include "model.cuh"
#include "rhs.cuh"

namespace gbc {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? GBC_ENOMEM : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? GBC_ENODEV : GBC_ECUDA;
}

int set_smem_limit(const void* fn, int bytes) {
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> done;  // (kernel, device) -> limit set
    std::lock_guard<std::mutex> lk(mu);
    int& have = done[std::make_pair(fn, dev)];
    if (have >= bytes) return 0;
    GBC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    have = bytes;
    return 0;
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kSMs;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = kSMs;
        cached[dev] = n;
    }
    return cached[dev];
}

static int check_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(GBC_ENODEV, "no CUDA device available (libgbcycle has no CPU fallback)");
    return 0;
}

// col-major (R x C) source -> row-major destination with leading dimension ld
__global__ void k_cm_to_rm(const double* __restrict__ src, long long R, long long C, double* __restrict__ dst, size_t ld) {
    __shared__ double tile[32][33];
    const long long r0 = (long long)blockIdx.y * 32, c0 = (long long)blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const long long c = c0 + k, r = r0 + threadIdx.x;
        tile[k][threadIdx.x] = (r < R && c < C) ? src[r + R * c] : 0.0;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const long long r = r0 + k, c = c0 + threadIdx.x;
        if (r < R && c < C) dst[(size_t)r * ld + c] = tile[threadIdx.x][k];
    }
}

__global__ void k_rm_to_cm(const double* __restrict__ src, size_t ld, long long R, long long C, double* __restrict__ dst) {
    __shared__ double tile[32][33];
    const long long r0 = (long long)blockIdx.y * 32, c0 = (long long)blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const long long r = r0 + k, c = c0 + threadIdx.x;
        tile[k][threadIdx.x] = (r < R && c < C) ? src[(size_t)r * ld + c] : 0.0;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const long long c = c0 + k, r = r0 + threadIdx.x;
        if (r < R && c < C) dst[r + R * c] = tile[threadIdx.x][k];
    }
}

static int cm_to_rm(const double* src, long long R, long long C, double* dst, size_t ld, cudaStream_t s) {
    if (R == 0 || C == 0) return 0;
    dim3 grid((unsigned)((C + 31) / 32), (unsigned)((R + 31) / 32)), block(32, 8);
    k_cm_to_rm<<<grid, block, 0, s>>>(src, R, C, dst, ld);
    GBC_CUDA(cudaGetLastError());
    return 0;
}
static int rm_to_cm(const double* src, size_t ld, long long R, long long C, double* dst, cudaStream_t s) {
    if (R == 0 || C == 0) return 0;
    dim3 grid((unsigned)((C + 31) / 32), (unsigned)((R + 31) / 32)), block(32, 8);
    k_rm_to_cm<<<grid, block, 0, s>>>(src, ld, R, C, dst);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

static std::atomic<long long> g_launches{0};

void count_launches(long long n) { g_launches += n; }

}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return (int)g_err.size();
    size_t n = std::min(len - 1, g_err.size());
    memcpy(buf, g_err.data(), n);
    buf[n] = 0;
    return (int)g_err.size();
}

const char* gbc_version(void) { return "gbcycle 0.1 (sm_103a)"; }

long long gbc_kernel_launches(void) { return g_launches.load(); }

// ---- Green's functions ------------------------------------------------------------------------
static int fault_dev(const gbc_fault_mesh* mf, std::vector<DevBuf>& keep, FaultDev& f, cudaStream_t s) {
    if (!mf || mf->nx <= 0 || mf->nxi <= 0 || !mf->x || !mf->y || !mf->z || !mf->ax || !mf->axi)
        return fail(GBC_EINVAL, "invalid fault mesh");
    keep.resize(keep.size() + 5);
    DevBuf* k = &keep[keep.size() - 5];
    if (int rc = upload(k[0], mf->x, mf->nx, s)) return rc;
    if (int rc = upload(k[1], mf->y, mf->nxi, s)) return rc;
    if (int rc = upload(k[2], mf->z, mf->nxi, s)) return rc;
    if (int rc = upload(k[3], mf->ax, 2 * (size_t)mf->nx, s)) return rc;
    if (int rc = upload(k[4], mf->axi, 2 * (size_t)mf->nxi, s)) return rc;
    for (int j = 0; j < mf->nxi; ++j)
        if (mf->z[j] > 0) return fail(GBC_EINVAL, "fault receivers must lie at z <= 0");
    f = FaultDev{mf->nx, mf->nxi, k[0].p, k[1].p, k[2].p, k[3].p, k[4].p, mf->dx, mf->dep, mf->dip};
    return 0;
}

static int hex_dev(const gbc_hex_mesh* ma, std::vector<DevBuf>& keep, HexDev& h, cudaStream_t s) {
    if (!ma || ma->ne <= 0) return fail(GBC_EINVAL, "invalid hex mesh");
    const double* src[9] = {ma->cx, ma->cy, ma->cz, ma->qx, ma->qy, ma->qz, ma->dx, ma->dy, ma->dz};
    keep.resize(keep.size() + 9);
    DevBuf* k = &keep[keep.size() - 9];
    for (int i = 0; i < 9; ++i) {
        if (!src[i]) return fail(GBC_EINVAL, "invalid hex mesh (null field)");
        if (int rc = upload(k[i], src[i], ma->ne, s)) return rc;
    }
    for (int i = 0; i < ma->ne; ++i)
        if (ma->qz[i] > 0 || ma->dx[i] <= 0 || ma->dy[i] <= 0 || ma->dz[i] <= 0)
            return fail(GBC_EINVAL, "hex cells must lie below the surface with positive sizes");
    h = HexDev{ma->ne, k[0].p, k[1].p, k[2].p, k[3].p, k[4].p, k[5].p, k[6].p, k[7].p, k[8].p};
    return 0;
}

static int quad_dev(const double* qc, const double* qw, int nq, std::vector<DevBuf>& keep,
                    const double*& dqc, const double*& dqw, cudaStream_t s) {
    static const double c0[3] = {0, 0, 0}, w0[1] = {1};
    if (nq <= 0 || !qc || !qw) { qc = c0; qw = w0; nq = 1; }
    keep.resize(keep.size() + 2);
    DevBuf* k = &keep[keep.size() - 2];
    if (int rc = upload(k[0], qc, 3 * (size_t)nq, s)) return rc;
    if (int rc = upload(k[1], qw, nq, s)) return rc;
    dqc = k[0].p;
    dqw = k[1].p;
    return 0;
}

int gbc_stress_gf_ff(const gbc_fault_mesh* mf, double lambda, double mu, int ftype, int fourier,
                     int nrept, double buffer_ratio, double* out) {
    if (int rc = check_device()) return rc;
    if (!(buffer_ratio >= 0)) return fail(GBC_EINVAL, "Argument `buffer_ratio` must be ≥ 0.");
    if (ftype != GBC_STRIKE_SLIP && ftype != GBC_DIP_SLIP) return fail(GBC_EINVAL, "unknown fault type");
    if (nrept < 0 || !out) return fail(GBC_EINVAL, "invalid nrept or output");
    std::vector<DevBuf> keep;
    keep.reserve(16);
    FaultDev f;
    if (int rc = fault_dev(mf, keep, f, 0)) return rc;
    const size_t n = (size_t)mf->nx * mf->nxi * mf->nxi;
    DevBuf st, dft;
    if (int rc = st.alloc(n)) return rc;
    if (int rc = launch_gf_ff(f, lambda, mu, ftype, nrept, buffer_ratio, st.p, 0)) return rc;
    g_launches += 1;
    const double* res = st.p;
    size_t count = n;
    if (fourier) {
        if (int rc = dft.alloc(2 * n)) return rc;
        if (int rc = launch_gf_ff_dft(mf->nx, mf->nxi, st.p, dft.p, 0)) return rc;
        g_launches += 1;
        res = dft.p;
        count = 2 * n;
    }
    GBC_CUDA(cudaMemcpy(out, res, sizeof(double) * count, cudaMemcpyDeviceToHost));
    return 0;
}

int gbc_stress_gf_fm(const gbc_fault_mesh* mf, const gbc_hex_mesh* ma, double lambda, double mu, int ftype,
                     const double* qcoords, const double* qweights, int nq, int nrept, double buffer_ratio,
                     double* out) {
    if (int rc = check_device()) return rc;
    if (!(buffer_ratio >= 0)) return fail(GBC_EINVAL, "Argument `buffer_ratio` must be ≥ 0.");
    if (ftype != GBC_STRIKE_SLIP && ftype != GBC_DIP_SLIP) return fail(GBC_EINVAL, "unknown fault type");
    if (nq > 0 && (!qcoords || !qweights)) return fail(GBC_EINVAL, "Wrong format of quadrature!");
    if (!out) return fail(GBC_EINVAL, "null output");
    std::vector<DevBuf> keep;
    keep.reserve(32);
    FaultDev f;
    HexDev h;
    const double *qc, *qw;
    if (int rc = fault_dev(mf, keep, f, 0)) return rc;
    if (int rc = hex_dev(ma, keep, h, 0)) return rc;
    if (int rc = quad_dev(qcoords, qweights, nq, keep, qc, qw, 0)) return rc;
    const long long R = 6LL * ma->ne, C = (long long)mf->nx * mf->nxi;
    DevBuf rm, cm;
    if (int rc = rm.alloc((size_t)(R * C))) return rc;
    if (int rc = cm.alloc((size_t)(R * C))) return rc;
    if (int rc = launch_gf_fm(f, h, lambda, mu, ftype, nrept, buffer_ratio, qc, qw, nq > 0 ? nq : 1, rm.p, (size_t)C, 0)) return rc;
    if (int rc = rm_to_cm(rm.p, (size_t)C, R, C, cm.p, 0)) return rc;
    g_launches += 2;
    GBC_CUDA(cudaMemcpy(out, cm.p, sizeof(double) * R * C, cudaMemcpyDeviceToHost));
    return 0;
}

int gbc_stress_gf_mf(const gbc_hex_mesh* ma, const gbc_fault_mesh* mf, double lambda, double mu, int ftype,
                     double* out) {
    if (int rc = check_device()) return rc;
    if (ftype != GBC_STRIKE_SLIP && ftype != GBC_DIP_SLIP) return fail(GBC_EINVAL, "unknown fault type");
    if (!out) return fail(GBC_EINVAL, "null output");
    std::vector<DevBuf> keep;
    keep.reserve(32);
    FaultDev f;
    HexDev h;
    if (int rc = fault_dev(mf, keep, f, 0)) return rc;
    if (int rc = hex_dev(ma, keep, h, 0)) return rc;
    const long long R = (long long)mf->nx * mf->nxi, C = 6LL * ma->ne;
    DevBuf rm, cm;
    if (int rc = rm.alloc((size_t)(R * C))) return rc;
    if (int rc = cm.alloc((size_t)(R * C))) return rc;
    if (int rc = launch_gf_mf(h, f, lambda, mu, ftype, rm.p, (size_t)C, 0)) return rc;
    if (int rc = rm_to_cm(rm.p, (size_t)C, R, C, cm.p, 0)) return rc;
    g_launches += 2;
    GBC_CUDA(cudaMemcpy(out, cm.p, sizeof(double) * R * C, cudaMemcpyDeviceToHost));
    return 0;
}

int gbc_hex_mesh_grid(const gbc_hex_mesh* ma, int* nX, int* nY, int* nZ) {
    if (!ma || ma->ne <= 0) return 0;
    MMGrid g;
    if (!mm_grid(ma, g)) return 0;
    if (nX) *nX = g.nX;
    if (nY) *nY = g.nY;
    if (nZ) *nZ = g.nZ;
    return 1;
}

int gbc_stress_gf_mm(const gbc_hex_mesh* ma, double lambda, double mu, const double* qcoords,
                     const double* qweights, int nq, double* out) {
    if (int rc = check_device()) return rc;
    if (nq > 0 && (!qcoords || !qweights)) return fail(GBC_EINVAL, "Wrong format of quadrature!");
    if (!out) return fail(GBC_EINVAL, "null output");
    std::vector<DevBuf> keep;
    keep.reserve(32);
    HexDev h;
    const double *qc, *qw;
    if (int rc = hex_dev(ma, keep, h, 0)) return rc;
    if (int rc = quad_dev(qcoords, qweights, nq, keep, qc, qw, 0)) return rc;
    const long long R = 6LL * ma->ne;
    DevBuf rm, cm;
    if (int rc = rm.alloc((size_t)(R * R))) return rc;
    if (int rc = cm.alloc((size_t)(R * R))) return rc;
    MMGrid grid;
    const bool structured = mm_grid(ma, grid);
    if (int rc = launch_gf_mm(h, lambda, mu, qc, qw, nq > 0 ? nq : 1, rm.p, (size_t)R, 0, structured ? &grid : nullptr))
        return rc;
    if (int rc = rm_to_cm(rm.p, (size_t)R, R, R, cm.p, 0)) return rc;
    g_launches += 2;
    GBC_CUDA(cudaMemcpy(out, cm.p, sizeof(double) * R * R, cudaMemcpyDeviceToHost));
    return 0;
}

// ---- models -------------------------------------------------------------------------------------
int gbc_model_create(int nx, int nxi, int ne, gbc_model** out) {
    if (!out) return fail(GBC_EINVAL, "null output handle");
    *out = nullptr;
    if (nx <= 0 || nxi <= 0 || ne < 0) return fail(GBC_EINVAL, "model sizes must be positive (ne >= 0)");
    if (int rc = check_device()) return rc;
    gbc_model* m = new gbc_model();
    m->nx = nx; m->nxi = nxi; m->ne = ne; m->N = nx * nxi;
    m->npad = (m->N + 31) / 32 * 32;
    m->M = 6LL * ne;
    m->ldm = (size_t)((m->npad + m->M + 31) / 32 * 32);
    m->ld21 = (size_t)((m->M + 31) / 32 * 32);
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    int rc = 0;
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
    if (!rc) rc = m->st.alloc((size_t)nx * nxi * nxi);
    if (!rc) rc = m->xm.alloc((size_t)(m->npad + m->M));
    if (!rc) rc = m->u.alloc((size_t)m->state_len());
    if (!rc) rc = m->du.alloc((size_t)m->state_len());
    if (!rc && ne > 0) rc = m->gm.alloc((size_t)m->M * m->ldm);
    if (!rc && ne > 0) rc = m->g21.alloc((size_t)m->N * m->ld21);
    if (!rc) {
        e = cudaMemsetAsync(m->xm.p, 0, sizeof(double) * m->xm.n, m->stream);
        if (e == cudaSuccess && ne > 0) e = cudaMemsetAsync(m->gm.p, 0, sizeof(double) * m->gm.n, m->stream);
        if (e == cudaSuccess && ne > 0) e = cudaMemsetAsync(m->g21.p, 0, sizeof(double) * m->g21.n, m->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemset");
    }
    if (rc) {
        gbc_model_destroy(m);
        return rc;
    }
    *out = m;
    return 0;
}

void gbc_model_destroy(gbc_model* m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    integrator_free(m->integ);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

long long gbc_model_state_len(const gbc_model* m) { return m ? m->state_len() : 0; }

void* gbc_model_stream(gbc_model* m) { return m ? (void*)m->stream : nullptr; }

int gbc_model_set_fault_props(gbc_model* m, const double* a, const double* b, const double* L,
                              const double* sigma, double eta, double vpl, double f0, double v0) {
    if (!m || !a || !b || !L || !sigma) return fail(GBC_EINVAL, "null argument");
    if (!(f0 > 0)) return fail(GBC_EINVAL, "AssertionError: f₀ > 0");
    if (!(v0 > 0)) return fail(GBC_EINVAL, "AssertionError: v₀ > 0");
    if (!(eta > 0)) return fail(GBC_EINVAL, "AssertionError: η > 0");
    if (!(vpl > 0)) return fail(GBC_EINVAL, "AssertionError: vpl > 0");
    cudaStream_t s = m->stream;
    if (int rc = upload(m->a, a, m->N, s)) return rc;
    if (int rc = upload(m->b, b, m->N, s)) return rc;
    if (int rc = upload(m->L, L, m->N, s)) return rc;
    if (int rc = upload(m->sig, sigma, m->N, s)) return rc;
    GBC_CUDA(cudaStreamSynchronize(s));
    m->eta = eta; m->vpl = vpl; m->f0 = f0; m->v0 = v0;
    m->props = true;
    return 0;
}

int gbc_model_set_mantle_props(gbc_model* m, const double* gamma, const double* n, const double* deps0) {
    return gbc_model_set_mantle_props_composite(m, 1, gamma, n, deps0);
}

int gbc_model_set_mantle_props_composite(gbc_model* m, int nlaws, const double* gamma, const double* n,
                                         const double* deps0) {
    if (!m || !gamma || !n || !deps0) return fail(GBC_EINVAL, "null argument");
    if (m->ne == 0) return fail(GBC_EINVAL, "fault-only model has no mantle");
    if (nlaws < 1) return fail(GBC_EINVAL, "a composite viscosity needs at least one law");
    cudaStream_t s = m->stream;
    if (int rc = upload(m->gamma, gamma, (size_t)nlaws * m->ne, s)) return rc;
    if (int rc = upload(m->nexp, n, (size_t)nlaws * m->ne, s)) return rc;
    GBC_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < 6; ++k) m->deps0[k] = deps0[k];
    m->nlaws = nlaws;
    m->mprops = true;
    return 0;
}

int gbc_model_set_dilatancy(gbc_model* m, const double* tp, const double* eps, const double* beta, const double* p0) {
    if (!m || !tp || !eps || !beta || !p0) return fail(GBC_EINVAL, "null argument");
    if (m->ne != 0) return fail(GBC_EINVAL, "dilatancy applies to fault-only models (equation.jl:168-183)");
    cudaStream_t s = m->stream;
    if (int rc = upload(m->tp, tp, m->N, s)) return rc;
    if (int rc = upload(m->deps_d, eps, m->N, s)) return rc;
    if (int rc = upload(m->beta_d, beta, m->N, s)) return rc;
    if (int rc = upload(m->p0, p0, m->N, s)) return rc;
    m->dila = 1;
    if (int rc = m->u.alloc((size_t)m->state_len())) return rc;
    if (int rc = m->du.alloc((size_t)m->state_len())) return rc;
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_model_set_gf(gbc_model* m, int which, const double* host) {
    if (!m || !host) return fail(GBC_EINVAL, "null argument");
    cudaStream_t s = m->stream;
    const size_t nst = (size_t)m->nx * m->nxi * m->nxi;
    DevBuf tmp;
    switch (which) {
        case GBC_GF11_REAL:
            GBC_CUDA(cudaMemcpyAsync(m->st.p, host, sizeof(double) * nst, cudaMemcpyHostToDevice, s));
            m->has_st = true;
            break;
        case GBC_GF11_DFT:
            if (int rc = upload(tmp, host, 2 * nst, s)) return rc;
            if (int rc = launch_gf_ff_idft(m->nx, m->nxi, tmp.p, m->st.p, s)) return rc;
            g_launches += 1;
            m->has_st = true;
            break;
        case GBC_GF12:
        case GBC_GF21:
        case GBC_GF22: {
            if (m->ne == 0) return fail(GBC_EINVAL, "fault-only model has no mantle Green's functions");
            const long long R = (which == GBC_GF21) ? m->N : m->M;
            const long long C = (which == GBC_GF12) ? m->N : m->M;
            if (int rc = upload(tmp, host, (size_t)(R * C), s)) return rc;
            double* dst = (which == GBC_GF21) ? m->g21.p : (which == GBC_GF12) ? m->gm.p : m->gm.p + m->npad;
            const size_t ld = (which == GBC_GF21) ? m->ld21 : m->ldm;
            if (int rc = cm_to_rm(tmp.p, R, C, dst, ld, s)) return rc;
            g_launches += 1;
            (which == GBC_GF12 ? m->has_g12 : which == GBC_GF21 ? m->has_g21 : m->has_g22) = true;
            break;
        }
        default:
            return fail(GBC_EINVAL, "unknown Green's function id");
    }
    m->mixed_dirty = true;
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_model_export_gf(gbc_model* m, int which, double* host) {
    if (!m || !host) return fail(GBC_EINVAL, "null argument");
    cudaStream_t s = m->stream;
    const size_t nst = (size_t)m->nx * m->nxi * m->nxi;
    DevBuf tmp;
    switch (which) {
        case GBC_GF11_REAL:
            if (!m->has_st) return fail(GBC_ESTATE, "gf11 not set");
            GBC_CUDA(cudaMemcpyAsync(host, m->st.p, sizeof(double) * nst, cudaMemcpyDeviceToHost, s));
            break;
        case GBC_GF11_DFT:
            if (!m->has_st) return fail(GBC_ESTATE, "gf11 not set");
            if (int rc = tmp.alloc(2 * nst)) return rc;
            if (int rc = launch_gf_ff_dft(m->nx, m->nxi, m->st.p, tmp.p, s)) return rc;
            g_launches += 1;
            GBC_CUDA(cudaMemcpyAsync(host, tmp.p, sizeof(double) * 2 * nst, cudaMemcpyDeviceToHost, s));
            break;
        case GBC_GF12:
        case GBC_GF21:
        case GBC_GF22: {
            if (m->ne == 0) return fail(GBC_EINVAL, "fault-only model has no mantle Green's functions");
            const long long R = (which == GBC_GF21) ? m->N : m->M;
            const long long C = (which == GBC_GF12) ? m->N : m->M;
            const double* src = (which == GBC_GF21) ? m->g21.p : (which == GBC_GF12) ? m->gm.p : m->gm.p + m->npad;
            const size_t ld = (which == GBC_GF21) ? m->ld21 : m->ldm;
            if (int rc = tmp.alloc((size_t)(R * C))) return rc;
            if (int rc = rm_to_cm(src, ld, R, C, tmp.p, s)) return rc;
            g_launches += 1;
            GBC_CUDA(cudaMemcpyAsync(host, tmp.p, sizeof(double) * R * C, cudaMemcpyDeviceToHost, s));
            break;
        }
        default:
            return fail(GBC_EINVAL, "unknown Green's function id");
    }
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_model_export_gf_rows(gbc_model* m, int which, int nrows, const int* rows, double* host) {
    if (!m || !host || (nrows > 0 && !rows) || nrows < 0) return fail(GBC_EINVAL, "null argument");
    if (which != GBC_GF12 && which != GBC_GF21 && which != GBC_GF22)
        return fail(GBC_EINVAL, "row export covers GBC_GF12, GBC_GF21 and GBC_GF22");
    if (m->ne == 0) return fail(GBC_EINVAL, "fault-only model has no mantle Green's functions");
    if ((which == GBC_GF12 && !m->has_g12) || (which == GBC_GF21 && !m->has_g21) || (which == GBC_GF22 && !m->has_g22))
        return fail(GBC_ESTATE, "Green's function not set");
    // the device keeps these blocks row-major with the reference's row numbering, so a row is one
    // contiguous run: G12 row r = gm[r, 0:N), G22 row r = gm[r, npad:npad+M), G21 row i = g21[i, 0:M)
    const long long R = (which == GBC_GF21) ? m->N : m->M;
    const long long C = (which == GBC_GF12) ? m->N : m->M;
    const double* src = (which == GBC_GF21) ? m->g21.p : (which == GBC_GF12) ? m->gm.p : m->gm.p + m->npad;
    const size_t ld = (which == GBC_GF21) ? m->ld21 : m->ldm;
    for (int k = 0; k < nrows; ++k)
        if (rows[k] < 0 || rows[k] >= R) return fail(GBC_EINVAL, "row index out of range");
    cudaStream_t s = m->stream;
    for (int k = 0; k < nrows; ++k)
        GBC_CUDA(cudaMemcpyAsync(host + (size_t)k * C, src + (size_t)rows[k] * ld, sizeof(double) * C,
                                 cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_model_assemble(gbc_model* m, const gbc_fault_mesh* mf, const gbc_hex_mesh* ma, double lambda, double mu,
                       int ftype, int nrept, double buffer_ratio, const double* qcoords, const double* qweights,
                       int nq) {
    if (!m) return fail(GBC_EINVAL, "null model");
    if (!(buffer_ratio >= 0)) return fail(GBC_EINVAL, "Argument `buffer_ratio` must be ≥ 0.");
    if (ftype != GBC_STRIKE_SLIP && ftype != GBC_DIP_SLIP) return fail(GBC_EINVAL, "unknown fault type");
    if (!mf || mf->nx != m->nx || mf->nxi != m->nxi) return fail(GBC_EINVAL, "fault mesh does not match the model");
    if (m->ne > 0 && (!ma || ma->ne != m->ne)) return fail(GBC_EINVAL, "hex mesh does not match the model");
    cudaStream_t s = m->stream;
    std::vector<DevBuf> keep;
    keep.reserve(32);
    FaultDev f;
    if (int rc = fault_dev(mf, keep, f, s)) return rc;
    if (int rc = launch_gf_ff(f, lambda, mu, ftype, nrept, buffer_ratio, m->st.p, s)) return rc;
    g_launches += 1;
    m->has_st = true;
    if (m->ne > 0) {
        HexDev h;
        const double *qc, *qw;
        if (int rc = hex_dev(ma, keep, h, s)) return rc;
        if (int rc = quad_dev(qcoords, qweights, nq, keep, qc, qw, s)) return rc;
        if (int rc = launch_gf_fm(f, h, lambda, mu, ftype, nrept, buffer_ratio, qc, qw, nq > 0 ? nq : 1, m->gm.p, m->ldm, s)) return rc;
        if (int rc = launch_gf_mf(h, f, lambda, mu, ftype, m->g21.p, m->ld21, s)) return rc;
        MMGrid grid;
        const bool structured = mm_grid(ma, grid);
        if (int rc = launch_gf_mm(h, lambda, mu, qc, qw, nq > 0 ? nq : 1, m->gm.p + m->npad, m->ldm, s,
                                  structured ? &grid : nullptr))
            return rc;
        g_launches += 3;
        m->has_g12 = m->has_g21 = m->has_g22 = true;
    }
    m->mixed_dirty = true;
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

int gbc_model_set_precision(gbc_model* m, int mode) {
    if (!m) return fail(GBC_EINVAL, "null model");
    if (mode != GBC_PREC_F64 && mode != GBC_PREC_BF16 && mode != GBC_PREC_F16 && mode != GBC_PREC_DF64)
        return fail(GBC_EINVAL, "unknown precision mode");
    if (mode != m->precision) m->mixed_dirty = true;
    m->precision = mode;
    return 0;
}

int gbc_model_set_log_theta(gbc_model* m, int on) {
    if (!m) return fail(GBC_EINVAL, "null model");
    m->log_theta = on ? 1 : 0;
    return 0;
}

int gbc_model_error_word(gbc_model* m) {
    if (!m || !m->err.p) return 0;
    int h = 0;
    if (cudaMemcpy(&h, m->err.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h;
}

int gbc_model_clear_error_word(gbc_model* m) {
    if (!m) return fail(GBC_EINVAL, "null model");
    if (!m->err.p) return 0;
    GBC_CUDA(cudaMemsetAsync(m->err.p, 0, sizeof(int), m->stream));
    GBC_CUDA(cudaStreamSynchronize(m->stream));
    return 0;
}

int gbc_debug_pipeline_fault(int mode) {
    if (mode != 0 && mode != 1) return fail(GBC_EINVAL, "gbc_debug_pipeline_fault: mode must be 0 or 1");
    return set_pipeline_fault(mode);
}

int gbc_rhs_dev(gbc_model* m, double t, const double* u, double* du) {
    (void)t;
    if (!m || !u || !du) return fail(GBC_EINVAL, "null argument");
    if (int rc = m->ready()) return rc;
    if (int rc = m->prepare()) return rc;
    if (int rc = launch_rhs(m->args(), u, du, m->stream)) return rc;
    g_launches += rhs_kernel_count(m->args());
    return 0;
}

int gbc_rhs(gbc_model* m, double t, const double* const* u_parts, double* const* du_parts, int nparts) {
    if (!m || !u_parts || !du_parts) return fail(GBC_EINVAL, "null argument");
    const int want = m->ne > 0 ? 5 : (m->dila ? 4 : 3);
    if (nparts != want) return fail(GBC_EINVAL, "ArrayPartition must have " + std::to_string(want) + " components");
    if (int rc = m->ready()) return rc;
    if (int rc = m->prepare()) return rc;
    const long long N = m->N, E = m->M;
    long long len[5] = {N, N, N, N, 0};
    if (want == 5) { len[2] = E; len[3] = E; len[4] = N; }
    cudaStream_t s = m->stream;
    long long off = 0;
    for (int p = 0; p < want; ++p) {
        if (!u_parts[p] || !du_parts[p]) return fail(GBC_EINVAL, "null ArrayPartition component");
        GBC_CUDA(cudaMemcpyAsync(m->u.p + off, u_parts[p], sizeof(double) * len[p], cudaMemcpyHostToDevice, s));
        off += len[p];
    }
    if (int rc = launch_rhs(m->args(), m->u.p, m->du.p, s)) return rc;
    g_launches += rhs_kernel_count(m->args());
    off = 0;
    for (int p = 0; p < want; ++p) {
        GBC_CUDA(cudaMemcpyAsync(du_parts[p], m->du.p + off, sizeof(double) * len[p], cudaMemcpyDeviceToHost, s));
        off += len[p];
    }
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

__global__ void k_theta_transform(double* th, int n, int to_log) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        th[i] = to_log ? log(th[i]) : exp(th[i]);
}

static int theta_transform(double* th, int n, int to_log, cudaStream_t s) {
    k_theta_transform<<<(n + 255) / 256, 256, 0, s>>>(th, n, to_log);
    GBC_CUDA(cudaGetLastError());
    g_launches += 1;
    return 0;
}

static int integrate_common(gbc_model* m, double* u_dev, double t0, double t1, const gbc_solver_opts* o,
                            gbc_solver_stats* st, Recorder* rec = nullptr) {
    if (!o) return fail(GBC_EINVAL, "null solver options");
    if (!(o->reltol > 0) || !(o->abstol >= 0) || !(o->dt0 > 0) || !(o->dtmax > 0) || o->maxiters <= 0)
        return fail(GBC_EINVAL, "invalid solver options");
    if (int rc = m->ready()) return rc;
    if (int rc = m->prepare()) return rc;
    if (int rc = integrator_alloc(m->integ, m->state_len())) return rc;
    RhsArgs args = m->args();
    args.log_theta = m->dila ? 0 : m->log_theta;
    if (args.log_theta) {
        if (int rc = theta_transform(u_dev + m->N, m->N, 1, m->stream)) return rc;
    }
    int rc = integrator_run(m->integ, args, u_dev, t0, t1, o->reltol, o->abstol, o->dt0, o->dtmax,
                            o->dtmin, o->maxiters, m->stream, rec, o->alg);
    if (args.log_theta) {
        if (int rc2 = theta_transform(u_dev + m->N, m->N, 0, m->stream)) return rc2;
    }
    const Ctrl& c = *m->integ.ctrl_host;
    // kernels enqueued: the FSAL seed RHS, then every kernel node of every graph launch (steps
    // past completion return at once but still count as launches)
    const int rhs_k = rhs_kernel_count(args);
    const long long per_step = 6LL * (1 + rhs_k) + 3;
    g_launches += rhs_k + m->integ.graph_launches * m->integ.steps_per_launch * per_step;
    if (st) {
        st->naccept = c.naccept;
        st->nreject = c.nreject;
        st->nrhs = c.nrhs + 1;
        st->t = c.t;
        st->dt = c.dt;
        st->status = c.status;
    }
    if (rc > 0) rc = 0;
    if (rc == 0 && c.status != 0) return fail(GBC_ESOLVER, "integration stopped early (dt < dtmin, maxiters or non-finite state)");
    return rc;
}

int gbc_integrate_dev(gbc_model* m, double* u_dev, double t0, double t1, const gbc_solver_opts* o,
                      gbc_solver_stats* st) {
    if (!m || !u_dev) return fail(GBC_EINVAL, "null argument");
    return integrate_common(m, u_dev, t0, t1, o, st);
}

int gbc_integrate_record(gbc_model* m, double* u, double t0, double t1, const gbc_solver_opts* o, int stride,
                         long long max_records, double* t_out, double* u_out, long long* nrec, gbc_solver_stats* st) {
    if (!m || !u || !t_out || !u_out || !nrec) return fail(GBC_EINVAL, "null argument");
    if (stride < 1 || max_records < 1) return fail(GBC_EINVAL, "stride and max_records must be positive");
    const long long n = m->state_len();
    // record 0: the initial state (the reference's callback also fires at t0)
    t_out[0] = t0;
    memcpy(u_out, u, sizeof(double) * n);
    GBC_CUDA(cudaMemcpyAsync(m->u.p, u, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    Recorder rec;
    rec.stride = stride;
    rec.max_records = max_records;
    rec.t_out = t_out;
    rec.u_out = u_out;
    int rc = integrate_common(m, m->u.p, t0, t1, o, st, &rec);
    *nrec = std::min(max_records, rec.drained + 1);
    if (rc != 0 && rc != GBC_ESOLVER) return rc;
    GBC_CUDA(cudaMemcpyAsync(u, m->u.p, sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
    GBC_CUDA(cudaStreamSynchronize(m->stream));
    return rc;
}

int gbc_integrate(gbc_model* m, double* u, double t0, double t1, const gbc_solver_opts* o, gbc_solver_stats* st) {
    if (!m || !u) return fail(GBC_EINVAL, "null argument");
    const long long n = m->state_len();
    GBC_CUDA(cudaMemcpyAsync(m->u.p, u, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    int rc = integrate_common(m, m->u.p, t0, t1, o, st);
    if (rc != 0 && rc != GBC_ESOLVER) return rc;
    GBC_CUDA(cudaMemcpyAsync(u, m->u.p, sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
    GBC_CUDA(cudaStreamSynchronize(m->stream));
    return rc;
}

}  // extern "C"
