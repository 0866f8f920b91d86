// gbc_rhs_visco_noalloc: the viscoelastic right-hand side for callers that cannot allocate device
// memory when they evaluate it. Typical cases: a caller that evaluates the RHS while another
// library is capturing its CUDA stream into a graph (cudaMalloc is not permitted during capture),
// a host process whose device memory is owned and accounted by its own pool (an ODE solver that
// sizes every buffer up front and then calls the RHS millions of times), and foreign-language
// bindings that can only hand over raw device pointers. The caller passes every input and output;
// the one scratch vector the RHS needs lives in the fixed array below.
#include <cuda_runtime.h>

#include <mutex>

#include "gbc_internal.cuh"
#include "rhs.cuh"

namespace gbc {

// Scratch vector x = [v - vpl (N); 0 (npad - N); dϵ - dϵ₀ (6ne)] of the no-allocation RHS. Every
// GPU that loads this library holds these 8 MiB until the process exits. All calls share it, so
// calls whose work overlaps on the GPU (different streams, or different host threads) race.
constexpr long long kNoAllocScratch = 1LL << 20;  // doubles
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratch];

// Device address of the array above, looked up once per device with that device current. A host
// reference to g_noalloc_scratch is only a host-side stand-in and must never reach a kernel.
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(double** out) {
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(GBC_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        GBC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return 0;
}

void count_launches(long long n);

}  // namespace gbc

using namespace gbc;

extern "C" int gbc_rhs_visco_noalloc(int nx, int nxi, int ne, const double* st, const double* gm, size_t ldm,
                                     const double* g21, size_t ld21, const double* a, const double* b,
                                     const double* L, const double* sigma, double eta, double vpl, double f0,
                                     double v0, const double* gamma, const double* n, const double* deps0,
                                     const double* u, double* du, void* stream) {
    if (nx <= 0 || nxi <= 0 || ne <= 0) return fail(GBC_EINVAL, "gbc_rhs_visco_noalloc: sizes must be positive");
    if (!st || !gm || !g21 || !a || !b || !L || !sigma || !gamma || !n || !deps0 || !u || !du)
        return fail(GBC_EINVAL, "gbc_rhs_visco_noalloc: null pointer argument");
    const long long N = (long long)nx * nxi, M = 6LL * ne;
    const long long npad = (N + 31) / 32 * 32;
    if (npad + M > kNoAllocScratch)
        return fail(GBC_EINVAL, "gbc_rhs_visco_noalloc: model too large for the fixed scratch (need npad + 6*ne <= "
                                    "1048576 doubles, npad = nx*nxi rounded up to 32)");
    if (ldm < (size_t)(npad + M) || ld21 < (size_t)M || (ldm & 1) || (ld21 & 1))
        return fail(GBC_EINVAL, "gbc_rhs_visco_noalloc: leading dimensions must be even and cover the rows");
    // the row GEMV reads gm and g21 as 16-byte pairs: an 8-byte-offset view (a slice of a larger
    // buffer) would be a misaligned access on the device, so refuse it here
    if ((reinterpret_cast<uintptr_t>(gm) | reinterpret_cast<uintptr_t>(g21)) & 15)
        return fail(GBC_EINVAL, "gbc_rhs_visco_noalloc: gm and g21 must be 16-byte aligned device pointers");
    if (!(eta > 0) || !(vpl > 0) || !(f0 > 0) || !(v0 > 0))
        return fail(GBC_EINVAL, "gbc_rhs_visco_noalloc: eta, vpl, f0, v0 must be positive");
    double* x = nullptr;
    if (int rc = noalloc_scratch(&x)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the array keeps the previous call's contents: zero the padding the GEMV reads
    if (npad > N) GBC_CUDA(cudaMemsetAsync(x + N, 0, sizeof(double) * (npad - N), s));
    RhsArgs r{};
    r.nx = nx; r.nxi = nxi; r.ne = ne; r.N = (int)N; r.npad = (int)npad;
    r.st = st; r.gm = gm; r.ldm = ldm; r.g21 = g21; r.ld21 = ld21;
    r.a = a; r.b = b; r.L = L; r.sig = sigma;
    r.eta = eta; r.vpl = vpl; r.f0 = f0; r.v0 = v0;
    r.gamma = gamma; r.nexp = n; r.nlaws = 1;
    for (int k = 0; k < 6; ++k) r.deps0[k] = deps0[k];  // host array, passed by value to the kernels
    r.xm = x;
    r.skip = nullptr;
    if (int rc = launch_rhs(r, u, du, s)) return rc;
    count_launches(2);
    return 0;
}
