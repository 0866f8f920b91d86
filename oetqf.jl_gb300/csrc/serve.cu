// Serving loop: a native scheduler thread that admits cycle-simulation requests by HBM budget and
// keeps their state on the device.
//  * Fault-only requests join a continuous batch: every scheduler iteration is one persistent
//    launch of the ensemble kernel over the active requests with a wall-clock budget; requests
//    that arrived meanwhile are assembled on a separate stream and join at the next iteration,
//    finished ones leave and free their memory. A request's trajectory does not depend on the
//    iteration boundaries or on the other requests (each model's step control state persists in
//    its descriptor), so results are bitwise the same alone and in the mix.
//  * Requests with a mantle run on their own model stream in a worker thread (block-scaled BF16
//    Green's functions; ln θ state under Tsit5, θ under VCABM5); their kernels overlap with the
//    batch on the device.
//  * Assembled Green's functions are cached on the device, keyed by the exact bytes of everything
//    they depend on (mesh, elastic constants, fault type, images, buffer ratio, quadrature and
//    storage precision): fault-only requests share one read-only spectrum buffer per geometry,
//    mantle requests take an idle assembled model of their geometry (its FP64 and 16-bit copies)
//    and skip assembly. Idle entries stay resident and count against the HBM budget; admission
//    evicts them least recently used first when the next request would not fit otherwise.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ensemble.cuh"
#include "gbc_internal.cuh"

namespace gbc {

struct Req {
    long long id = 0;
    // inputs (host copies)
    int nx = 0, nxi = 0, ne = 0;
    std::vector<double> fx, fxi, fy, fz, fax, faxi;
    double dx = 0, dxi = 0, dep = 0, dip = 90;
    std::vector<double> hex[9];
    double lambda = 0, mu = 0, buffer_ratio = 0;
    int nrept = 2, ftype = 0, precision = GBC_PREC_BF16;
    std::vector<double> a, b, L, sig, gamma, nexp;
    double eta = 0, vpl = 0, f0 = 0.6, v0 = 1e-6, deps0[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> qc, qw;
    std::vector<double> u0, u1;
    double t0 = 0, t1 = 0;
    gbc_solver_opts opts{};
    // bookkeeping: own bytes (state, properties) plus the Green's-function part, charged only when
    // the geometry is not cached
    size_t own = 0, gf = 0;
    std::string key;
    struct GfEntry* entry = nullptr;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int status = 0;
    bool done = false;
    gbc_solver_stats stats{};
    // device state of a batched (fault-only) request
    void* dmem = nullptr;
    EnsModel desc{};
    size_t smem = 0;
    // worker of a mantle request
    std::thread worker;
    bool worker_done = false;
};

// A cached geometry: the spectra of a fault-only geometry, or an assembled model with a mantle.
struct GfEntry {
    std::string key;
    bool mantle = false;
    bool valid = false;        // assembly finished successfully
    float* ghat = nullptr;     // fault-only
    gbc_model* model = nullptr;  // mantle: FP64 + storage-precision Green's functions, state buffers
    size_t bytes = 0;
    int refs = 0;
    double last = 0;
};

static void key_put(std::string& k, const void* p, size_t n) { k.append(static_cast<const char*>(p), n); }
static void key_vec(std::string& k, const std::vector<double>& v) {
    const size_t n = v.size();
    key_put(k, &n, sizeof(n));
    if (n) key_put(k, v.data(), sizeof(double) * n);
}
static std::string gf_key(const Req& r) {
    std::string k(1, r.ne > 0 ? 'M' : 'F');
    const int ints[5] = {r.nx, r.nxi, r.ne, r.ftype, r.nrept};
    const double d[7] = {r.dx, r.dxi, r.dep, r.dip, r.lambda, r.mu, r.buffer_ratio};
    key_put(k, ints, sizeof(ints));
    key_put(k, d, sizeof(d));
    for (const auto* v : {&r.fx, &r.fxi, &r.fy, &r.fz, &r.fax, &r.faxi}) key_vec(k, *v);
    if (r.ne > 0) {
        for (int j = 0; j < 9; ++j) key_vec(k, r.hex[j]);
        key_vec(k, r.qc);
        key_vec(k, r.qw);
        key_put(k, &r.precision, sizeof(r.precision));
    }
    return k;
}

}  // namespace gbc

using namespace gbc;

extern "C" void gbc_model_destroy(gbc_model*);

struct gbc_server {
    double budget = 0;
    size_t in_use = 0, peak = 0;
    gbc_solver_opts batch_opts{};
    int block = 512;
    unsigned long long slice_ns = 20000000ull;  // wall-clock budget of one batch iteration
    cudaStream_t batch = nullptr, admit = nullptr;
    EnsModel* d_desc = nullptr;
    int d_desc_cap = 0;
    EnsLaunch lp;
    std::mutex mu;
    std::condition_variable cv;       // new work / stop
    std::condition_variable done_cv;  // request finished
    std::deque<std::shared_ptr<Req>> queue;
    std::vector<std::shared_ptr<Req>> batch_active, mantle_active;
    std::map<long long, std::shared_ptr<Req>> all;
    long long next_id = 1;
    bool stop = false;
    std::thread sched;
    std::chrono::steady_clock::time_point t_start;
    long long iterations = 0;
    std::string fatal;
    std::vector<std::unique_ptr<GfEntry>> cache;
    bool cache_on = true;
    long long hits = 0, misses = 0;
    // evicted mantle models, destroyed by the reaper thread: freeing device memory waits for the
    // device's queued work (another request's assembly can be seconds), which the scheduler thread
    // must not do while it holds the lock or between batch iterations; the budget is a policy figure
    // below the device's memory, so a free that lands a little later is safe
    std::vector<gbc_model*> graveyard;
    std::condition_variable reap_cv;
    bool reap_stop = false;
    std::thread reaper;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
};

// own: properties, c1, b/a, 1/L (7N) and state, stages, candidate (30N); gf: the spectra plus the
// transient FP64 Toeplitz kernel and mesh they are computed from
static size_t fault_own_bytes(const EnsModel& m) { return sizeof(double) * 37 * (size_t)m.N + 4096; }
static size_t fault_gf_bytes(const Req& r, const EnsModel& m) {
    return sizeof(double) * ((size_t)m.nx * m.nxi * m.nxi + 3 * (size_t)r.nx + 4 * (size_t)r.nxi) +
           sizeof(float) * ens_ghat_floats(m) + 512;
}

static size_t mantle_bytes(const Req& r) {
    const size_t N = (size_t)r.nx * r.nxi, M = 6 * (size_t)r.ne;
    const size_t npad = (N + 31) / 32 * 32, ldm = (npad + M + 31) / 32 * 32, ld21 = (M + 31) / 32 * 32;
    const size_t rowsq = (M + 127) / 128 * 128 + (N + 127) / 128 * 128, ldq = (npad + M + 255) / 256 * 256;
    const size_t state = 3 * N + 2 * M;
    return 8 * (M * ldm + N * ld21 + (size_t)r.nx * r.nxi * r.nxi + 12 * state) + 2 * rowsq * ldq + (64 << 20);
}

// ---- fault-only requests: admission, batch iterations, completion -------------------------------
__global__ void k_theta_one(double* th, int n, int to_log) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        th[i] = to_log ? log(th[i]) : exp(th[i]);
}

static int admit_fault(gbc_server* s, Req& r) {
    EnsModel& m = r.desc;
    GfEntry* ge = r.entry;
    if (int rc = ens_prepare_model(m, r.nx, r.nxi, &r.smem)) return rc;
    const size_t N = m.N, nst = (size_t)r.nx * r.nxi * r.nxi, ng = ens_ghat_floats(m);
    cudaStream_t st = s->admit;
    auto up = [&](double* dd, const std::vector<double>& h) {
        return cudaMemcpyAsync(dd, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, st);
    };
    if (!ge->valid) {  // first request of this geometry: its spectra, from a transient FP64 kernel
        struct Tmp {  // released on every path, after the stream's work on it
            double* p = nullptr;
            cudaStream_t s;
            ~Tmp() { if (p) cudaFreeAsync(p, s); }
        } tg;
        tg.s = st;
        GBC_CUDA(cudaMallocAsync(&tg.p, sizeof(double) * (nst + 3 * (size_t)r.nx + 4 * (size_t)r.nxi), st));
        double* tmp = tg.p;
        GBC_CUDA(cudaMallocAsync(&ge->ghat, sizeof(float) * ng, st));
        double* mx = tmp + nst;  // mesh: x (nx), y, z (nxi), ax (2nx), axi (2nxi)
        double *my = mx + r.nx, *mz = my + r.nxi, *max_ = mz + r.nxi, *maxi = max_ + 2 * r.nx;
        cudaError_t e = cudaSuccess;
        for (auto pr : {std::make_pair(mx, &r.fx), std::make_pair(my, &r.fy), std::make_pair(mz, &r.fz),
                        std::make_pair(max_, &r.fax), std::make_pair(maxi, &r.faxi)})
            if (e == cudaSuccess) e = up(pr.first, *pr.second);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (mesh)");
        FaultDev f{r.nx, r.nxi, mx, my, mz, max_, maxi, r.dx, r.dep, r.dip};
        if (int rc = launch_gf_ff(f, r.lambda, r.mu, r.ftype, r.nrept, r.buffer_ratio, tmp, st)) return rc;
        if (int rc = ens_ghat(tmp, m, ge->ghat, st)) return rc;
        count_launches(2);
    }
    GBC_CUDA(cudaMallocAsync(&r.dmem, sizeof(double) * 37 * N + 256, st));
    double* pa = static_cast<double*>(r.dmem);
    double *pb = pa + N, *pL = pb + N, *ps = pL + N, *pc = ps + N, *pboa = pc + N, *piL = pboa + N;
    double* pu = piL + N;
    double* pk = pu + 3 * N;          // 7 x 3N
    double* py = pk + 21 * N;
    double* pun = py + 3 * N;
    std::vector<double> c1(N), boa(N), iL(N);
    for (size_t i = 0; i < N; ++i) {
        c1[i] = r.f0 / r.a[i] + (r.b[i] / r.a[i]) * std::log(r.v0 / r.L[i]) - std::log(2.0 * r.v0);
        boa[i] = r.b[i] / r.a[i];
        iL[i] = 1.0 / r.L[i];
    }
    cudaError_t e = cudaSuccess;
    for (auto pr : {std::make_pair(pa, &r.a), std::make_pair(pb, &r.b), std::make_pair(pL, &r.L),
                    std::make_pair(ps, &r.sig), std::make_pair(pu, &r.u0), std::make_pair(pc, &c1),
                    std::make_pair(pboa, &boa), std::make_pair(piL, &iL)})
        if (e == cudaSuccess) e = up(pr.first, *pr.second);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (admission)");
    // Tsit5 integrates ln θ; VCABM5 integrates θ itself
    const int lt = (s->batch_opts.alg == GBC_ALG_VCABM5) ? 0 : 1;
    if (lt) {
        k_theta_one<<<(int)((N + 255) / 256), 256, 0, st>>>(pu + N, (int)N, 1);
        GBC_CUDA(cudaGetLastError());
        count_launches(1);
    }
    GBC_CUDA(cudaStreamSynchronize(st));
    ge->valid = true;
    m.ghat = ge->ghat;
    m.a = pa; m.b = pb; m.L = pL; m.sig = ps; m.c1 = pc; m.boa = pboa; m.iL = piL;
    m.u = pu; m.y = py; m.un = pun;
    for (int k = 0; k < 7; ++k) m.k[k] = pk + 3 * N * k;
    m.eta = r.eta; m.vpl = r.vpl; m.f0 = r.f0; m.v0 = r.v0;
    m.t = r.t0; m.t1 = r.t1;
    m.dt = std::min(r.opts.dt0, r.opts.dtmax);
    if (m.dt > r.t1 - r.t0) m.dt = r.t1 - r.t0;
    m.qold = 1e-4;
    m.maxiters = r.opts.maxiters;
    m.done = (r.t1 <= r.t0) ? 1 : 0;
    m.log_theta = lt;
    m.logged = lt;
    return 0;
}

static void finish_fault(gbc_server* s, Req& r) {
    const EnsModel& m = r.desc;
    const int N = m.N;
    if (m.logged) {
        k_theta_one<<<(N + 255) / 256, 256, 0, s->batch>>>(m.u + N, N, 0);
        count_launches(1);
    }
    r.u1.resize(3 * (size_t)N);
    cudaMemcpyAsync(r.u1.data(), m.u, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s->batch);
    cudaFreeAsync(r.dmem, s->batch);
    cudaError_t e = cudaStreamSynchronize(s->batch);
    r.dmem = nullptr;
    r.stats.naccept = m.naccept;
    r.stats.nreject = m.nreject;
    r.stats.nrhs = (s->batch_opts.alg == GBC_ALG_VCABM5) ? m.iters + m.naccept + 1 : 6 * m.iters + 1;
    r.stats.t = m.t;
    r.stats.dt = m.dt;
    r.stats.status = m.status;
    r.status = (e != cudaSuccess) ? GBC_ECUDA : (m.status != 0 ? GBC_ESOLVER : 0);
}

// ---- mantle requests --------------------------------------------------------------------------
extern "C" int gbc_model_create(int, int, int, gbc_model**);
extern "C" int gbc_model_assemble(gbc_model*, const gbc_fault_mesh*, const gbc_hex_mesh*, double, double, int, int,
                                  double, const double*, const double*, int);
extern "C" int gbc_model_set_fault_props(gbc_model*, const double*, const double*, const double*, const double*, double,
                                         double, double, double);
extern "C" int gbc_model_set_mantle_props(gbc_model*, const double*, const double*, const double*);
extern "C" int gbc_model_set_precision(gbc_model*, int);
extern "C" int gbc_model_set_log_theta(gbc_model*, int);
extern "C" int gbc_integrate(gbc_model*, double*, double, double, const gbc_solver_opts*, gbc_solver_stats*);

static void run_mantle(gbc_server* s, std::shared_ptr<Req> rp) {
    Req& r = *rp;
    GfEntry* ge = r.entry;  // exclusively this request's while it runs (refs == 1)
    gbc_model* m = ge->model;
    int rc = 0;
    bool assembled = ge->valid;
    if (!assembled) {
        rc = gbc_model_create(r.nx, r.nxi, r.ne, &m);
        gbc_fault_mesh mf{r.nx, r.nxi, r.fx.data(), r.fxi.data(), r.fy.data(), r.fz.data(), r.fax.data(),
                          r.faxi.data(), r.dx, r.dxi, r.dep, r.dip};
        gbc_hex_mesh ma{r.ne, r.hex[0].data(), r.hex[1].data(), r.hex[2].data(), r.hex[3].data(), r.hex[4].data(),
                        r.hex[5].data(), r.hex[6].data(), r.hex[7].data(), r.hex[8].data()};
        if (!rc) rc = gbc_model_assemble(m, &mf, &ma, r.lambda, r.mu, r.ftype, r.nrept, r.buffer_ratio,
                                         r.qc.empty() ? nullptr : r.qc.data(), r.qw.empty() ? nullptr : r.qw.data(),
                                         (int)r.qw.size());
        if (!rc) rc = gbc_model_set_precision(m, r.precision);
        assembled = (rc == 0);
    }
    if (!rc) rc = gbc_model_set_fault_props(m, r.a.data(), r.b.data(), r.L.data(), r.sig.data(), r.eta, r.vpl, r.f0, r.v0);
    if (!rc) rc = gbc_model_set_mantle_props(m, r.gamma.data(), r.nexp.data(), r.deps0);
    if (!rc) rc = gbc_model_set_log_theta(m, r.precision != GBC_PREC_F64 && r.opts.alg != GBC_ALG_VCABM5);
    r.u1 = r.u0;
    if (!rc) rc = gbc_integrate(m, r.u1.data(), r.t0, r.t1, &r.opts, &r.stats);
    std::lock_guard<std::mutex> lk(s->mu);
    ge->model = m;
    ge->valid = assembled;
    r.status = rc;
    r.worker_done = true;
    s->cv.notify_all();
}

// destroys evicted models outside the lock
static void reaper(gbc_server* s) {
    cudaSetDevice(0);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->reap_cv.wait(lk, [&] { return !s->graveyard.empty() || s->reap_stop; });
        if (s->graveyard.empty()) break;  // stop requested and nothing left
        std::vector<gbc_model*> g;
        g.swap(s->graveyard);
        lk.unlock();
        for (gbc_model* m : g) gbc_model_destroy(m);
        lk.lock();
    }
}

// ---- scheduler ----------------------------------------------------------------------------------
// the following hold s->mu
static void drop_entry(gbc_server* s, GfEntry* e) {
    if (e->ghat) cudaFreeAsync(e->ghat, s->admit);
    if (e->model) {
        s->graveyard.push_back(e->model);
        s->reap_cv.notify_one();
    }
    s->in_use -= e->bytes;
    for (size_t i = 0; i < s->cache.size(); ++i)
        if (s->cache[i].get() == e) { s->cache.erase(s->cache.begin() + i); break; }
}

// evicts idle entries, least recently used first, until `need` more bytes fit; false if they cannot,
// and then nothing is evicted (a request that cannot be admitted yet must not empty the cache on
// every pass of the scheduler)
static bool make_room(gbc_server* s, size_t need) {
    if (s->in_use + need <= s->budget) return true;
    size_t idle = 0;
    for (auto& e : s->cache)
        if (e->refs == 0) idle += e->bytes;
    if (s->in_use + need > s->budget + idle) return false;
    while (s->in_use + need > s->budget) {
        GfEntry* victim = nullptr;
        for (auto& e : s->cache)
            if (e->refs == 0 && (!victim || e->last < victim->last)) victim = e.get();
        if (!victim) return false;
        drop_entry(s, victim);
    }
    return true;
}

// takes a cached entry for request r (or makes a new one) and charges the budget; false: no room yet
static bool acquire(gbc_server* s, Req& r) {
    GfEntry* hit = nullptr;
    if (s->cache_on)
        for (auto& e : s->cache)
            if (e->valid && e->key == r.key && (!e->mantle || e->refs == 0)) { hit = e.get(); break; }
    const size_t need = r.own + (hit ? 0 : r.gf);
    if (hit) ++hit->refs;  // pinned: make_room never evicts it
    if (!make_room(s, need)) {
        if (hit) --hit->refs;
        return false;
    }
    s->in_use += need;
    if (hit) {
        ++s->hits;
        r.entry = hit;
    } else {
        ++s->misses;
        auto e = std::make_unique<GfEntry>();
        e->key = r.key;
        e->mantle = r.ne > 0;
        e->bytes = r.gf;
        e->refs = 1;
        r.entry = e.get();
        s->cache.push_back(std::move(e));
    }
    r.entry->last = s->now();
    return true;
}

static void complete(gbc_server* s, Req& r) {
    r.t_done = s->now();
    r.done = true;
    s->in_use -= r.own;
    if (GfEntry* e = r.entry) {
        --e->refs;
        e->last = r.t_done;
        if (e->refs == 0 && (!e->valid || !s->cache_on)) drop_entry(s, e);
        r.entry = nullptr;
    }
    s->done_cv.notify_all();
}

static void scheduler(gbc_server* s) {
    cudaSetDevice(0);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        // admit from the head of the queue while the HBM budget allows (arrival order); cached
        // Green's functions are reused, idle ones evicted when the head would not fit otherwise
        auto start = [&](std::shared_ptr<Req> r) {
            s->peak = std::max(s->peak, s->in_use);
            r->t_admit = s->now();
            if (r->ne > 0) {
                s->mantle_active.push_back(r);
                r->worker = std::thread(run_mantle, s, r);
            } else {
                lk.unlock();
                int rc = admit_fault(s, *r);
                lk.lock();
                if (rc) {
                    r->status = rc;
                    if (r->dmem) { cudaFreeAsync(r->dmem, s->admit); r->dmem = nullptr; }
                    cudaStreamSynchronize(s->admit);
                    complete(s, *r);
                } else {
                    s->batch_active.push_back(r);
                }
            }
        };
        while (!s->queue.empty() && acquire(s, *s->queue.front())) {
            std::shared_ptr<Req> r = s->queue.front();
            s->queue.pop_front();
            start(r);
        }
        // a head that does not fit yet (a mantle request waiting for gigabytes) keeps its place;
        // fault-only requests queued behind it that fit now (megabytes each) run around it, so a
        // stream of small requests is not held behind one large one
        for (size_t i = 1; i < s->queue.size() && i <= 256;) {
            std::shared_ptr<Req> r = s->queue[i];
            if (r->ne == 0 && acquire(s, *r)) {
                s->queue.erase(s->queue.begin() + (long)i);
                start(r);
            } else {
                ++i;
            }
        }
        // reap finished mantle workers
        for (size_t i = 0; i < s->mantle_active.size();) {
            auto& r = s->mantle_active[i];
            if (r->worker_done) {
                lk.unlock();
                r->worker.join();
                lk.lock();
                complete(s, *r);
                s->mantle_active.erase(s->mantle_active.begin() + i);
            } else {
                ++i;
            }
        }
        if (s->batch_active.empty()) {
            if (s->stop && s->queue.empty() && s->mantle_active.empty()) break;
            s->cv.wait_for(lk, std::chrono::milliseconds(2));
            continue;
        }
        // one batch iteration over the active fault-only requests
        std::vector<std::shared_ptr<Req>> act = s->batch_active;
        lk.unlock();
        const int n = (int)act.size();
        size_t smem = 0;
        std::vector<EnsModel> h(n);
        for (int i = 0; i < n; ++i) {
            h[i] = act[i]->desc;
            smem = std::max(smem, act[i]->smem);
        }
        int rc = 0;
        if (n > s->d_desc_cap) {
            if (s->d_desc) cudaFree(s->d_desc);
            ens_launch_destroy(s->lp);
            s->d_desc_cap = std::max(n, 2 * s->d_desc_cap);
            if (cudaMalloc(&s->d_desc, sizeof(EnsModel) * s->d_desc_cap) != cudaSuccess) rc = GBC_ENOMEM;
            if (!rc) rc = ens_launch_create(s->lp, s->d_desc_cap);
        }
        if (!rc && cudaMemcpyAsync(s->d_desc, h.data(), sizeof(EnsModel) * n, cudaMemcpyHostToDevice, s->batch) != cudaSuccess) rc = GBC_ECUDA;
        if (!rc) rc = ens_launch_prepare(s->lp, s->d_desc, h.data(), n, 8, ens_boost(n), s->batch);
        if (!rc) rc = ens_run_groups(s->lp, s->batch_opts.reltol, s->batch_opts.abstol, s->batch_opts.dtmax,
                                     s->batch_opts.dtmin, s->slice_ns, s->block, smem, s->batch, s->batch_opts.alg,
                                     0, 2);
        if (!rc && cudaMemcpyAsync(h.data(), s->d_desc, sizeof(EnsModel) * n, cudaMemcpyDeviceToHost, s->batch) != cudaSuccess) rc = GBC_ECUDA;
        if (!rc && cudaStreamSynchronize(s->batch) != cudaSuccess) rc = GBC_ECUDA;
        std::vector<std::shared_ptr<Req>> fin;
        for (int i = 0; i < n; ++i) {
            act[i]->desc = h[i];
            if (rc || h[i].done) fin.push_back(act[i]);
        }
        for (auto& r : fin) {
            finish_fault(s, *r);
            if (rc) r->status = rc;
        }
        lk.lock();
        ++s->iterations;
        for (auto& r : fin) {
            complete(s, *r);
            for (size_t i = 0; i < s->batch_active.size(); ++i)
                if (s->batch_active[i] == r) { s->batch_active.erase(s->batch_active.begin() + i); break; }
        }
    }
}

extern "C" {

int gbc_server_create(double hbm_budget_bytes, const gbc_solver_opts* batch_opts, gbc_server** out) {
    if (!out || !batch_opts || !(hbm_budget_bytes > 0)) return fail(GBC_EINVAL, "bad server arguments");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GBC_ENODEV, "no CUDA device available (libgbcycle has no CPU fallback)");
    gbc_server* s = new gbc_server();
    s->budget = hbm_budget_bytes;
    s->batch_opts = *batch_opts;
    s->t_start = std::chrono::steady_clock::now();
    // the scheduler's admission and batch work at the greatest stream priority: a mantle request's
    // Green's-function assembly fills the GPU for seconds, and the scheduler thread waits for each
    // admission; at a higher priority the small kernels are dispatched as the assembly's CTAs retire
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->batch, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->admit, cudaStreamNonBlocking, greatest);
    if (e != cudaSuccess) { delete s; return cuda_fail(e, "cudaStreamCreate"); }
    if (int rc = upload_gl_tables()) { delete s; return rc; }
    // batch descriptors for up to 1024 requests, allocated now: growing them later frees device
    // memory on the scheduler thread, which waits for all queued work
    s->d_desc_cap = 1024;
    if (cudaMalloc(&s->d_desc, sizeof(EnsModel) * s->d_desc_cap) != cudaSuccess) { delete s; return fail(GBC_ENOMEM, "server batch descriptors"); }
    if (int rc = ens_launch_create(s->lp, s->d_desc_cap)) { cudaFree(s->d_desc); delete s; return rc; }
    s->reaper = std::thread(reaper, s);
    s->sched = std::thread(scheduler, s);
    *out = s;
    return 0;
}

int gbc_server_submit(gbc_server* s, const gbc_request* q, long long* id) {
    if (!s || !q || !id || !q->mf || !q->u0) return fail(GBC_EINVAL, "bad request");
    const gbc_fault_mesh* mf = q->mf;
    if (mf->nx <= 0 || mf->nxi <= 0 || !(q->t1 >= q->t0)) return fail(GBC_EINVAL, "bad request sizes or horizon");
    auto r = std::make_shared<Req>();
    r->nx = mf->nx; r->nxi = mf->nxi; r->ne = q->ma ? q->ma->ne : 0;
    const size_t N = (size_t)r->nx * r->nxi;
    r->fx.assign(mf->x, mf->x + r->nx); r->fxi.assign(mf->xi, mf->xi + r->nxi);
    r->fy.assign(mf->y, mf->y + r->nxi); r->fz.assign(mf->z, mf->z + r->nxi);
    r->fax.assign(mf->ax, mf->ax + 2 * r->nx); r->faxi.assign(mf->axi, mf->axi + 2 * r->nxi);
    r->dx = mf->dx; r->dxi = mf->dxi; r->dep = mf->dep; r->dip = mf->dip;
    r->lambda = q->lambda; r->mu = q->mu; r->nrept = q->nrept; r->buffer_ratio = q->buffer_ratio; r->ftype = q->ftype;
    r->a.assign(q->a, q->a + N); r->b.assign(q->b, q->b + N); r->L.assign(q->L, q->L + N); r->sig.assign(q->sigma, q->sigma + N);
    r->eta = q->eta; r->vpl = q->vpl; r->f0 = q->f0; r->v0 = q->v0;
    r->t0 = q->t0; r->t1 = q->t1;
    r->opts = q->ne_opts_valid ? q->opts : s->batch_opts;
    r->precision = q->precision;
    if (r->ne > 0) {
        const gbc_hex_mesh* ma = q->ma;
        const double* src[9] = {ma->cx, ma->cy, ma->cz, ma->qx, ma->qy, ma->qz, ma->dx, ma->dy, ma->dz};
        for (int k = 0; k < 9; ++k) r->hex[k].assign(src[k], src[k] + r->ne);
        if (!q->gamma || !q->n || !q->deps0) return fail(GBC_EINVAL, "mantle request needs viscosity properties");
        r->gamma.assign(q->gamma, q->gamma + r->ne); r->nexp.assign(q->n, q->n + r->ne);
        for (int k = 0; k < 6; ++k) r->deps0[k] = q->deps0[k];
        if (q->nq > 0) { r->qc.assign(q->qcoords, q->qcoords + 3 * q->nq); r->qw.assign(q->qweights, q->qweights + q->nq); }
        r->u0.assign(q->u0, q->u0 + 3 * N + 12 * (size_t)r->ne);
        r->own = 0;  // the assembled model holds the state too
        r->gf = mantle_bytes(*r);
    } else {
        EnsModel m;
        size_t smem;
        if (int rc = ens_prepare_model(m, r->nx, r->nxi, &smem)) return rc;
        r->u0.assign(q->u0, q->u0 + 3 * N);
        r->own = fault_own_bytes(m);
        r->gf = fault_gf_bytes(*r, m);
    }
    r->key = gf_key(*r);
    if ((double)(r->own + r->gf) > s->budget) return fail(GBC_ENOMEM, "request larger than the server's HBM budget");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(GBC_ESTATE, "server is shutting down");
    r->id = s->next_id++;
    r->t_submit = s->now();
    s->all[r->id] = r;
    s->queue.push_back(r);
    *id = r->id;
    s->cv.notify_all();
    return 0;
}

int gbc_server_wait(gbc_server* s, long long id, double* u_out, gbc_request_result* res) {
    if (!s) return fail(GBC_EINVAL, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return fail(GBC_EINVAL, "unknown request id");
    std::shared_ptr<Req> r = it->second;
    s->done_cv.wait(lk, [&] { return r->done; });
    s->all.erase(id);
    if (u_out && !r->u1.empty()) memcpy(u_out, r->u1.data(), sizeof(double) * r->u1.size());
    if (res) {
        res->id = r->id;
        res->status = r->status;
        res->submit_s = r->t_submit;
        res->admit_s = r->t_admit;
        res->done_s = r->t_done;
        res->stats = r->stats;
    }
    return r->status;
}

int gbc_server_query(gbc_server* s, gbc_server_info* out) {
    if (!s || !out) return fail(GBC_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    out->queued = (int)s->queue.size();
    out->batched = (int)s->batch_active.size();
    out->mantle = (int)s->mantle_active.size();
    out->bytes_in_use = (double)s->in_use;
    out->peak_bytes = (double)s->peak;
    out->iterations = s->iterations;
    out->cache_entries = (int)s->cache.size();
    double cb = 0;
    for (auto& e : s->cache) cb += (double)e->bytes;
    out->cache_bytes = cb;
    out->cache_hits = s->hits;
    out->cache_misses = s->misses;
    return 0;
}

int gbc_server_set_gf_cache(gbc_server* s, int enabled) {
    if (!s) return fail(GBC_EINVAL, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    s->cache_on = enabled != 0;
    if (!s->cache_on)
        for (size_t i = s->cache.size(); i-- > 0;)
            if (s->cache[i]->refs == 0) drop_entry(s, s->cache[i].get());
    return 0;
}

void gbc_server_destroy(gbc_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->sched.joinable()) s->sched.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        while (!s->cache.empty()) drop_entry(s, s->cache.back().get());
        s->reap_stop = true;
        s->reap_cv.notify_all();
    }
    if (s->reaper.joinable()) s->reaper.join();
    if (s->d_desc) cudaFree(s->d_desc);
    ens_launch_destroy(s->lp);
    cudaStreamSynchronize(s->batch);
    cudaStreamSynchronize(s->admit);
    cudaStreamDestroy(s->batch);
    cudaStreamDestroy(s->admit);
    delete s;
}

}  // extern "C"
