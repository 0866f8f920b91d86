// Green's-function assembly kernels: one thread per source-receiver pair (all images, quadrature
// points and, for strain volumes, all six unit eigenstrains evaluated in-thread), writing
// row-major receiver rows so consecutive threads store consecutive source columns.
//
// Reference loops restated (src/BEM/GF.jl): fault-fault :31-71, fault->mantle :123-174,
// mantle->fault :194-227, mantle-mantle :250-296. The strain-volume stress (the quantity of
// GeoGreensFunctions.stress_vol_hex8!, called at GF.jl:215-221 and :277-283) is computed as a
// stack of Okada dislocation planes through the cuboid integrated over its thickness with
// Gauss-Legendre panels: a uniform eigenstrain eps* equals a continuous stack of dislocations
// with sym(b (x) n) = eps* per unit thickness.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>
#include <set>
#include <cuda_runtime.h>

#include "gbc_internal.cuh"
#include "okada_device.cuh"

namespace gbc {

__constant__ double c_glx[4][16];
__constant__ double c_glw[4][16];
__constant__ int c_glord[4] = {4, 8, 12, 16};

void gl_rule(int n, double* x, double* w) {
    // Newton iteration on P_n (same rule the CPU oracle tabulates)
    for (int i = 0; i < n; ++i) {
        double t = cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = t;
            for (int k = 2; k <= n; ++k) {
                double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                p0 = p1; p1 = p2;
            }
            double dp = n * (t * p1 - p0) / (t * t - 1.0);
            double dt = p1 / dp;
            t -= dt;
            if (fabs(dt) < 1e-16) break;
        }
        double p0 = 1.0, p1 = t;
        for (int k = 2; k <= n; ++k) {
            double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
            p0 = p1; p1 = p2;
        }
        double dp = n * (t * p1 - p0) / (t * t - 1.0);
        x[i] = -t;
        w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
    }
}

// constant memory is per device: the tables are uploaded once for each device that assembles
int upload_gl_tables() {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return 0;
    double x[4][16] = {{0}}, w[4][16] = {{0}};
    const int ord[4] = {4, 8, 12, 16};
    for (int k = 0; k < 4; ++k) gl_rule(ord[k], x[k], w[k]);
    GBC_CUDA(cudaMemcpyToSymbol(c_glx, x, sizeof(x)));
    GBC_CUDA(cudaMemcpyToSymbol(c_glw, w, sizeof(w)));
    done.insert(dev);
    return 0;
}

// ---------------------------------------------------------------------------------------------
// traction projections (GF.jl:76-96); u-gradient G[i][j] = d u_i / d x_j
__device__ __forceinline__ double traction_from_grad(int ftype, const double (&G)[3][3], double lam,
                                                     double mu, double sd, double cd, double s2d,
                                                     double c2d) {
    if (ftype == 0) {
        double sxy = mu * (G[1][0] + G[0][1]);
        double sxz = mu * (G[2][0] + G[0][2]);
        return -sxy * sd + sxz * cd;
    }
    double tr = G[0][0] + G[1][1] + G[2][2];
    double szz = lam * tr + 2.0 * mu * G[2][2];
    double syy = lam * tr + 2.0 * mu * G[1][1];
    double syz = mu * (G[2][1] + G[1][2]);
    return (szz - syy) / 2.0 * s2d + syz * c2d;
}

__device__ __forceinline__ double traction_from_stress(int ftype, const double* s, double sd, double cd,
                                                       double s2d, double c2d) {
    if (ftype == 0) return -s[1] * sd + s[2] * cd;
    return (s[5] - s[3]) / 2.0 * s2d + s[4] * c2d;
}

__device__ __forceinline__ void grad_to_stress(const double (&G)[3][3], double lam, double mu, double* s) {
    double tr = G[0][0] + G[1][1] + G[2][2];
    s[0] = lam * tr + 2.0 * mu * G[0][0];
    s[1] = mu * (G[0][1] + G[1][0]);
    s[2] = mu * (G[0][2] + G[2][0]);
    s[3] = lam * tr + 2.0 * mu * G[1][1];
    s[4] = mu * (G[1][2] + G[2][1]);
    s[5] = lam * tr + 2.0 * mu * G[2][2];
}

// ---------------------------------------------------------------------------------------------
__global__ void k_gf_ff(FaultDev f, double lam, double mu, int ftype, int nrept, double lrept,
                        double* __restrict__ st) {
    const int nx = f.nx, nxi = f.nxi;
    const long long total = (long long)nx * nxi * nxi;
    const double alpha = (lam + mu) / (lam + 2.0 * mu);
    double sd, cd, s2d, c2d;
    sincosd(f.dip, &sd, &cd);
    sincosd(2.0 * f.dip, &s2d, &c2d);
    const double slip[1][3] = {{ftype == 0 ? 1.0 : 0.0, ftype == 0 ? 0.0 : 1.0, 0.0}};
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % nx), j = (int)((t / nx) % nxi), l = (int)(t / ((long long)nx * nxi));
        double G[1][3][3] = {};
        for (int p = -nrept; p <= nrept; ++p) {
            const double jump = p * lrept;
            Rect r = make_rect(f.dep, f.dip, f.ax[0] + jump, f.ax[1] + jump, f.axi[2 * l], f.axi[2 * l + 1]);
            dc3d_grad_acc<1>(f.x[i], f.y[j], f.z[j], alpha, r, slip, 1.0, G);
        }
        st[t] = traction_from_grad(ftype, G[0], lam, mu, sd, cd, s2d, c2d);
    }
}

// rFFT of [st[:,j,l]; reverse(st[2:end,j,l])] (length 2nx-1, nx bins), one thread per bin
__global__ void k_gf_ff_dft(int nx, int nxi, const double* __restrict__ st, double* __restrict__ out) {
    const int n = 2 * nx - 1;
    const long long total = (long long)nx * nxi * nxi;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % nx);
        const double* col = st + (t - k);
        double re = 0.0, im = 0.0;
        for (int m = 0; m < n; ++m) {
            const double v = (m < nx) ? col[m] : col[n - m];
            const int idx = (int)(((long long)k * m) % n);
            double s, c;
            sincospi(2.0 * idx / n, &s, &c);
            re += v * c;
            im -= v * s;
        }
        out[2 * t] = re;
        out[2 * t + 1] = im;
    }
}

// inverse of the above: st[m] = (X0 + 2 sum_k Re(X_k e^{2 pi i k m / n})) / n for m < nx
__global__ void k_gf_ff_idft(int nx, int nxi, const double* __restrict__ in, double* __restrict__ st) {
    const int n = 2 * nx - 1;
    const long long total = (long long)nx * nxi * nxi;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(t % nx);
        const double* col = in + 2 * (t - m);
        double acc = col[0];
        for (int k = 1; k < nx; ++k) {
            const int idx = (int)(((long long)k * m) % n);
            double s, c;
            sincospi(2.0 * idx / n, &s, &c);
            acc += 2.0 * (col[2 * k] * c - col[2 * k + 1] * s);
        }
        st[t] = acc / n;
    }
}

__global__ void k_gf_fm(FaultDev f, HexDev h, double lam, double mu, int ftype, int nrept, double lrept,
                        const double* __restrict__ qc, const double* __restrict__ qw, int nq,
                        double* __restrict__ out, size_t ld) {
    const int N = f.nx * f.nxi, ne = h.ne;
    const long long total = (long long)N * ne;
    const double alpha = (lam + mu) / (lam + 2.0 * mu);
    const double slip[1][3] = {{ftype == 0 ? 1.0 : 0.0, ftype == 0 ? 0.0 : 1.0, 0.0}};
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(t % N), i = (int)(t / N);  // j: source patch, i: receiver cell
        const int q1 = j % f.nx, q2 = j / f.nx;
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w < nq; ++w) {
            const double rx = h.cx[i] + qc[3 * w] * h.dx[i] / 2.0;
            const double ry = h.cy[i] + qc[3 * w + 1] * h.dy[i] / 2.0;
            const double rz = h.cz[i] + qc[3 * w + 2] * h.dz[i] / 2.0;
            double G[1][3][3] = {};
            for (int p = -nrept; p <= nrept; ++p) {
                const double jump = p * lrept;
                Rect r = make_rect(f.dep, f.dip, f.ax[2 * q1] + jump, f.ax[2 * q1 + 1] + jump,
                                   f.axi[2 * q2], f.axi[2 * q2 + 1]);
                dc3d_grad_acc<1>(rx, ry, rz, alpha, r, slip, 1.0, G);
            }
            double s[6];
            grad_to_stress(G[0], lam, mu, s);
            for (int k = 0; k < 6; ++k) acc[k] += qw[w] * s[k];
        }
        for (int k = 0; k < 6; ++k) out[((size_t)k * ne + i) * ld + j] = acc[k];
    }
}

// ---------------------------------------------------------------------------------------------
// strain-volume stacks
__device__ __forceinline__ double rect_boundary_dist(double u, double v, double u1, double u2,
                                                     double v1, double v2) {
    if (u >= u1 && u <= u2 && v >= v1 && v <= v2)
        return fmin(fmin(u - u1, u2 - u), fmin(v - v1, v2 - v));
    double du = fmax(fmax(u1 - u, 0.0), u - u2);
    double dv = fmax(fmax(v1 - v, 0.0), v - v2);
    return sqrt(du * du + dv * dv);
}

__device__ __forceinline__ double panel_rho(double sr, double d, double m, double h) {
    double zr = (sr - m) / h, zi = d / h;
    double a = 0.5 * (hypot(zr - 1.0, zi) + hypot(zr + 1.0, zi));
    return a + sqrt(fmax(a * a - 1.0, 0.0));
}

__device__ __forceinline__ int order_for_rho(double rho) {
    double need = 18.420680743952367 / log(rho);
    for (int k = 0; k < 4; ++k)
        if (c_glord[k] >= need) return k;
    return 3;
}

// Visits Gauss nodes (s, w) of adaptive panels covering [s0, s1], left to right.
template <class F>
__device__ __forceinline__ void for_each_node(double s0, double s1, double sr, double d, F&& fn) {
    constexpr int MAXD = 24, MAXP = 64;
    double sa[MAXD + 2], sb[MAXD + 2];
    int sdp[MAXD + 2];
    int top = 1, np = 0;
    sa[0] = s0; sb[0] = s1; sdp[0] = 0;
    while (top > 0) {
        --top;
        const double a = sa[top], b = sb[top];
        const int dep = sdp[top];
        const double m = 0.5 * (a + b), h = 0.5 * (b - a);
        const double rho = panel_rho(sr, d, m, h);
        if (rho < 3.0 && dep < MAXD && top + 2 <= MAXD + 2 && np + top + 2 <= MAXP) {
            sa[top] = m; sb[top] = b; sdp[top] = dep + 1; ++top;
            sa[top] = a; sb[top] = m; sdp[top] = dep + 1; ++top;
            continue;
        }
        const int o = (rho < 3.0) ? 3 : order_for_rho(rho);
        const int n = c_glord[o];
        for (int i = 0; i < n; ++i) fn(m + h * c_glx[o][i], h * c_glw[o][i]);
        ++np;
    }
}

// S[p][k]: stress component k at (x,y,z) from unit eigenstrain component p in the cuboid
// [qx-T/2, qx+T/2] x [qy, qy+L] x [qz-W, qz]. Component order (xx, xy, xz, yy, yz, zz).
__device__ void hex8_unit_stresses(double x, double y, double z, double qx, double qy, double qz,
                                   double T, double L, double W, double lam, double mu,
                                   double (&S)[6][6]) {
    const double alpha = (lam + mu) / (lam + 2.0 * mu);
    const double x1 = qx - 0.5 * T, x2 = qx + 0.5 * T, y1 = qy, y2 = qy + L, z1 = qz - W, z2 = qz;
    {   // planes normal to y (dip 90, strike x): eps_xy = -U1/2, eps_yz = -U2/2, eps_yy = U3
        const double slip[3][3] = {{-2.0, 0.0, 0.0}, {0.0, -2.0, 0.0}, {0.0, 0.0, 1.0}};
        double G[3][3][3] = {};
        const Rect r = make_rect(0.0, 90.0, x1, x2, z1, z2);
        for_each_node(y1, y2, y, rect_boundary_dist(x, z, x1, x2, z1, z2),
                      [&](double s, double w) { dc3d_grad_acc<3>(x, y - s, z, alpha, r, slip, w, G); });
        grad_to_stress(G[0], lam, mu, S[1]);
        grad_to_stress(G[1], lam, mu, S[4]);
        grad_to_stress(G[2], lam, mu, S[3]);
    }
    {   // horizontal planes at height s (depth -s; dip 0, strike x): eps_xz = U1/2, eps_zz = U3
        const double slip[2][3] = {{2.0, 0.0, 0.0}, {0.0, 0.0, 1.0}};
        double G[2][3][3] = {};
        for_each_node(z1, z2, z, rect_boundary_dist(x, y, x1, x2, y1, y2), [&](double s, double w) {
            const Rect r = make_rect(-s, 0.0, x1, x2, y1, y2);
            dc3d_grad_acc<2>(x, y, z, alpha, r, slip, w, G);
        });
        grad_to_stress(G[0], lam, mu, S[2]);
        grad_to_stress(G[1], lam, mu, S[5]);
    }
    {   // planes normal to x in the frame X = y, Y = -x, Z = z (dip 90, strike X): eps_xx = U3
        const double slip[1][3] = {{0.0, 0.0, 1.0}};
        double Gr[1][3][3] = {};
        const Rect r = make_rect(0.0, 90.0, y1, y2, z1, z2);
        for_each_node(x1, x2, x, rect_boundary_dist(y, z, y1, y2, z1, z2),
                      [&](double s, double w) { dc3d_grad_acc<1>(y, s - x, z, alpha, r, slip, w, Gr); });
        // G = Q^T Gr Q, Q = [[0,1,0],[-1,0,0],[0,0,1]]
        double G[3][3];
        G[0][0] = Gr[0][1][1];  G[0][1] = -Gr[0][1][0]; G[0][2] = -Gr[0][1][2];
        G[1][0] = -Gr[0][0][1]; G[1][1] = Gr[0][0][0];  G[1][2] = Gr[0][0][2];
        G[2][0] = -Gr[0][2][1]; G[2][1] = Gr[0][2][0];  G[2][2] = Gr[0][2][2];
        grad_to_stress(G, lam, mu, S[0]);
    }
}

__global__ void k_gf_mf(HexDev h, FaultDev f, double lam, double mu, int ftype,
                        double* __restrict__ out, size_t ld) {
    const int N = f.nx * f.nxi, ne = h.ne;
    const long long total = (long long)N * ne;
    double sd, cd, s2d, c2d;
    sincosd(f.dip, &sd, &cd);
    sincosd(2.0 * f.dip, &s2d, &c2d);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(t % ne), i = (int)(t / ne);  // j: source cell, i: receiver patch
        const int q1 = i % f.nx, q2 = i / f.nx;
        double S[6][6];
        hex8_unit_stresses(f.x[q1], f.y[q2], f.z[q2], h.qx[j], h.qy[j], h.qz[j], h.dx[j], h.dy[j],
                           h.dz[j], lam, mu, S);
        for (int p = 0; p < 6; ++p)
            out[(size_t)i * ld + (size_t)p * ne + j] = traction_from_stress(ftype, S[p], sd, cd, s2d, c2d);
    }
}

// stress components k at receiver cell jr (quadrature-averaged) from unit eigenstrain p in source
// cell is (GF.jl:250-296)
__device__ __forceinline__ void mm_pair(const HexDev& h, int jr, int is, double lam, double mu,
                                        const double* __restrict__ qc, const double* __restrict__ qw, int nq,
                                        double (&acc)[6][6]) {
    for (int p = 0; p < 6; ++p)
        for (int k = 0; k < 6; ++k) acc[p][k] = 0.0;
    for (int q = 0; q < nq; ++q) {
        const double rx = h.cx[jr] + qc[3 * q] * h.dx[jr] / 2.0;
        const double ry = h.cy[jr] + qc[3 * q + 1] * h.dy[jr] / 2.0;
        const double rz = h.cz[jr] + qc[3 * q + 2] * h.dz[jr] / 2.0;
        double S[6][6];
        hex8_unit_stresses(rx, ry, rz, h.qx[is], h.qy[is], h.qz[is], h.dx[is], h.dy[is], h.dz[is], lam, mu, S);
        for (int p = 0; p < 6; ++p)
            for (int k = 0; k < 6; ++k) acc[p][k] += S[p][k] * qw[q];
    }
}

__global__ void k_gf_mm(HexDev h, double lam, double mu, const double* __restrict__ qc,
                        const double* __restrict__ qw, int nq, double* __restrict__ out, size_t ld) {
    const int ne = h.ne;
    const long long total = (long long)ne * ne;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int is = (int)(t % ne), jr = (int)(t / ne);  // is: source cell, jr: receiver cell
        double acc[6][6];
        mm_pair(h, jr, is, lam, mu, qc, qw, nq, acc);
        for (int p = 0; p < 6; ++p)
            for (int k = 0; k < 6; ++k) out[((size_t)k * ne + jr) * ld + (size_t)p * ne + is] = acc[p][k];
    }
}

// Structured boxes (a complete nX x nY x nZ grid of equal cells): an entry depends only on the
// horizontal offset of the two cells and their layers (the half-space is invariant under horizontal
// translation), so each key (dx, dy, layer_r, layer_s) is evaluated once on a representative pair
// of the mesh and the dense matrix is filled from the table.
__global__ void k_gf_mm_keys(HexDev h, double lam, double mu, const double* __restrict__ qc,
                             const double* __restrict__ qw, int nq, const int2* __restrict__ reps, long long nkeys,
                             double* __restrict__ table) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nkeys;
         t += (long long)gridDim.x * blockDim.x) {
        const int2 r = reps[t];  // (receiver, source)
        double acc[6][6];
        mm_pair(h, r.x, r.y, lam, mu, qc, qw, nq, acc);
        for (int p = 0; p < 6; ++p)
            for (int k = 0; k < 6; ++k) table[t * 36 + p * 6 + k] = acc[p][k];
    }
}

__global__ void k_gf_mm_expand(int ne, const int4* __restrict__ cell, int nX, int nY, int nZ,
                               const double* __restrict__ table, double* __restrict__ out, size_t ld) {
    const long long total = (long long)ne * ne;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int is = (int)(t % ne), jr = (int)(t / ne);
        const int4 a = cell[jr], b = cell[is];  // (ix, iy, iz, -)
        const long long key = (((long long)(a.x - b.x + nX - 1) * (2 * nY - 1) + (a.y - b.y + nY - 1)) * nZ + a.z) * nZ + b.z;
        const double* v = table + key * 36;
        for (int p = 0; p < 6; ++p)
            for (int k = 0; k < 6; ++k) out[((size_t)k * ne + jr) * ld + (size_t)p * ne + is] = v[p * 6 + k];
    }
}

// ---------------------------------------------------------------------------------------------
// One item per thread: the CTAs are short-lived (an Okada evaluation each), so a multi-second
// assembly does not hold the SMs for its whole duration and higher-priority work on other streams
// (a server's batch and admissions) is dispatched as CTAs retire. The kernels keep their
// grid-stride loops for grids beyond the launch limit.
static int grid_for(long long total, int block) {
    long long g = (total + block - 1) / block;
    const long long cap = 0x7fffffffLL;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

int launch_gf_ff(const FaultDev& f, double lambda, double mu, int ftype, int nrept, double buffer_ratio,
                 double* st, cudaStream_t s) {
    const double lrept = (buffer_ratio + 1.0) * (f.dx * f.nx);
    const long long total = (long long)f.nx * f.nxi * f.nxi;
    k_gf_ff<<<grid_for(total, 128), 128, 0, s>>>(f, lambda, mu, ftype, nrept, lrept, st);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int launch_gf_ff_dft(int nx, int nxi, const double* st, double* out, cudaStream_t s) {
    const long long total = (long long)nx * nxi * nxi;
    k_gf_ff_dft<<<grid_for(total, 128), 128, 0, s>>>(nx, nxi, st, out);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int launch_gf_ff_idft(int nx, int nxi, const double* in, double* st, cudaStream_t s) {
    const long long total = (long long)nx * nxi * nxi;
    k_gf_ff_idft<<<grid_for(total, 128), 128, 0, s>>>(nx, nxi, in, st);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int launch_gf_fm(const FaultDev& f, const HexDev& m, double lambda, double mu, int ftype, int nrept,
                 double buffer_ratio, const double* qc, const double* qw, int nq, double* out, size_t ld,
                 cudaStream_t s) {
    const double lrept = (buffer_ratio + 1.0) * (f.dx * f.nx);
    const long long total = (long long)f.nx * f.nxi * m.ne;
    k_gf_fm<<<grid_for(total, 128), 128, 0, s>>>(f, m, lambda, mu, ftype, nrept, lrept, qc, qw, nq, out, ld);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

int launch_gf_mf(const HexDev& m, const FaultDev& f, double lambda, double mu, int ftype, double* out,
                 size_t ld, cudaStream_t s) {
    if (int rc = upload_gl_tables()) return rc;
    const long long total = (long long)f.nx * f.nxi * m.ne;
    k_gf_mf<<<grid_for(total, 64), 64, 0, s>>>(m, f, lambda, mu, ftype, out, ld);
    GBC_CUDA(cudaGetLastError());
    return 0;
}

// Host side: is the mesh a complete grid of equal cells (centres on uniform x and y grids with the
// cell size as spacing, any set of depths, the same source-corner offsets)? Fills per-cell indices.
bool mm_grid(const gbc_hex_mesh* ma, MMGrid& g) {
    const int ne = ma->ne;
    if (ne < 2) return false;
    // equal within 1e-12 of the cell size (sizes and offsets computed from non-binary spacings
    // differ in the last bits between cells); a pair then differs from its key's representative
    // by a geometry change of that order
    const double tol = 1e-12 * std::max(std::fabs(ma->dx[0]), std::max(std::fabs(ma->dy[0]), std::fabs(ma->dz[0])));
    auto same = [&](double a, double b) { return std::fabs(a - b) <= tol; };
    for (int i = 0; i < ne; ++i)
        if (!same(ma->dx[i], ma->dx[0]) || !same(ma->dy[i], ma->dy[0]) || !same(ma->dz[i], ma->dz[0]) ||
            !same(ma->qx[i] - ma->cx[i], ma->qx[0] - ma->cx[0]) || !same(ma->qy[i] - ma->cy[i], ma->qy[0] - ma->cy[0]) ||
            !same(ma->qz[i] - ma->cz[i], ma->qz[0] - ma->cz[0]))
            return false;
    auto axis = [&](const double* c, double d, std::vector<int>& idx, int& n) {
        double lo = c[0], hi = c[0];
        for (int i = 1; i < ne; ++i) { lo = std::min(lo, c[i]); hi = std::max(hi, c[i]); }
        n = (int)std::llround((hi - lo) / d) + 1;
        idx.resize(ne);
        for (int i = 0; i < ne; ++i) {
            const double f = (c[i] - lo) / d;
            const long long k = std::llround(f);
            if (std::fabs(f - (double)k) > 1e-9) return false;
            idx[i] = (int)k;
        }
        return n >= 1;
    };
    if (!axis(ma->cx, ma->dx[0], g.ix, g.nX) || !axis(ma->cy, ma->dy[0], g.iy, g.nY)) return false;
    std::vector<double> zs(ma->cz, ma->cz + ne);
    std::sort(zs.begin(), zs.end());
    zs.erase(std::unique(zs.begin(), zs.end(), [&](double a, double b) { return std::fabs(a - b) <= tol; }), zs.end());
    g.nZ = (int)zs.size();
    g.iz.resize(ne);
    for (int i = 0; i < ne; ++i) {
        const auto it = std::lower_bound(zs.begin(), zs.end(), ma->cz[i] - tol);
        if (it == zs.end() || std::fabs(*it - ma->cz[i]) > tol) return false;
        g.iz[i] = (int)(it - zs.begin());
    }
    if ((long long)g.nX * g.nY * g.nZ != ne) return false;
    g.cell.assign((size_t)ne, -1);  // (ix, iy, iz) -> cell, every slot exactly once
    for (int i = 0; i < ne; ++i) {
        int& c = g.cell[((size_t)g.iz[i] * g.nY + g.iy[i]) * g.nX + g.ix[i]];
        if (c >= 0) return false;
        c = i;
    }
    const long long keys = (2LL * g.nX - 1) * (2LL * g.nY - 1) * g.nZ * g.nZ;
    return keys * 4 <= (long long)ne * ne;  // worth it only when keys are far fewer than pairs
}

int launch_gf_mm(const HexDev& m, double lambda, double mu, const double* qc, const double* qw, int nq,
                 double* out, size_t ld, cudaStream_t s, const MMGrid* grid) {
    if (int rc = upload_gl_tables()) return rc;
    const long long total = (long long)m.ne * m.ne;
    if (!grid) {
        k_gf_mm<<<grid_for(total, 64), 64, 0, s>>>(m, lambda, mu, qc, qw, nq, out, ld);
        GBC_CUDA(cudaGetLastError());
        return 0;
    }
    const MMGrid& g = *grid;
    const long long nk = (2LL * g.nX - 1) * (2LL * g.nY - 1) * g.nZ * g.nZ;
    std::vector<int2> reps((size_t)nk);
    for (int dx = -(g.nX - 1); dx <= g.nX - 1; ++dx)
        for (int dy = -(g.nY - 1); dy <= g.nY - 1; ++dy)
            for (int zr = 0; zr < g.nZ; ++zr)
                for (int zs = 0; zs < g.nZ; ++zs) {
                    const int xs = std::max(0, -dx), ys = std::max(0, -dy);
                    const long long key = (((long long)(dx + g.nX - 1) * (2 * g.nY - 1) + (dy + g.nY - 1)) * g.nZ + zr) * g.nZ + zs;
                    const int jr = g.cell[((size_t)zr * g.nY + ys + dy) * g.nX + xs + dx];
                    const int is = g.cell[((size_t)zs * g.nY + ys) * g.nX + xs];
                    reps[(size_t)key] = make_int2(jr, is);
                }
    std::vector<int4> cells((size_t)m.ne);
    for (int i = 0; i < m.ne; ++i) cells[(size_t)i] = make_int4(g.ix[i], g.iy[i], g.iz[i], 0);
    // temporaries freed on every path; the stream is drained before the host vectors go away
    struct Tmp {
        int2* reps = nullptr;
        int4* cells = nullptr;
        double* table = nullptr;
        cudaStream_t s;
        ~Tmp() {
            cudaStreamSynchronize(s);
            if (reps) cudaFree(reps);
            if (cells) cudaFree(cells);
            if (table) cudaFree(table);
        }
    } t;
    t.s = s;
    GBC_CUDA(cudaMalloc(&t.reps, sizeof(int2) * nk));
    GBC_CUDA(cudaMalloc(&t.cells, sizeof(int4) * m.ne));
    GBC_CUDA(cudaMalloc(&t.table, sizeof(double) * 36 * nk));
    GBC_CUDA(cudaMemcpyAsync(t.reps, reps.data(), sizeof(int2) * nk, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(t.cells, cells.data(), sizeof(int4) * m.ne, cudaMemcpyHostToDevice, s));
    k_gf_mm_keys<<<grid_for(nk, 64), 64, 0, s>>>(m, lambda, mu, qc, qw, nq, t.reps, nk, t.table);
    GBC_CUDA(cudaGetLastError());
    k_gf_mm_expand<<<grid_for(total, 256), 256, 0, s>>>(m.ne, t.cells, g.nX, g.nY, g.nZ, t.table, out, ld);
    GBC_CUDA(cudaGetLastError());
    GBC_CUDA(cudaStreamSynchronize(s));
    return 0;
}

}  // namespace gbc
