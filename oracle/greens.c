/*
 * Oracle: the four stress_greens_function methods of the reference (src/BEM/GF.jl) and the
 * Toeplitz -> rFFT embedding, restated loop for loop in C with OpenMP standing in for @threads.
 *
 * TEST INFRASTRUCTURE ONLY (the FP64 reference the CUDA path is tested against; never linked into the product).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "gbc_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_sincosd(double deg, double* s, double* c);
void orc_hex8_unit_stresses(double sig6x6[6][6], double x, double y, double z, double qx,
                            double qy, double qz, double T, double L, double W, double mu,
                            double nu);

int orc_num_threads(void) {
#ifdef _OPENMP
    int n = 1;
#pragma omp parallel
#pragma omp single
    n = omp_get_num_threads();
    return n;
#else
    return 1;
#endif
}

/* shear_traction_dc3d, src/BEM/GF.jl:76-87 (u is the 0-based 12-vector) */
static double traction_dc3d(int ftype, const double* u, double lam, double mu, double dip) {
    double sd, cd;
    if (ftype == 0) {
        orc_sincosd(dip, &sd, &cd);
        double sxy = mu * (u[4] + u[6]);
        double sxz = mu * (u[5] + u[9]);
        return -sxy * sd + sxz * cd;
    }
    orc_sincosd(2.0 * dip, &sd, &cd);
    double szz = (lam + 2.0 * mu) * u[11] + lam * u[3] + lam * u[7];
    double syy = (lam + 2.0 * mu) * u[7] + lam * u[3] + lam * u[11];
    double syz = mu * (u[10] + u[8]);
    return (szz - syy) / 2.0 * sd + syz * cd;
}

/* shear_traction_vol, src/BEM/GF.jl:89-96 (sigma order xx,xy,xz,yy,yz,zz) */
static double traction_vol(int ftype, const double* s, double dip) {
    double sd, cd;
    if (ftype == 0) {
        orc_sincosd(dip, &sd, &cd);
        return -s[1] * sd + s[2] * cd;
    }
    orc_sincosd(2.0 * dip, &sd, &cd);
    return (s[5] - s[3]) / 2.0 * sd + s[4] * cd;
}

/* fault-fault, src/BEM/GF.jl:31-58 (real Toeplitz form; the source is strike cell 1) */
int orc_gf_ff(const orc_fault_mesh* mf, double lambda, double mu, int ftype, int nrept,
              double buffer_ratio, double* st) {
    if (buffer_ratio < 0) return -1;
    const int nx = mf->nx, nxi = mf->nxi;
    const double lrept = (buffer_ratio + 1.0) * (mf->dx * nx);
    const double alpha = (lambda + mu) / (lambda + 2.0 * mu);
    const double ud1 = ftype == 0 ? 1.0 : 0.0, ud2 = ftype == 0 ? 0.0 : 1.0;
#pragma omp parallel for schedule(dynamic)
    for (int l = 0; l < nxi; ++l) {
        double u[12], acc[12];
        for (int j = 0; j < nxi; ++j)
            for (int i = 0; i < nx; ++i) {
                memset(acc, 0, sizeof(acc));
                for (int p = -nrept; p <= nrept; ++p) {
                    double jump = p * lrept;
                    orc_dc3d(mf->x[i], mf->y[j], mf->z[j], alpha, mf->dep, mf->dip,
                             mf->ax[0] + jump, mf->ax[1] + jump, mf->axi[2 * l], mf->axi[2 * l + 1],
                             ud1, ud2, 0.0, u);
                    for (int k = 0; k < 12; ++k) acc[k] += u[k];
                }
                st[i + (size_t)nx * (j + (size_t)nxi * l)] = traction_dc3d(ftype, acc, lambda, mu, mf->dip);
            }
    }
    return 0;
}

/* rfft of [st[:,j,l]; reverse(st[2:end,j,l])], length 2nx-1, nx bins (src/BEM/GF.jl:60-67) */
void orc_gf_ff_dft(int nx, int nxi, const double* st, double* out) {
    const int n = 2 * nx - 1;
    double* cs = (double*)malloc(sizeof(double) * n);
    double* sn = (double*)malloc(sizeof(double) * n);
    for (int m = 0; m < n; ++m) {
        cs[m] = cos(2.0 * M_PI * m / n);
        sn[m] = sin(2.0 * M_PI * m / n);
    }
#pragma omp parallel for schedule(static)
    for (int jl = 0; jl < nxi * nxi; ++jl) {
        const double* col = st + (size_t)nx * jl;
        for (int k = 0; k < nx; ++k) {
            double re = 0.0, im = 0.0;
            for (int m = 0; m < n; ++m) {
                double v = (m < nx) ? col[m] : col[n - m];
                int idx = (int)(((long long)k * m) % n);
                re += v * cs[idx];
                im -= v * sn[idx];
            }
            out[2 * ((size_t)k + (size_t)nx * jl)] = re;
            out[2 * ((size_t)k + (size_t)nx * jl) + 1] = im;
        }
    }
    free(cs);
    free(sn);
}

/* fault -> mantle, src/BEM/GF.jl:123-174 */
int orc_gf_fm(const orc_fault_mesh* mf, const orc_hex_mesh* ma, double lambda, double mu,
              int ftype, int nrept, double buffer_ratio, const double* qc, const double* qw,
              int nq, double* st) {
    if (buffer_ratio < 0) return -1;
    const int ne = ma->ne, nx = mf->nx, ndisl = mf->nx * mf->nxi;
    const size_t M = 6 * (size_t)ne;
    const double lrept = (buffer_ratio + 1.0) * (mf->dx * nx);
    const double alpha = (lambda + mu) / (lambda + 2.0 * mu);
    const double ud1 = ftype == 0 ? 1.0 : 0.0, ud2 = ftype == 0 ? 0.0 : 1.0;
    memset(st, 0, sizeof(double) * M * ndisl);
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < ndisl; ++j) {
        const int q1 = j % nx, q2 = j / nx;
        double u[12], acc[12];
        double* colj = st + M * j;
        for (int i = 0; i < ne; ++i)
            for (int w = 0; w < nq; ++w) {
                double rx = ma->cx[i] + qc[3 * w] * ma->dx[i] / 2.0;
                double ry = ma->cy[i] + qc[3 * w + 1] * ma->dy[i] / 2.0;
                double rz = ma->cz[i] + qc[3 * w + 2] * ma->dz[i] / 2.0;
                memset(acc, 0, sizeof(acc));
                for (int p = -nrept; p <= nrept; ++p) {
                    double jump = p * lrept;
                    orc_dc3d(rx, ry, rz, alpha, mf->dep, mf->dip, mf->ax[2 * q1] + jump,
                             mf->ax[2 * q1 + 1] + jump, mf->axi[2 * q2], mf->axi[2 * q2 + 1],
                             ud1, ud2, 0.0, u);
                    for (int k = 0; k < 12; ++k) acc[k] += u[k];
                }
                double lekk = lambda * (acc[3] + acc[7] + acc[11]);
                colj[i] += qw[w] * (lekk + 2.0 * mu * acc[3]);
                colj[i + ne] += qw[w] * (mu * (acc[4] + acc[6]));
                colj[i + 2 * (size_t)ne] += qw[w] * (mu * (acc[5] + acc[9]));
                colj[i + 3 * (size_t)ne] += qw[w] * (lekk + 2.0 * mu * acc[7]);
                colj[i + 4 * (size_t)ne] += qw[w] * (mu * (acc[8] + acc[10]));
                colj[i + 5 * (size_t)ne] += qw[w] * (lekk + 2.0 * mu * acc[11]);
            }
    }
    return 0;
}

/* mantle -> fault, src/BEM/GF.jl:194-227 (all six unit strains per pair in one evaluation) */
int orc_gf_mf(const orc_hex_mesh* ma, const orc_fault_mesh* mf, double lambda, double mu,
              int ftype, double* st) {
    const int ne = ma->ne, nx = mf->nx, ndisl = mf->nx * mf->nxi;
    const double nu = lambda / 2.0 / (lambda + mu);
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < ne; ++j) {
        double s66[6][6];
        for (int i = 0; i < ndisl; ++i) {
            const int q1 = i % nx, q2 = i / nx;
            orc_hex8_unit_stresses(s66, mf->x[q1], mf->y[q2], mf->z[q2], ma->qx[j], ma->qy[j],
                                   ma->qz[j], ma->dx[j], ma->dy[j], ma->dz[j], mu, nu);
            for (int p = 0; p < 6; ++p)
                st[i + (size_t)ndisl * ((size_t)p * ne + j)] = traction_vol(ftype, s66[p], mf->dip);
        }
    }
    return 0;
}

/* mantle-mantle, src/BEM/GF.jl:250-290 (the optional eigvals check is left to the caller) */
int orc_gf_mm(const orc_hex_mesh* ma, double lambda, double mu, const double* qc,
              const double* qw, int nq, double* st) {
    const int ne = ma->ne;
    const size_t M = 6 * (size_t)ne;
    const double nu = lambda / 2.0 / (lambda + mu);
    memset(st, 0, sizeof(double) * M * M);
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < ne; ++i) {  /* source */
        double s66[6][6];
        for (int j = 0; j < ne; ++j)  /* receiver */
            for (int q = 0; q < nq; ++q) {
                double rx = ma->cx[j] + qc[3 * q] * ma->dx[j] / 2.0;
                double ry = ma->cy[j] + qc[3 * q + 1] * ma->dy[j] / 2.0;
                double rz = ma->cz[j] + qc[3 * q + 2] * ma->dz[j] / 2.0;
                orc_hex8_unit_stresses(s66, rx, ry, rz, ma->qx[i], ma->qy[i], ma->qz[i], ma->dx[i],
                                       ma->dy[i], ma->dz[i], mu, nu);
                for (int p = 0; p < 6; ++p)
                    for (int k = 0; k < 6; ++k)
                        st[((size_t)k * ne + j) + M * ((size_t)p * ne + i)] += s66[p][k] * qw[q];
            }
    }
    return 0;
}

/* ---- receiver subsets (the same loops as above restricted to chosen receivers) -------------
 * For parity checks of device-assembled Green's functions at sizes where the full matrices are
 * too costly for the oracle. Rows are the reference layout's rows: fault->mantle and
 * mantle-mantle row (k, j) = k*ne + j (stress component k at cell j), mantle->fault row i (patch i).
 * out is row-major: one output row per requested reference row, all sources in the reference's
 * column order. */

/* fault -> mantle rows of receiver cells recv[0..nr) (GF.jl:123-174); out (6*nr, N) */
int orc_gf_fm_rows(const orc_fault_mesh* mf, const orc_hex_mesh* ma, double lambda, double mu,
                   int ftype, int nrept, double buffer_ratio, const double* qc, const double* qw,
                   int nq, int nr, const int* recv, double* out) {
    if (buffer_ratio < 0) return -1;
    const int nx = mf->nx, ndisl = mf->nx * mf->nxi;
    const double lrept = (buffer_ratio + 1.0) * (mf->dx * nx);
    const double alpha = (lambda + mu) / (lambda + 2.0 * mu);
    const double ud1 = ftype == 0 ? 1.0 : 0.0, ud2 = ftype == 0 ? 0.0 : 1.0;
    memset(out, 0, sizeof(double) * 6 * (size_t)nr * ndisl);
#pragma omp parallel for schedule(dynamic) collapse(2)
    for (int r = 0; r < nr; ++r)
        for (int j = 0; j < ndisl; ++j) {
            const int i = recv[r], q1 = j % nx, q2 = j / nx;
            double u[12], acc[12], s[6] = {0, 0, 0, 0, 0, 0};
            for (int w = 0; w < nq; ++w) {
                double rx = ma->cx[i] + qc[3 * w] * ma->dx[i] / 2.0;
                double ry = ma->cy[i] + qc[3 * w + 1] * ma->dy[i] / 2.0;
                double rz = ma->cz[i] + qc[3 * w + 2] * ma->dz[i] / 2.0;
                memset(acc, 0, sizeof(acc));
                for (int p = -nrept; p <= nrept; ++p) {
                    double jump = p * lrept;
                    orc_dc3d(rx, ry, rz, alpha, mf->dep, mf->dip, mf->ax[2 * q1] + jump,
                             mf->ax[2 * q1 + 1] + jump, mf->axi[2 * q2], mf->axi[2 * q2 + 1],
                             ud1, ud2, 0.0, u);
                    for (int k = 0; k < 12; ++k) acc[k] += u[k];
                }
                double lekk = lambda * (acc[3] + acc[7] + acc[11]);
                s[0] += qw[w] * (lekk + 2.0 * mu * acc[3]);
                s[1] += qw[w] * (mu * (acc[4] + acc[6]));
                s[2] += qw[w] * (mu * (acc[5] + acc[9]));
                s[3] += qw[w] * (lekk + 2.0 * mu * acc[7]);
                s[4] += qw[w] * (mu * (acc[8] + acc[10]));
                s[5] += qw[w] * (lekk + 2.0 * mu * acc[11]);
            }
            for (int k = 0; k < 6; ++k) out[((size_t)r * 6 + k) * ndisl + j] = s[k];
        }
    return 0;
}

/* mantle -> fault rows of receiver patches recv[0..nr) (GF.jl:194-227); out (nr, 6ne) */
int orc_gf_mf_rows(const orc_hex_mesh* ma, const orc_fault_mesh* mf, double lambda, double mu,
                   int ftype, int nr, const int* recv, double* out) {
    const int ne = ma->ne, nx = mf->nx;
    const size_t M = 6 * (size_t)ne;
    const double nu = lambda / 2.0 / (lambda + mu);
#pragma omp parallel for schedule(dynamic) collapse(2)
    for (int r = 0; r < nr; ++r)
        for (int j = 0; j < ne; ++j) {
            double s66[6][6];
            const int i = recv[r], q1 = i % nx, q2 = i / nx;
            orc_hex8_unit_stresses(s66, mf->x[q1], mf->y[q2], mf->z[q2], ma->qx[j], ma->qy[j],
                                   ma->qz[j], ma->dx[j], ma->dy[j], ma->dz[j], mu, nu);
            for (int p = 0; p < 6; ++p) out[(size_t)r * M + (size_t)p * ne + j] = traction_vol(ftype, s66[p], mf->dip);
        }
    return 0;
}

/* mantle-mantle rows of receiver cells recv[0..nr) (GF.jl:250-290); out (6*nr, 6ne) */
int orc_gf_mm_rows(const orc_hex_mesh* ma, double lambda, double mu, const double* qc,
                   const double* qw, int nq, int nr, const int* recv, double* out) {
    const int ne = ma->ne;
    const size_t M = 6 * (size_t)ne;
    const double nu = lambda / 2.0 / (lambda + mu);
    memset(out, 0, sizeof(double) * 6 * (size_t)nr * M);
#pragma omp parallel for schedule(dynamic) collapse(2)
    for (int r = 0; r < nr; ++r)
        for (int i = 0; i < ne; ++i) {  /* source */
            double s66[6][6];
            const int j = recv[r];      /* receiver */
            for (int q = 0; q < nq; ++q) {
                double rx = ma->cx[j] + qc[3 * q] * ma->dx[j] / 2.0;
                double ry = ma->cy[j] + qc[3 * q + 1] * ma->dy[j] / 2.0;
                double rz = ma->cz[j] + qc[3 * q + 2] * ma->dz[j] / 2.0;
                orc_hex8_unit_stresses(s66, rx, ry, rz, ma->qx[i], ma->qy[i], ma->qz[i], ma->dx[i],
                                       ma->dy[i], ma->dz[i], mu, nu);
                for (int p = 0; p < 6; ++p)
                    for (int k = 0; k < 6; ++k)
                        out[((size_t)r * 6 + k) * M + (size_t)p * ne + i] += s66[p][k] * qw[q];
            }
        }
    return 0;
}
