/*
 * CPU FP64 oracle for the earthquake-cycle hot path (Green's-function assembly + ODE right-hand
 * side + adaptive Runge-Kutta), restated from the reference Oetqf.jl v0.3.6.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the FP64 reference the CUDA path is tested against: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may load it. The product
 * (libgbcycle.so) never links or calls it.
 *
 * Parity status: the reference's Okada and strain-volume kernels live in the third-party Julia
 * package GeoGreensFunctions.jl (compat "0.2", Project.toml:11,32), which is not vendored and has
 * no published golden vectors. The dc3d restatement here follows Okada (1992, BSSA 82(2)) and is
 * pinned by physical identities (equilibrium, traction-free surface, slip jump, far-field decay)
 * and by the reference's own tests (test/BEM/tests.jl); the Okada/strain-volume VALUES are
 * therefore "parity unpinned" against the reference.
 */
#ifndef GBC_ORACLE_H
#define GBC_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Okada (1992) DC3D for a finite rectangle; follows the call at src/BEM/GF.jl:49-53.
 * u = (ux,uy,uz, uxx,uyx,uzx, uxy,uyy,uzy, uxz,uyz,uzz) with u_ij = d u_i / d x_j.
 * Returns 0, 1 (receiver on a fault edge: outputs zero) or 2 (z > 0: outputs zero). */
int orc_dc3d(double x, double y, double z, double alpha, double depth, double dip,
             double al1, double al2, double aw1, double aw2,
             double disl1, double disl2, double disl3, double u[12]);

/* Stress (xx,xy,xz,yy,yz,zz) at (x,y,z) from a uniform eigenstrain in the cuboid
 * [qx-T/2,qx+T/2] x [qy,qy+L] x [qz-W,qz] (z up), in the argument convention of the reference's
 * call at src/BEM/GF.jl:215-221 (T-L-W <=> x-y-z, no rotation). */
void orc_stress_vol_hex8(double sig[6], double x, double y, double z,
                         double qx, double qy, double qz, double T, double L, double W,
                         const double eps[6], double mu, double nu);

/* Mesh views (column-major like the reference's Julia arrays). */
typedef struct {
    int nx, nxi;
    const double *x, *xi, *y, *z;   /* x: nx ; xi,y,z: nxi */
    const double *ax, *axi;         /* (nx,2) and (nxi,2) row-major pairs (lo,hi) */
    double dx, dxi, dep, dip;
} orc_fault_mesh;

typedef struct {
    int ne;
    const double *cx, *cy, *cz, *qx, *qy, *qz, *dx, *dy, *dz;
} orc_hex_mesh;

/* The four stress_greens_function methods of src/BEM/GF.jl (:31, :123, :194, :250). ftype 0 =
 * StrikeSlip, 1 = DipSlip. Outputs are column-major, exactly the reference layouts:
 *   ff: real (nx,nxi,nxi)            fm: (6ne, nx*nxi)
 *   mf: (nx*nxi, 6ne)                mm: (6ne, 6ne)
 * qcoords (3*nq, local coords in [-1,1]) and qweights (nq, already normalised). */
int orc_gf_ff(const orc_fault_mesh* mf, double lambda, double mu, int ftype, int nrept,
              double buffer_ratio, double* st);
int orc_gf_fm(const orc_fault_mesh* mf, const orc_hex_mesh* ma, double lambda, double mu,
              int ftype, int nrept, double buffer_ratio, const double* qcoords,
              const double* qweights, int nq, double* st);
int orc_gf_mf(const orc_hex_mesh* ma, const orc_fault_mesh* mf, double lambda, double mu,
              int ftype, double* st);
int orc_gf_mm(const orc_hex_mesh* ma, double lambda, double mu, const double* qcoords,
              const double* qweights, int nq, double* st);
/* rfft of the symmetric circulant embedding [st[:,j,l]; reverse(st[2:end,j,l])]
 * (src/BEM/GF.jl:60-67): out is complex interleaved (re,im) of shape (nx,nxi,nxi). */
void orc_gf_ff_dft(int nx, int nxi, const double* st, double* st_dft);
/* receiver subsets of the three mantle Green's functions (rows in the reference layout, out
 * row-major: fault->mantle (6*nr, N), mantle->fault (nr, 6ne), mantle-mantle (6*nr, 6ne)) */
int orc_gf_fm_rows(const orc_fault_mesh* mf, const orc_hex_mesh* ma, double lambda, double mu,
                   int ftype, int nrept, double buffer_ratio, const double* qc, const double* qw,
                   int nq, int nr, const int* recv, double* out);
int orc_gf_mf_rows(const orc_hex_mesh* ma, const orc_fault_mesh* mf, double lambda, double mu,
                   int ftype, int nr, const int* recv, double* out);
int orc_gf_mm_rows(const orc_hex_mesh* ma, double lambda, double mu, const double* qc,
                   const double* qw, int nq, int nr, const int* recv, double* out);

/* Right-hand side of src/BEM/equation.jl. gf_dft is the complex (nx,nxi,nxi) kernel. */
typedef struct {
    int nx, nxi, ne;
    const double *a, *b, *L, *sigma;      /* N each */
    double eta, vpl, f0, v0;
    const double *gamma, *n;              /* ne each (viscous); nlaws x ne when nlaws > 1 */
    int nlaws;                            /* CompositePowerLawViscosityProperty: number of laws (0/1 = one) */
    double deps0[6];
    const double *tp, *deps, *beta, *p0;  /* DilatancyProperty (N each); NULL unless dilatancy */
    const double *gf11_dft;               /* complex interleaved (nx,nxi,nxi) */
    const double *gf12, *gf21, *gf22;     /* (6ne,N), (N,6ne), (6ne,6ne) col-major; NULL if ne=0 */
} orc_model;

/* relative_velocity! + dτ_dt! (equation.jl:35-61): traction rate (nx,nxi) from v. */
void orc_dtau_dt(const orc_model* m, const double* v, double* dtau);
/* Tsit5 tableau rows a[s][0..s-1] and error weights (b - bhat). */
void orc_tsit5_tableau(double a[7][6], double e[7]);
/* Stack-quadrature Gauss-Legendre rule `which` (0..3 = 4, 8, 12, 16 nodes). */
void orc_gl_table(int which, double* x, double* w);
/* All six unit-eigenstrain stresses: sig6x6[p][k] = sigma_k for eps_p = 1. */
void orc_hex8_unit_stresses(double sig6x6[6][6], double x, double y, double z, double qx,
                            double qy, double qz, double T, double L, double W, double mu,
                            double nu);

/* Fault-only ode (equation.jl:156-166): u = (v, theta, delta), du likewise; each N. */
void orc_ode_fault(const orc_model* m, const double* v, const double* th, double* dv,
                   double* dth, double* ddelta);
/* Viscoelastic ode (equation.jl:185-205): u = (v, theta, eps(ne,6), sigma(ne,6), delta). */
void orc_ode_visco(const orc_model* m, const double* v, const double* th, const double* sig,
                   double* dv, double* dth, double* deps, double* dsig, double* ddelta);

/* Fault-only ode with dilatancy (equation.jl:168-183, :248-276, :282):
 * u = (v, θ, δ, 𝓅), du likewise; each N. */
void orc_ode_dilatancy(const orc_model* m, const double* v, const double* th, const double* p,
                       double* dv, double* dth, double* ddelta, double* dp);

/* Adaptive integration of the flattened state in ArrayPartition order: Tsit5 (the reference's
 * tests) or VCABM5 (the reference's example, examples/otf-with-mantle.jl:160-162).
 * Returns 0 on reaching t1, else a negative status; fills counters. */
typedef struct {
    double reltol, abstol, dt0, dtmax, dtmin;
    long long maxiters;
    int mantle;                            /* 0: fault-only, 1: viscoelastic, 2: dilatancy state */
    int alg;                               /* 0: Tsit5, 1: VCABM5 (Adams-Bashforth-Moulton, PECE) */
} orc_solver_opts;
typedef struct { long long naccept, nreject, nrhs; double t, dt; int status; } orc_solver_stats;
int orc_integrate(const orc_model* m, double* u, double t0, double t1, const orc_solver_opts* o,
                  orc_solver_stats* st);
long long orc_state_len(const orc_model* m, int mantle);
/* orc_integrate that also records (t, u) at t0 and after every stride-th accepted step, as the
 * reference's wsolve callback does (src/io.jl:51-58), up to max_records; *nrec gets the count. */
int orc_integrate_record(const orc_model* m, double* u, double t0, double t1, const orc_solver_opts* o,
                         orc_solver_stats* st, int stride, long long max_records, double* t_out,
                         double* u_out, long long* nrec);
int orc_num_threads(void);

/* Timed-baseline variant (fastconv.c): the same Toeplitz traction rate through radix-2 FFTs of
 * length P >= 2nx - 1 (H: the real spectra of the even kernel columns, P x nxi x nxi), and many
 * models integrated in parallel, one model per host thread, optionally with that convolution. */
typedef struct { int P, nx, nxi; double* H; } orc_fftconv;
extern _Thread_local const orc_fftconv* orc_tl_fastconv;
int orc_fftconv_init(const orc_model* m, orc_fftconv* c);
void orc_fftconv_free(orc_fftconv* c);
void orc_dtau_dt_fft(const orc_fftconv* c, const orc_model* m, const double* v, double* dtau);
int orc_integrate_many(const orc_model* const* ms, int nm, double* const* us, const double* t0, const double* t1,
                       const orc_solver_opts* o, orc_solver_stats* st, int fft, int nthreads);
/* The VCABM step coefficients psi (k), beta (k) and Adams weights g_0..g_k for order k and step h
 * given psi_prev (the previous step's psi); exposed for tests. */
void orc_abm_coefficients(int k, double h, const double* psi_prev, double* psi, double* beta, double* g);

#ifdef __cplusplus
}
#endif
#endif
