/*
 * Oracle: stress from a uniform eigenstrain (anelastic strain) confined in a cuboid in an elastic
 * half-space -- the quantity GeoGreensFunctions.stress_vol_hex8! (Barbot, Moore & Lambert 2017,
 * BSSA 107(2)) returns at the reference's calls src/BEM/GF.jl:215-221 and :277-283.
 *
 * TEST INFRASTRUCTURE ONLY (the FP64 reference the CUDA path is tested against; never linked into the product).
 *
 * Method (not Barbot's closed form, which is not available here): a uniform eigenstrain
 * eps*_ij in a volume equals a continuous stack of planar Volterra dislocations whose slip per
 * unit thickness b satisfies sym(b (x) n) = eps* (the plastic distortion b_i n_j delta(s)).
 * Stacking Okada rectangles (orc_dc3d) through the cuboid and integrating the elastic stress of
 * the stack over the thickness gives the physical stress C:(grad u - eps*), including the
 * -C:eps* term inside the volume. Three stacks cover the six components:
 *   planes normal to y (dip 90, strike x):    eps_xy, eps_yz, eps_yy
 *   planes normal to z (dip 0,  strike x):    eps_xz, eps_zz
 *   planes normal to x (dip 90, strike y):    eps_xx
 * The thickness integral uses Gauss-Legendre panels. Singularities of the integrand in the complex
 * thickness coordinate sit at s_r +- i d, where s_r is the receiver's coordinate along the stack
 * and d its in-plane distance to the rectangle's boundary; panels are bisected until the
 * Bernstein-ellipse parameter rho >= 3 and the order is picked from rho so that rho^(-2n) is
 * below 1e-16.
 *
 * Geometry convention (as the reference's call site fixes it, "T-L-W <=> x-y-z"):
 * x in [qx - T/2, qx + T/2], y in [qy, qy + L], z in [qz - W, qz], z up, no rotation.
 */
#include <math.h>
#include <string.h>
#include "gbc_oracle.h"

#define NORD 4
static const int ORD[NORD] = {4, 8, 12, 16};
static double GLX[NORD][16], GLW[NORD][16];
static int gl_ready = 0;

/* Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n. */
static void gl_rule(int n, double* x, double* w) {
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
            if (fabs(dt) < 1e-16) {
                p0 = 1.0; p1 = t;
                for (int k = 2; k <= n; ++k) {
                    double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                    p0 = p1; p1 = p2;
                }
                dp = n * (t * p1 - p0) / (t * t - 1.0);
                break;
            }
        }
        double p0 = 1.0, p1 = t;
        for (int k = 2; k <= n; ++k) {
            double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
            p0 = p1; p1 = p2;
        }
        double dp = n * (t * p1 - p0) / (t * t - 1.0);
        x[i] = -t;  /* ascending */
        w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
    }
}

static void gl_init(void) {
    if (gl_ready) return;
    for (int k = 0; k < NORD; ++k) gl_rule(ORD[k], GLX[k], GLW[k]);
    __sync_synchronize();
    gl_ready = 1;
}

void orc_gl_table(int which, double* x, double* w) {
    gl_init();
    memcpy(x, GLX[which], ORD[which] * sizeof(double));
    memcpy(w, GLW[which], ORD[which] * sizeof(double));
}

/* in-plane distance from (u, v) to the boundary of [u1,u2] x [v1,v2] */
static double rect_boundary_dist(double u, double v, double u1, double u2, double v1, double v2) {
    if (u >= u1 && u <= u2 && v >= v1 && v <= v2) {
        double d = fmin(fmin(u - u1, u2 - u), fmin(v - v1, v2 - v));
        return d;
    }
    double du = fmax(fmax(u1 - u, 0.0), u - u2);
    double dv = fmax(fmax(v1 - v, 0.0), v - v2);
    return sqrt(du * du + dv * dv);
}

/* Bernstein-ellipse parameter of the point ((sr - m) + i d)/h for the panel [m-h, m+h]. */
static double panel_rho(double sr, double d, double m, double h) {
    double zr = (sr - m) / h, zi = d / h;
    double a = 0.5 * (hypot(zr - 1.0, zi) + hypot(zr + 1.0, zi));
    return a + sqrt(fmax(a * a - 1.0, 0.0));
}

static int order_for_rho(double rho) {
    /* smallest tabulated n with rho^(-2n) <= 1e-16 */
    double need = 18.420680743952367 / log(rho);  /* 8 ln(10) / ln(rho) * ... = ln(1e16)/(2 ln rho) */
    for (int k = 0; k < NORD; ++k)
        if (ORD[k] >= need) return k;
    return NORD - 1;
}

#define RHO_MIN 3.0
#define MAX_DEPTH 24
#define MAX_PANELS 64

/* Fill panels (a_i, b_i, order index) covering [s0, s1], left to right. */
static int make_panels(double s0, double s1, double sr, double d, double* pa, double* pb, int* po) {
    double sa[MAX_DEPTH + 2], sbv[MAX_DEPTH + 2];
    int sdp[MAX_DEPTH + 2], top = 0, np = 0;
    sa[0] = s0; sbv[0] = s1; sdp[0] = 0; top = 1;
    while (top > 0) {
        --top;
        double a = sa[top], b = sbv[top];
        int dep = sdp[top];
        double m = 0.5 * (a + b), h = 0.5 * (b - a);
        double rho = panel_rho(sr, d, m, h);
        if (rho < RHO_MIN && dep < MAX_DEPTH && top + 2 <= MAX_DEPTH + 2 && np + top + 2 <= MAX_PANELS) {
            /* push right first so the left half is processed first */
            sa[top] = m; sbv[top] = b; sdp[top] = dep + 1; ++top;
            sa[top] = a; sbv[top] = m; sdp[top] = dep + 1; ++top;
            continue;
        }
        pa[np] = a; pb[np] = b; po[np] = (rho < RHO_MIN) ? NORD - 1 : order_for_rho(rho);
        ++np;
    }
    return np;
}

/* Accumulate grad u (g[i][j] = du_i/dx_j) scaled by w into G. */
static void acc_grad(double G[3][3], const double u[12], double w) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) G[i][j] += w * u[3 + 3 * j + i];
}

static void grad_to_stress(const double G[3][3], double lam, double mu, double s[6]) {
    double tr = G[0][0] + G[1][1] + G[2][2];
    s[0] = lam * tr + 2.0 * mu * G[0][0];
    s[1] = mu * (G[0][1] + G[1][0]);
    s[2] = mu * (G[0][2] + G[2][0]);
    s[3] = lam * tr + 2.0 * mu * G[1][1];
    s[4] = mu * (G[1][2] + G[2][1]);
    s[5] = lam * tr + 2.0 * mu * G[2][2];
}

/* Stress (6 comps) for each of the 6 unit eigenstrain components (xx,xy,xz,yy,yz,zz):
 * sig6x6[p][k] = sigma_k from eps_p = 1 (tensor component). */
void orc_hex8_unit_stresses(double sig6x6[6][6], double x, double y, double z, double qx,
                            double qy, double qz, double T, double L, double W, double mu,
                            double nu) {
    gl_init();
    double lam = 2.0 * mu * nu / (1.0 - 2.0 * nu);
    double alpha = (lam + mu) / (lam + 2.0 * mu);
    double x1 = qx - 0.5 * T, x2 = qx + 0.5 * T, y1 = qy, y2 = qy + L, z1 = qz - W, z2 = qz;
    double G[6][3][3];
    memset(G, 0, sizeof(G));
    double pa[MAX_PANELS], pb[MAX_PANELS];
    int po[MAX_PANELS];
    double u[12];

    /* stack 1: planes normal to y at s in [y1, y2]; dip 90, strike x, up-dip = z */
    {
        double d = rect_boundary_dist(x, z, x1, x2, z1, z2);
        int np = make_panels(y1, y2, y, d, pa, pb, po);
        double Gxy[3][3] = {{0}}, Gyz[3][3] = {{0}}, Gyy[3][3] = {{0}};
        for (int p = 0; p < np; ++p) {
            int o = po[p], n = ORD[o];
            double m = 0.5 * (pa[p] + pb[p]), h = 0.5 * (pb[p] - pa[p]);
            for (int i = 0; i < n; ++i) {
                double s = m + h * GLX[o][i], w = h * GLW[o][i];
                /* eps_xy = -U1/2, eps_yz = -U2/2, eps_yy = U3 for this plane orientation */
                orc_dc3d(x, y - s, z, alpha, 0.0, 90.0, x1, x2, z1, z2, -2.0, 0.0, 0.0, u);
                acc_grad(Gxy, u, w);
                orc_dc3d(x, y - s, z, alpha, 0.0, 90.0, x1, x2, z1, z2, 0.0, -2.0, 0.0, u);
                acc_grad(Gyz, u, w);
                orc_dc3d(x, y - s, z, alpha, 0.0, 90.0, x1, x2, z1, z2, 0.0, 0.0, 1.0, u);
                acc_grad(Gyy, u, w);
            }
        }
        memcpy(G[1], Gxy, sizeof(Gxy));
        memcpy(G[4], Gyz, sizeof(Gyz));
        memcpy(G[3], Gyy, sizeof(Gyy));
    }
    /* stack 2: horizontal planes at height s in [z1, z2] (depth -s); dip 0, strike x, up-dip = y */
    {
        double d = rect_boundary_dist(x, y, x1, x2, y1, y2);
        int np = make_panels(z1, z2, z, d, pa, pb, po);
        double Gxz[3][3] = {{0}}, Gzz[3][3] = {{0}};
        for (int p = 0; p < np; ++p) {
            int o = po[p], n = ORD[o];
            double m = 0.5 * (pa[p] + pb[p]), h = 0.5 * (pb[p] - pa[p]);
            for (int i = 0; i < n; ++i) {
                double s = m + h * GLX[o][i], w = h * GLW[o][i];
                /* eps_xz = U1/2, eps_zz = U3 */
                orc_dc3d(x, y, z, alpha, -s, 0.0, x1, x2, y1, y2, 2.0, 0.0, 0.0, u);
                acc_grad(Gxz, u, w);
                orc_dc3d(x, y, z, alpha, -s, 0.0, x1, x2, y1, y2, 0.0, 0.0, 1.0, u);
                acc_grad(Gzz, u, w);
            }
        }
        memcpy(G[2], Gxz, sizeof(Gxz));
        memcpy(G[5], Gzz, sizeof(Gzz));
    }
    /* stack 3: planes normal to x at s in [x1, x2], in the frame X = y, Y = -x, Z = z
     * (dip 90, strike X, normal -Y = +x): eps_xx = U3 */
    {
        double d = rect_boundary_dist(y, z, y1, y2, z1, z2);
        int np = make_panels(x1, x2, x, d, pa, pb, po);
        double Gr[3][3] = {{0}};
        for (int p = 0; p < np; ++p) {
            int o = po[p], n = ORD[o];
            double m = 0.5 * (pa[p] + pb[p]), h = 0.5 * (pb[p] - pa[p]);
            for (int i = 0; i < n; ++i) {
                double s = m + h * GLX[o][i], w = h * GLW[o][i];
                /* plane at x = s is at Y = -s: receiver Y - (-s) = -x + s */
                orc_dc3d(y, s - x, z, alpha, 0.0, 90.0, y1, y2, z1, z2, 0.0, 0.0, 1.0, u);
                acc_grad(Gr, u, w);
            }
        }
        /* rotate back: G = Q^T Gr Q with Q = [[0,1,0],[-1,0,0],[0,0,1]] */
        static const double Q[3][3] = {{0, 1, 0}, {-1, 0, 0}, {0, 0, 1}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double acc = 0.0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) acc += Q[a][i] * Gr[a][b] * Q[b][j];
                G[0][i][j] = acc;
            }
    }
    for (int p = 0; p < 6; ++p) grad_to_stress(G[p], lam, mu, sig6x6[p]);
}

void orc_stress_vol_hex8(double sig[6], double x, double y, double z, double qx, double qy,
                         double qz, double T, double L, double W, const double eps[6], double mu,
                         double nu) {
    double s66[6][6];
    orc_hex8_unit_stresses(s66, x, y, z, qx, qy, qz, T, L, W, mu, nu);
    for (int k = 0; k < 6; ++k) {
        double acc = 0.0;
        for (int p = 0; p < 6; ++p) acc += eps[p] * s66[p][k];
        sig[k] = acc;
    }
}
