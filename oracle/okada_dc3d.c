/*
 * Oracle: Okada (1992) internal deformation of a finite rectangular dislocation in an elastic
 * half-space (BSSA 82(2), 1018-1040), the arithmetic behind GeoGreensFunctions.dc3d that the
 * reference calls at src/BEM/GF.jl:49-53 and :156-160 (dc3d_cache at :43,:142).
 *
 * TEST INFRASTRUCTURE ONLY (the FP64 reference the CUDA path is tested against; never linked into the product).
 *
 * Written from the paper's decomposition u = uA(image) - uA(real) + uB + z uC with Chinnery's
 * corner notation. The displacement formulas per corner are evaluated on forward-mode dual
 * numbers carrying d/dx, d/dy, d/dz of the receiver, so the 9 gradient entries are the exact
 * derivatives of the displacement expressions (no separate derivative tables). The formulas were
 * pinned by physical identities, checked by tests/test_oracle_okada.py: Navier equilibrium, a
 * traction-free surface at z = 0, the slip jump across the fault, and far-field decay.
 *
 * Conventions: x along strike, z up (receivers need z <= 0); the fault passes through the line
 * (x, 0, -depth) and dips at `dip` degrees; al1..al2 along strike, aw1..aw2 up-dip; slip
 * (disl1, disl2, disl3) = (strike, up-dip, opening) is u(+n) - u(-n), n = (0, -sin dip, cos dip).
 */
#include <math.h>
#include <string.h>
#include "gbc_oracle.h"

typedef struct { double v, x, y, z; } dn;

static inline dn K(double v) { dn r = {v, 0, 0, 0}; return r; }
static inline dn ad(dn a, dn b) { dn r = {a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline dn sb(dn a, dn b) { dn r = {a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline dn ml(dn a, dn b) {
    dn r = {a.v * b.v, a.x * b.v + a.v * b.x, a.y * b.v + a.v * b.y, a.z * b.v + a.v * b.z};
    return r;
}
static inline dn sc(dn a, double s) { dn r = {a.v * s, a.x * s, a.y * s, a.z * s}; return r; }
static inline dn dv(dn a, dn b) {
    double iv = 1.0 / b.v, q = a.v * iv;
    dn r = {q, (a.x - q * b.x) * iv, (a.y - q * b.y) * iv, (a.z - q * b.z) * iv};
    return r;
}
static inline dn rc(dn a) {
    double iv = 1.0 / a.v, d = -iv * iv;
    dn r = {iv, a.x * d, a.y * d, a.z * d};
    return r;
}
static inline dn sq(dn a) {
    double s = sqrt(a.v), h = 0.5 / s;
    dn r = {s, a.x * h, a.y * h, a.z * h};
    return r;
}
static inline dn lg(dn a) {
    double iv = 1.0 / a.v;
    dn r = {log(a.v), a.x * iv, a.y * iv, a.z * iv};
    return r;
}
/* atan(n/d) taking the value 0 on d == 0 (the paper's convention for theta at q = 0 and for the
 * I4 arctangent at xi = 0); the derivative is the smooth (d dn - n dd)/(d^2 + n^2) on both sides. */
static inline dn at(dn n, dn d) {
    double den = d.v * d.v + n.v * n.v;
    if (den == 0.0) return K(0.0);
    double id = 1.0 / den;
    dn r = {d.v == 0.0 ? 0.0 : atan(n.v / d.v), (d.v * n.x - n.v * d.x) * id,
            (d.v * n.y - n.v * d.y) * id, (d.v * n.z - n.v * d.z) * id};
    return r;
}

/* sin/cos of an angle in degrees, exact at multiples of 90 (the reference uses sind/cosd). */
void orc_sincosd(double deg, double* s, double* c) {
    double r = fmod(deg, 360.0);
    if (r < 0) r += 360.0;
    int k = (int)floor(r / 90.0 + 0.5);
    double t = (r - 90.0 * k) * (M_PI / 180.0);
    double st = (t == 0.0) ? 0.0 : sin(t), ct = (t == 0.0) ? 1.0 : cos(t);
    switch (k & 3) {
    case 0: *s = st; *c = ct; break;
    case 1: *s = ct; *c = -st; break;
    case 2: *s = -st; *c = -ct; break;
    default: *s = -ct; *c = st; break;
    }
}

/* Per-corner quantities shared by the A/B/C parts. */
typedef struct {
    dn R, R3, th, X11, X32, Y11, Y32, lnRxi, lnRet, yt, dt, ct, Z32, I1, I2, I3, I4, Rdt;
} corner;

/* R+a computed without cancellation when a < 0: (R+a) = (R^2 - a^2)/(R - a). Returns 0 in the
 * singular case (receiver on the line R + a = 0), where the paper drops the X/Y terms and uses
 * -ln(R - a) for ln(R + a). */
static int plus_stable(dn R, dn a, dn other2, dn R2, dn* Rpa, dn* lnRpa) {
    if (a.v >= 0.0) {
        *Rpa = ad(R, a);
        *lnRpa = lg(*Rpa);
        return 1;
    }
    if (other2.v <= 1e-24 * R2.v) {
        *lnRpa = sc(lg(sb(R, a)), -1.0);
        return 0;
    }
    *Rpa = dv(other2, sb(R, a));
    *lnRpa = lg(*Rpa);
    return 1;
}

static void corner_eval(dn xi, dn et, dn q, dn z, double sd, double cd, int full, corner* c) {
    dn xi2 = ml(xi, xi), et2 = ml(et, et), q2 = ml(q, q);
    dn R2 = ad(ad(xi2, et2), q2);
    c->R = sq(R2);
    c->R3 = ml(R2, c->R);
    dn Rxi, Ret;
    if (plus_stable(c->R, xi, ad(et2, q2), R2, &Rxi, &c->lnRxi)) {
        c->X11 = rc(ml(c->R, Rxi));
        c->X32 = dv(ad(sc(c->R, 2.0), xi), ml(c->R3, ml(Rxi, Rxi)));
    } else {
        c->X11 = K(0); c->X32 = K(0);
    }
    if (plus_stable(c->R, et, ad(xi2, q2), R2, &Ret, &c->lnRet)) {
        c->Y11 = rc(ml(c->R, Ret));
        c->Y32 = dv(ad(sc(c->R, 2.0), et), ml(c->R3, ml(Ret, Ret)));
    } else {
        c->Y11 = K(0); c->Y32 = K(0);
    }
    c->th = at(ml(xi, et), ml(q, c->R));
    if (!full) return;
    c->yt = ad(sc(et, cd), sc(q, sd));
    c->dt = sb(sc(et, sd), sc(q, cd));
    c->ct = ad(c->dt, z);
    dn h = sb(sc(q, cd), z);
    c->Z32 = sb(dv(K(sd), c->R3), ml(h, c->Y32));
    c->Rdt = ad(c->R, c->dt);
    dn lnRdt = lg(c->Rdt);
    if (cd == 0.0) {
        dn Rdt2 = ml(c->Rdt, c->Rdt);
        dn xq = dv(ml(xi, q), Rdt2);
        c->I1 = sc(xq, -0.5);
        c->I3 = sc(sb(ad(dv(et, c->Rdt), dv(ml(c->yt, q), Rdt2)), c->lnRet), 0.5);
        c->I4 = sc(xq, 0.5);
    } else {
        dn X = sq(ad(xi2, q2));
        dn RX = ad(c->R, X);
        dn num = ad(ml(et, ad(X, sc(q, cd))), sc(ml(X, RX), sd));
        dn den = sc(ml(xi, RX), cd);
        c->I4 = ad(sc(dv(xi, c->Rdt), sd / cd), sc(at(num, den), 2.0 / (cd * cd)));
        c->I3 = sb(sc(dv(c->yt, c->Rdt), 1.0 / cd),
                   sc(sb(c->lnRet, sc(lnRdt, sd)), 1.0 / (cd * cd)));
        c->I1 = sb(sc(dv(xi, c->Rdt), -cd), sc(c->I4, sd));
    }
    c->I2 = ad(lnRdt, sc(c->I3, sd));
}

/* Part A (full-space term) for slip type j, components in the fault frame
 * (strike, up-dip, normal). */
static void partA(const corner* c, dn xi, dn et, dn q, double alpha, int j, dn o[3]) {
    double a1 = 0.5 * (1.0 - alpha), a2 = 0.5 * alpha;
    dn q2 = ml(q, q), hth = sc(c->th, 0.5);
    if (j == 0) {
        o[0] = ad(hth, sc(ml(ml(xi, q), c->Y11), a2));
        o[1] = sc(dv(q, c->R), a2);
        o[2] = sb(sc(c->lnRet, a1), sc(ml(q2, c->Y11), a2));
    } else if (j == 1) {
        o[0] = sc(dv(q, c->R), a2);
        o[1] = ad(hth, sc(ml(ml(et, q), c->X11), a2));
        o[2] = sb(sc(c->lnRxi, a1), sc(ml(q2, c->X11), a2));
    } else {
        o[0] = sb(sc(c->lnRet, -a1), sc(ml(q2, c->Y11), a2));
        o[1] = sb(sc(c->lnRxi, -a1), sc(ml(q2, c->X11), a2));
        o[2] = sb(hth, sc(ml(q, ad(ml(et, c->X11), ml(xi, c->Y11))), a2));
    }
}

/* Part B (surface correction independent of z) for slip type j. */
static void partB(const corner* c, dn xi, dn et, dn q, double alpha, double sd, double cd, int j,
                  dn o[3]) {
    double a3 = (1.0 - alpha) / alpha;
    dn q2 = ml(q, q);
    dn qR = dv(q, c->R);
    dn xiRdt = dv(xi, c->Rdt);
    if (j == 0) {
        o[0] = sb(sb(sc(ml(ml(xi, q), c->Y11), -1.0), c->th), sc(c->I1, a3 * sd));
        o[1] = ad(sc(qR, -1.0), sc(dv(c->yt, c->Rdt), a3 * sd));
        o[2] = sb(ml(q2, c->Y11), sc(c->I2, a3 * sd));
    } else if (j == 1) {
        o[0] = ad(sc(qR, -1.0), sc(c->I3, a3 * sd * cd));
        o[1] = sb(sb(sc(ml(ml(et, q), c->X11), -1.0), c->th), sc(xiRdt, a3 * sd * cd));
        o[2] = ad(ml(q2, c->X11), sc(c->I4, a3 * sd * cd));
    } else {
        o[0] = sb(ml(q2, c->Y11), sc(c->I3, a3 * sd * sd));
        o[1] = ad(ml(q2, c->X11), sc(xiRdt, a3 * sd * sd));
        o[2] = sb(sb(ml(q, ad(ml(et, c->X11), ml(xi, c->Y11))), c->th), sc(c->I4, a3 * sd * sd));
    }
}

/* Part C (surface correction multiplied by z) for slip type j. */
static void partC(const corner* c, dn xi, dn et, dn q, dn z, double alpha, double sd, double cd,
                  int j, dn o[3]) {
    double a4 = 1.0 - alpha;
    dn q2 = ml(q, q);
    dn iR = rc(c->R);
    dn iR3 = rc(c->R3);
    dn qY = ml(q, c->Y11), xY = ml(xi, c->Y11);
    dn ctqR3 = ml(ml(c->ct, q), iR3);
    if (j == 0) {
        o[0] = sb(sc(xY, a4 * cd), sc(ml(ml(xi, q), c->Z32), alpha));
        o[1] = sb(sc(ad(sc(iR, cd), sc(qY, 2.0 * sd)), a4), sc(ctqR3, alpha));
        o[2] = sb(sc(qY, a4 * cd),
                  sc(ad(sb(ml(ml(c->ct, et), iR3), ml(z, c->Y11)), ml(ml(xi, xi), c->Z32)), alpha));
    } else if (j == 1) {
        o[0] = sb(sb(sc(iR, a4 * cd), sc(qY, sd)), sc(ctqR3, alpha));
        o[1] = sb(sc(ml(c->yt, c->X11), a4), sc(ml(ml(ml(c->ct, et), q), c->X32), alpha));
        o[2] = sb(sb(sc(ml(c->dt, c->X11), -1.0), sc(xY, sd)),
                  sc(ml(c->ct, sb(c->X11, ml(q2, c->X32))), alpha));
    } else {
        o[0] = sb(sc(ad(sc(iR, sd), sc(qY, cd)), -a4),
                  sc(sb(ml(z, c->Y11), ml(q2, c->Z32)), alpha));
        o[1] = sb(ad(sc(xY, 2.0 * a4 * sd), ml(c->dt, c->X11)),
                  sc(ml(c->ct, sb(c->X11, ml(q2, c->X32))), alpha));
        o[2] = ad(sc(ad(ml(c->yt, c->X11), sc(xY, cd)), a4),
                  sc(ml(q, ad(ml(ml(c->ct, et), c->X32), ml(xi, c->Z32))), alpha));
    }
}

int orc_dc3d(double x, double y, double z, double alpha, double depth, double dip,
             double al1, double al2, double aw1, double aw2,
             double disl1, double disl2, double disl3, double u[12]) {
    memset(u, 0, 12 * sizeof(double));
    if (z > 0.0) return 2;
    double sd, cd;
    orc_sincosd(dip, &sd, &cd);
    if (fabs(cd) < 1e-6) { cd = 0.0; sd = sd > 0 ? 1.0 : -1.0; }
    const double disl[3] = {disl1, disl2, disl3};
    const double al[2] = {al1, al2}, aw[2] = {aw1, aw2};

    /* receiver on a fault edge: singular, outputs zero (as the paper prescribes) */
    {
        double dr = depth + z, pr = y * cd + dr * sd, qr = y * sd - dr * cd;
        double xa = x - al1, xb = x - al2, ea = pr - aw1, eb = pr - aw2;
        if (qr == 0.0 && ((xa * xb <= 0.0 && ea * eb == 0.0) || (ea * eb <= 0.0 && xa * xb == 0.0)))
            return 1;
    }
    dn X = {x, 1, 0, 0}, Y = {y, 0, 1, 0}, Z = {z, 0, 0, 1};
    /* real source: d = depth + z; image: d = depth - z */
    dn dR = ad(K(depth), Z), dI = sb(K(depth), Z);
    dn pR = ad(sc(Y, cd), sc(dR, sd)), qR = sb(sc(Y, sd), sc(dR, cd));
    dn pI = ad(sc(Y, cd), sc(dI, sd)), qI = sb(sc(Y, sd), sc(dI, cd));
    dn tot[3] = {K(0), K(0), K(0)};
    for (int k = 0; k < 2; ++k) {
        dn xi = sb(X, K(al[k]));
        for (int m = 0; m < 2; ++m) {
            double sgn = (k == m) ? 1.0 : -1.0;
            dn etR = sb(pR, K(aw[m])), etI = sb(pI, K(aw[m]));
            corner cR, cI;
            corner_eval(xi, etR, qR, Z, sd, cd, 0, &cR);
            corner_eval(xi, etI, qI, Z, sd, cd, 1, &cI);
            for (int j = 0; j < 3; ++j) {
                if (disl[j] == 0.0) continue;
                dn aR[3], aI[3], b[3], c[3];
                partA(&cR, xi, etR, qR, alpha, j, aR);
                partA(&cI, xi, etI, qI, alpha, j, aI);
                partB(&cI, xi, etI, qI, alpha, sd, cd, j, b);
                partC(&cI, xi, etI, qI, Z, alpha, sd, cd, j, c);
                /* fault frame (strike, up-dip, normal) -> (x, y, z); the C part's vertical
                 * component enters with the opposite sign */
                dn sA[3], sC[3];
                for (int i = 0; i < 3; ++i) { sA[i] = ad(sb(aI[i], aR[i]), b[i]); sC[i] = c[i]; }
                dn ux = ad(sA[0], ml(Z, sC[0]));
                dn uy = ad(sb(sc(sA[1], cd), sc(sA[2], sd)), ml(Z, sb(sc(sC[1], cd), sc(sC[2], sd))));
                dn uz = sb(ad(sc(sA[1], sd), sc(sA[2], cd)), ml(Z, ad(sc(sC[1], sd), sc(sC[2], cd))));
                double f = sgn * disl[j] / (2.0 * M_PI);
                tot[0] = ad(tot[0], sc(ux, f));
                tot[1] = ad(tot[1], sc(uy, f));
                tot[2] = ad(tot[2], sc(uz, f));
            }
        }
    }
    for (int i = 0; i < 3; ++i) {
        u[i] = tot[i].v;
        u[3 + i] = tot[i].x;  /* d u_i / dx */
        u[6 + i] = tot[i].y;  /* d u_i / dy */
        u[9 + i] = tot[i].z;  /* d u_i / dz */
    }
    return 0;
}
