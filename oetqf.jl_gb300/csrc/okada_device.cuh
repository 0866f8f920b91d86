// Device Okada (1992) finite rectangular dislocation: displacement gradient of the half-space
// field, evaluated on forward-mode dual numbers (value + d/dx, d/dy, d/dz of the receiver) so the
// nine gradient entries are exact derivatives of the displacement formulas. The corner quantities
// (R, logs, arctangents, I-terms) are computed once per Chinnery corner and shared by every slip
// component the caller asks for. Decomposition: u = uA(image) - uA(real) + uB + z uC with the C
// part's vertical component entering with the opposite sign; slip is u(+n) - u(-n) with
// n = (0, -sin dip, cos dip); x along strike, z up.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gbc {

struct Dn {
    double v, x, y, z;
};
__device__ __forceinline__ Dn dk(double v) { return Dn{v, 0.0, 0.0, 0.0}; }
__device__ __forceinline__ Dn operator+(Dn a, Dn b) { return Dn{a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ Dn operator-(Dn a, Dn b) { return Dn{a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ Dn operator-(Dn a) { return Dn{-a.v, -a.x, -a.y, -a.z}; }
__device__ __forceinline__ Dn operator*(Dn a, Dn b) {
    return Dn{a.v * b.v, fma(a.x, b.v, a.v * b.x), fma(a.y, b.v, a.v * b.y), fma(a.z, b.v, a.v * b.z)};
}
__device__ __forceinline__ Dn operator*(Dn a, double s) { return Dn{a.v * s, a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ Dn operator*(double s, Dn a) { return a * s; }
__device__ __forceinline__ Dn drcp(Dn a) {
    double iv = 1.0 / a.v, d = -iv * iv;
    return Dn{iv, a.x * d, a.y * d, a.z * d};
}
__device__ __forceinline__ Dn operator/(Dn a, Dn b) {
    double iv = 1.0 / b.v, q = a.v * iv;
    return Dn{q, (a.x - q * b.x) * iv, (a.y - q * b.y) * iv, (a.z - q * b.z) * iv};
}
__device__ __forceinline__ Dn dsqrt(Dn a) {
    double s = sqrt(a.v), h = 0.5 / s;
    return Dn{s, a.x * h, a.y * h, a.z * h};
}
__device__ __forceinline__ Dn dlog(Dn a) {
    double iv = 1.0 / a.v;
    return Dn{log(a.v), a.x * iv, a.y * iv, a.z * iv};
}
// atan(n/d), 0 on d == 0 (theta at q = 0, the I4 arctangent at xi = 0); smooth derivative
__device__ __forceinline__ Dn datan(Dn n, Dn d) {
    double den = d.v * d.v + n.v * n.v;
    if (den == 0.0) return dk(0.0);
    double id = 1.0 / den;
    return Dn{d.v == 0.0 ? 0.0 : atan(n.v / d.v), (d.v * n.x - n.v * d.x) * id,
              (d.v * n.y - n.v * d.y) * id, (d.v * n.z - n.v * d.z) * id};
}

__host__ __device__ inline void sincosd(double deg, double* s, double* c) {
    double r = fmod(deg, 360.0);
    if (r < 0) r += 360.0;
    int k = (int)floor(r / 90.0 + 0.5);
    double t = (r - 90.0 * k) * (3.14159265358979323846 / 180.0);
    double st = (t == 0.0) ? 0.0 : sin(t), ct = (t == 0.0) ? 1.0 : cos(t);
    switch (k & 3) {
        case 0: *s = st; *c = ct; break;
        case 1: *s = ct; *c = -st; break;
        case 2: *s = -st; *c = -ct; break;
        default: *s = -ct; *c = st; break;
    }
}

// Fault geometry in the dc3d convention, with sin/cos of dip already snapped (|cos| < 1e-6 -> 0).
struct Rect {
    double depth, sd, cd, al1, al2, aw1, aw2;
};
__host__ __device__ inline Rect make_rect(double depth, double dip, double al1, double al2,
                                          double aw1, double aw2) {
    Rect r;
    r.depth = depth;
    sincosd(dip, &r.sd, &r.cd);
    if (fabs(r.cd) < 1e-6) { r.cd = 0.0; r.sd = r.sd > 0 ? 1.0 : -1.0; }
    r.al1 = al1; r.al2 = al2; r.aw1 = aw1; r.aw2 = aw2;
    return r;
}

struct Corner {
    Dn R, R3, th, X11, X32, Y11, Y32, lnRxi, lnRet, yt, dt, ct, Z32, I1, I2, I3, I4, Rdt;
};

// R + a without cancellation for a < 0; false on the singular line R + a = 0.
__device__ __forceinline__ bool plus_stable(Dn R, Dn a, Dn other2, Dn R2, Dn& Rpa, Dn& lnRpa) {
    if (a.v >= 0.0) {
        Rpa = R + a;
        lnRpa = dlog(Rpa);
        return true;
    }
    if (other2.v <= 1e-24 * R2.v) {
        lnRpa = -dlog(R - a);
        return false;
    }
    Rpa = other2 / (R - a);
    lnRpa = dlog(Rpa);
    return true;
}

__device__ __forceinline__ void corner_eval(Dn xi, Dn et, Dn q, Dn z, double sd, double cd,
                                            bool full, Corner& c) {
    Dn xi2 = xi * xi, et2 = et * et, q2 = q * q;
    Dn R2 = xi2 + et2 + q2;
    c.R = dsqrt(R2);
    c.R3 = R2 * c.R;
    Dn Rxi, Ret;
    if (plus_stable(c.R, xi, et2 + q2, R2, Rxi, c.lnRxi)) {
        c.X11 = drcp(c.R * Rxi);
        c.X32 = (2.0 * c.R + xi) / (c.R3 * (Rxi * Rxi));
    } else {
        c.X11 = dk(0.0); c.X32 = dk(0.0);
    }
    if (plus_stable(c.R, et, xi2 + q2, R2, Ret, c.lnRet)) {
        c.Y11 = drcp(c.R * Ret);
        c.Y32 = (2.0 * c.R + et) / (c.R3 * (Ret * Ret));
    } else {
        c.Y11 = dk(0.0); c.Y32 = dk(0.0);
    }
    c.th = datan(xi * et, q * c.R);
    if (!full) return;
    c.yt = et * cd + q * sd;
    c.dt = et * sd - q * cd;
    c.ct = c.dt + z;
    Dn h = q * cd - z;
    c.Z32 = dk(sd) / c.R3 - h * c.Y32;
    c.Rdt = c.R + c.dt;
    Dn lnRdt = dlog(c.Rdt);
    if (cd == 0.0) {
        Dn Rdt2 = c.Rdt * c.Rdt;
        Dn xq = (xi * q) / Rdt2;
        c.I1 = xq * -0.5;
        c.I3 = ((et / c.Rdt + (c.yt * q) / Rdt2) - c.lnRet) * 0.5;
        c.I4 = xq * 0.5;
    } else {
        Dn X = dsqrt(xi2 + q2);
        Dn RX = c.R + X;
        Dn num = et * (X + q * cd) + (X * RX) * sd;
        Dn den = (xi * RX) * cd;
        c.I4 = (xi / c.Rdt) * (sd / cd) + datan(num, den) * (2.0 / (cd * cd));
        c.I3 = (c.yt / c.Rdt) * (1.0 / cd) - (c.lnRet - lnRdt * sd) * (1.0 / (cd * cd));
        c.I1 = (xi / c.Rdt) * (-cd) - c.I4 * sd;
    }
    c.I2 = lnRdt + c.I3 * sd;
}

__device__ __forceinline__ void partA(const Corner& c, Dn xi, Dn et, Dn q, double alpha, int j, Dn o[3]) {
    const double a1 = 0.5 * (1.0 - alpha), a2 = 0.5 * alpha;
    Dn q2 = q * q, hth = c.th * 0.5;
    if (j == 0) {
        o[0] = hth + (xi * q * c.Y11) * a2;
        o[1] = (q / c.R) * a2;
        o[2] = c.lnRet * a1 - (q2 * c.Y11) * a2;
    } else if (j == 1) {
        o[0] = (q / c.R) * a2;
        o[1] = hth + (et * q * c.X11) * a2;
        o[2] = c.lnRxi * a1 - (q2 * c.X11) * a2;
    } else {
        o[0] = c.lnRet * (-a1) - (q2 * c.Y11) * a2;
        o[1] = c.lnRxi * (-a1) - (q2 * c.X11) * a2;
        o[2] = hth - (q * (et * c.X11 + xi * c.Y11)) * a2;
    }
}

__device__ __forceinline__ void partB(const Corner& c, Dn xi, Dn et, Dn q, double alpha, double sd,
                                      double cd, int j, Dn o[3]) {
    const double a3 = (1.0 - alpha) / alpha;
    Dn q2 = q * q, qR = q / c.R, xiRdt = xi / c.Rdt;
    if (j == 0) {
        o[0] = -(xi * q * c.Y11) - c.th - c.I1 * (a3 * sd);
        o[1] = -qR + (c.yt / c.Rdt) * (a3 * sd);
        o[2] = q2 * c.Y11 - c.I2 * (a3 * sd);
    } else if (j == 1) {
        o[0] = -qR + c.I3 * (a3 * sd * cd);
        o[1] = -(et * q * c.X11) - c.th - xiRdt * (a3 * sd * cd);
        o[2] = q2 * c.X11 + c.I4 * (a3 * sd * cd);
    } else {
        o[0] = q2 * c.Y11 - c.I3 * (a3 * sd * sd);
        o[1] = q2 * c.X11 + xiRdt * (a3 * sd * sd);
        o[2] = (q * (et * c.X11 + xi * c.Y11)) - c.th - c.I4 * (a3 * sd * sd);
    }
}

__device__ __forceinline__ void partC(const Corner& c, Dn xi, Dn et, Dn q, Dn z, double alpha,
                                      double sd, double cd, int j, Dn o[3]) {
    const double a4 = 1.0 - alpha;
    Dn q2 = q * q, iR = drcp(c.R), iR3 = drcp(c.R3);
    Dn qY = q * c.Y11, xY = xi * c.Y11;
    Dn ctqR3 = c.ct * q * iR3;
    if (j == 0) {
        o[0] = xY * (a4 * cd) - (xi * q * c.Z32) * alpha;
        o[1] = (iR * cd + qY * (2.0 * sd)) * a4 - ctqR3 * alpha;
        o[2] = qY * (a4 * cd) - ((c.ct * et * iR3 - z * c.Y11) + xi * xi * c.Z32) * alpha;
    } else if (j == 1) {
        o[0] = iR * (a4 * cd) - qY * sd - ctqR3 * alpha;
        o[1] = (c.yt * c.X11) * a4 - (c.ct * et * q * c.X32) * alpha;
        o[2] = -(c.dt * c.X11) - xY * sd - (c.ct * (c.X11 - q2 * c.X32)) * alpha;
    } else {
        o[0] = (iR * sd + qY * cd) * (-a4) - (z * c.Y11 - q2 * c.Z32) * alpha;
        o[1] = xY * (2.0 * a4 * sd) + c.dt * c.X11 - (c.ct * (c.X11 - q2 * c.X32)) * alpha;
        o[2] = (c.yt * c.X11 + xY * cd) * a4 + (q * (c.ct * et * c.X32 + xi * c.Z32)) * alpha;
    }
}

// Accumulates w * grad(u) into G[s][i][j] (= d u_i / d x_j) for each requested slip vector
// slip[s] = (strike, dip, tensile). Returns false (adds nothing) on the fault-edge singularity.
template <int NS>
__device__ __forceinline__ bool dc3d_grad_acc(double x, double y, double z, double alpha,
                                              const Rect& r, const double (&slip)[NS][3],
                                              double w, double (&G)[NS][3][3]) {
    const double sd = r.sd, cd = r.cd;
    {
        double dr = r.depth + z, pr = y * cd + dr * sd, qr = y * sd - dr * cd;
        double xa = x - r.al1, xb = x - r.al2, ea = pr - r.aw1, eb = pr - r.aw2;
        if (qr == 0.0 && ((xa * xb <= 0.0 && ea * eb == 0.0) || (ea * eb <= 0.0 && xa * xb == 0.0)))
            return false;
    }
    const Dn X{x, 1.0, 0.0, 0.0}, Y{y, 0.0, 1.0, 0.0}, Z{z, 0.0, 0.0, 1.0};
    const Dn dR = dk(r.depth) + Z, dI = dk(r.depth) - Z;
    const Dn pR = Y * cd + dR * sd, qR = Y * sd - dR * cd;
    const Dn pI = Y * cd + dI * sd, qI = Y * sd - dI * cd;
    const double f = w / (2.0 * 3.14159265358979323846);
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        const Dn xi = X - dk(k == 0 ? r.al1 : r.al2);
#pragma unroll 1
        for (int m = 0; m < 2; ++m) {
            const double sgn = (k == m) ? f : -f;
            const double aw = (m == 0) ? r.aw1 : r.aw2;
            const Dn etR = pR - dk(aw), etI = pI - dk(aw);
            Corner cR, cI;
            corner_eval(xi, etR, qR, Z, sd, cd, false, cR);
            corner_eval(xi, etI, qI, Z, sd, cd, true, cI);
#pragma unroll 1
            for (int j = 0; j < 3; ++j) {
                bool used = false;
#pragma unroll
                for (int s = 0; s < NS; ++s) used |= (slip[s][j] != 0.0);
                if (!used) continue;
                Dn aR[3], aI[3], b[3], c[3];
                partA(cR, xi, etR, qR, alpha, j, aR);
                partA(cI, xi, etI, qI, alpha, j, aI);
                partB(cI, xi, etI, qI, alpha, sd, cd, j, b);
                partC(cI, xi, etI, qI, Z, alpha, sd, cd, j, c);
                Dn sA0 = aI[0] - aR[0] + b[0], sA1 = aI[1] - aR[1] + b[1], sA2 = aI[2] - aR[2] + b[2];
                Dn ux = sA0 + Z * c[0];
                Dn uy = (sA1 * cd - sA2 * sd) + Z * (c[1] * cd - c[2] * sd);
                Dn uz = (sA1 * sd + sA2 * cd) - Z * (c[1] * sd + c[2] * cd);
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    const double a = sgn * slip[s][j];
                    if (a == 0.0) continue;
                    G[s][0][0] += a * ux.x; G[s][0][1] += a * ux.y; G[s][0][2] += a * ux.z;
                    G[s][1][0] += a * uy.x; G[s][1][1] += a * uy.y; G[s][1][2] += a * uy.z;
                    G[s][2][0] += a * uz.x; G[s][2][1] += a * uz.y; G[s][2][2] += a * uz.z;
                }
            }
        }
    }
    return true;
}

}  // namespace gbc
