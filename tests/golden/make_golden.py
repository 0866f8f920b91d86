"""Generate tests/golden/okada_golden.json: high-precision known answers for the dc3d oracle.

Two independent restatements evaluated in 40-digit arithmetic (mpmath):
  * Okada (1992) finite rectangular source, internal field: displacement from the paper's
    u = uA(image) - uA(real) + uB + z uC decomposition; gradients by 40-digit central
    differences (step 1e-12, truncation ~1e-24).
  * Okada (1985) surface displacement (BSSA 75(4)) -- a separate paper and formula set, used
    as the known answer for z = 0.
Run:  python tests/golden/make_golden.py   (writes okada_golden.json next to this file)
"""
import json
import os
import random

import mpmath as mp

mp.mp.dps = 40


def _parts(xi, et, q, z, sd, cd, alpha):
    R = mp.sqrt(xi**2 + et**2 + q**2)
    yt, dt = et * cd + q * sd, et * sd - q * cd
    ct, X = dt + z, mp.sqrt(xi**2 + q**2)
    X11, X32, lnRxi = 1 / (R * (R + xi)), (2 * R + xi) / (R**3 * (R + xi)**2), mp.log(R + xi)
    Y11, Y32, lnRet = 1 / (R * (R + et)), (2 * R + et) / (R**3 * (R + et)**2), mp.log(R + et)
    th = 0 if q == 0 else mp.atan(xi * et / (q * R))
    Z32 = sd / R**3 - (q * cd - z) * Y32
    a1, a2, a3, a4 = (1 - alpha) / 2, alpha / 2, (1 - alpha) / alpha, 1 - alpha
    A = [[th / 2 + a2 * xi * q * Y11, a2 * q / R, a1 * lnRet - a2 * q * q * Y11],
         [a2 * q / R, th / 2 + a2 * et * q * X11, a1 * lnRxi - a2 * q * q * X11],
         [-a1 * lnRet - a2 * q * q * Y11, -a1 * lnRxi - a2 * q * q * X11, th / 2 - a2 * q * (et * X11 + xi * Y11)]]
    lnRdt = mp.log(R + dt)
    if cd == 0:
        I1 = -(xi / 2) * q / (R + dt)**2
        I3 = (et / (R + dt) + yt * q / (R + dt)**2 - lnRet) / 2
        I4 = xi * q / (2 * (R + dt)**2)
    else:
        I4 = sd / cd * xi / (R + dt) + 2 / cd**2 * mp.atan((et * (X + q * cd) + X * (R + X) * sd) / (xi * (R + X) * cd))
        I3 = yt / (cd * (R + dt)) - (lnRet - sd * lnRdt) / cd**2
        I1 = -xi * cd / (R + dt) - I4 * sd
    I2 = lnRdt + I3 * sd
    B = [[-xi * q * Y11 - th - a3 * I1 * sd, -q / R + a3 * yt / (R + dt) * sd, q * q * Y11 - a3 * I2 * sd],
         [-q / R + a3 * I3 * sd * cd, -et * q * X11 - th - a3 * xi / (R + dt) * sd * cd, q * q * X11 + a3 * I4 * sd * cd],
         [q * q * Y11 - a3 * I3 * sd * sd, q * q * X11 + a3 * xi / (R + dt) * sd * sd, q * (et * X11 + xi * Y11) - th - a3 * I4 * sd * sd]]
    C = [[a4 * xi * Y11 * cd - alpha * xi * q * Z32, a4 * (cd / R + 2 * q * Y11 * sd) - alpha * ct * q / R**3,
          a4 * q * Y11 * cd - alpha * (ct * et / R**3 - z * Y11 + xi * xi * Z32)],
         [a4 * cd / R - q * Y11 * sd - alpha * ct * q / R**3, a4 * yt * X11 - alpha * ct * et * q * X32,
          -dt * X11 - xi * Y11 * sd - alpha * ct * (X11 - q * q * X32)],
         [-a4 * (sd / R + q * Y11 * cd) - alpha * (z * Y11 - q * q * Z32),
          a4 * 2 * xi * Y11 * sd + dt * X11 - alpha * ct * (X11 - q * q * X32),
          a4 * (yt * X11 + xi * Y11 * cd) + alpha * q * (ct * et * X32 + xi * Z32)]]
    return A, B, C


def _sincosd(dip):
    dip = float(dip)
    if dip % 90 == 0:
        k = int(dip // 90) % 4
        return [(0, 1), (1, 0), (0, -1), (-1, 0)][k]
    return mp.sin(mp.radians(dip)), mp.cos(mp.radians(dip))


def okada92_u(x, y, z, alpha, c, dip, al1, al2, aw1, aw2, disl):
    sd, cd = _sincosd(dip)
    sd, cd = mp.mpf(sd), mp.mpf(cd)
    tot = [mp.mpf(0)] * 3
    for k, al in enumerate((al1, al2)):
        for m, aw in enumerate((aw1, aw2)):
            s = 1 if k == m else -1
            xi = x - al
            dr, di = c + z, c - z
            Ar, _, _ = _parts(xi, y * cd + dr * sd - aw, y * sd - dr * cd, -z, sd, cd, alpha)
            Ai, Bi, Ci = _parts(xi, y * cd + di * sd - aw, y * sd - di * cd, z, sd, cd, alpha)
            for j in range(3):
                if disl[j] == 0:
                    continue
                v = [Ai[j][i] - Ar[j][i] + Bi[j][i] for i in range(3)]
                w = Ci[j]
                ux = v[0] + z * w[0]
                uy = v[1] * cd - v[2] * sd + z * (w[1] * cd - w[2] * sd)
                uz = v[1] * sd + v[2] * cd - z * (w[1] * sd + w[2] * cd)
                for i, val in enumerate((ux, uy, uz)):
                    tot[i] += s * disl[j] / (2 * mp.pi) * val
    return tot


def okada92_full(args):
    x, y, z, alpha, c, dip, al1, al2, aw1, aw2, d1, d2, d3 = [mp.mpf(a) for a in args]
    f = lambda X, Y, Z: okada92_u(X, Y, Z, alpha, c, dip, al1, al2, aw1, aw2, (d1, d2, d3))
    u = f(x, y, z)
    h = mp.mpf("1e-12")
    out = [float(v) for v in u]
    for j in range(3):
        e = [0, 0, 0]
        e[j] = h
        if j == 2 and z == 0:  # one-sided in z at the free surface
            fs = [f(x, y, z - k * h) for k in range(5)]
            d = [(25 * fs[0][i] - 48 * fs[1][i] + 36 * fs[2][i] - 16 * fs[3][i] + 3 * fs[4][i]) / (12 * h) for i in range(3)]
        else:
            fp, fm = f(x + e[0], y + e[1], z + e[2]), f(x - e[0], y - e[1], z - e[2])
            d = [(fp[i] - fm[i]) / (2 * h) for i in range(3)]
        out += [float(v) for v in d]
    return out


def okada85_surface(x, y, c, dip, al1, al2, aw1, aw2, disl, lam, mu):
    sd, cd = _sincosd(dip)
    sd, cd = mp.mpf(sd), mp.mpf(cd)
    p, q = y * cd + c * sd, y * sd - c * cd
    f = mu / (lam + mu)
    tot = [mp.mpf(0)] * 3
    for k, al in enumerate((al1, al2)):
        for m, aw in enumerate((aw1, aw2)):
            s = 1 if k == m else -1
            xi, et = x - al, p - aw
            R, X = mp.sqrt(xi**2 + et**2 + q**2), mp.sqrt(xi**2 + q**2)
            yt, dt = et * cd + q * sd, et * sd - q * cd
            th = mp.atan(xi * et / (q * R)) if q != 0 else 0
            if cd != 0:
                I5 = f * 2 / cd * mp.atan((et * (X + q * cd) + X * (R + X) * sd) / (xi * (R + X) * cd)) if xi != 0 else 0
                I4 = f / cd * (mp.log(R + dt) - sd * mp.log(R + et))
                I3 = f * (yt / (cd * (R + dt)) - mp.log(R + et)) + sd / cd * I4
                I1 = f * (-xi / (cd * (R + dt))) - sd / cd * I5
            else:
                I1 = -f / 2 * xi * q / (R + dt)**2
                I3 = f / 2 * (et / (R + dt) + yt * q / (R + dt)**2 - mp.log(R + et))
                I4 = -f * q / (R + dt)
                I5 = -f * xi * sd / (R + dt)
            I2 = f * (-mp.log(R + et)) - I3
            ss = [-(xi * q / (R * (R + et)) + th + I1 * sd), -(yt * q / (R * (R + et)) + q * cd / (R + et) + I2 * sd),
                  -(dt * q / (R * (R + et)) + q * sd / (R + et) + I4 * sd)]
            ds = [-(q / R - I3 * sd * cd), -(yt * q / (R * (R + xi)) + cd * th - I1 * sd * cd),
                  -(dt * q / (R * (R + xi)) + sd * th - I5 * sd * cd)]
            tf = [q * q / (R * (R + et)) - I3 * sd * sd,
                  -dt * q / (R * (R + xi)) - sd * (xi * q / (R * (R + et)) - th) - I1 * sd * sd,
                  yt * q / (R * (R + xi)) + cd * (xi * q / (R * (R + et)) - th) - I5 * sd * sd]
            for j, part in enumerate((ss, ds, tf)):
                for i in range(3):
                    tot[i] += s * disl[j] * part[i] / (2 * mp.pi)
    return [float(v) for v in tot]


def main():
    rng = random.Random(20260101)
    pts = []
    for t in range(24):
        dip = rng.choice([90.0, 90.0, 60.0, 41.0, 33.0, 15.0, 120.0])
        c = rng.uniform(0.5, 3.0)
        z = 0.0 if t % 6 == 0 else rng.uniform(-6.0, -0.05)
        args = [rng.uniform(-5, 5), rng.uniform(-5, 5), z, 2.0 / 3.0, c, dip, -1.0, 2.0, -1.5, 0.2,
                rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1)]
        pts.append({"args": args, "u": okada92_full(args)})
    surf = []
    for t in range(12):
        dip = rng.choice([90.0, 60.0, 41.0, 20.0])
        c = rng.uniform(0.5, 3.0)
        x, y = rng.uniform(-5, 5), rng.uniform(-5, 5)
        disl = [rng.uniform(-1, 1) for _ in range(3)]
        lam, mu = 1.0, 1.0
        u = okada85_surface(mp.mpf(x), mp.mpf(y), mp.mpf(c), mp.mpf(dip), -1, 2, -1.5, 0.2, disl, mp.mpf(lam), mp.mpf(mu))
        surf.append({"args": [x, y, 0.0, (lam + mu) / (lam + 2 * mu), c, dip, -1.0, 2.0, -1.5, 0.2] + disl, "u": u})
    out = {"generator": "tests/golden/make_golden.py", "dc3d_okada92": pts, "surface_okada85": surf}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "okada_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
