"""TEST INFRASTRUCTURE ONLY -- independent numpy restatement of the host set-up.

Restates, for checking the product's C++ set-up code (include/fdp_prep.h),
the reference routines that run once before TIME_LOOP:
  CALCUL_VELOCITY  calcul_velocity.F90:16-36
  READ_MODEL       read_model.F90:57-89 (serial build)
  READ_MODEL_PAR   read_model_par.F90:63-74 (scaling)
  PPML             ppml.F90:156-306
  PRE_NR_COEF1     pre_nr_coef1.F90:187-202, NONREF nonref.F90:69-204,
                   HIGDON_FD, HIGCE_FD, HIGCE2_FD, OptAbsBc
  OPEN_SR_FILE     open_sr_file.F90:41-226 (spline, tridag, splint, locate)
Scalar Python loops in the precision ``dt`` (np.float32 or np.float64);
only tests use it, on small grids.
"""
from __future__ import annotations

import math

import numpy as np

COL = {n: i for i, n in enumerate(
    ["MU", "SXX1", "SXX2", "SXX3", "SZZ1", "SZZ2", "SZZ3", "P1", "P2", "P3", "R1U", "R1W", "R2U", "R2W", "R3U", "R3W",
     "R1QX", "R1QZ", "R2QX", "R2QZ", "R3QX", "R3QZ", "AUXW", "AUXQZ"])}


def calcul_velocity(sig1, p, ainv, mu, rel1, rel2, rel3, dt):
    f = dt
    a11, a22, a12, a21 = f(rel1), f(rel2), f(-rel3), f(-rel3)
    b11, b22, b12, b21 = f(sig1), f(ainv), f(p), f(p)
    t11 = f(a11 * b11 + a12 * b21)
    t12 = f(a11 * b12 + a12 * b22)
    t21 = f(a21 * b11 + a22 * b21)
    t22 = f(a21 * b12 + a22 * b22)
    delta = f((t11 + t22) * (t11 + t22) + f(4) * (t12 * t21 - t11 * t22))
    d1 = f(((t11 + t22) + np.sqrt(delta)) / f(2))
    d2 = f(((t11 + t22) - np.sqrt(delta)) / f(2))
    vpf, vps = np.sqrt(d1), np.sqrt(d2)
    vs = np.sqrt(f(rel1 * mu))
    if mu == 0:
        vs = vpf
    return f(vpf), f(vps), f(vs)


def scale_table(table, dt_, h_, dt):
    t = np.array(table, dtype=dt)
    DT, H = dt(dt_), dt(h_)
    for s in ("R1U", "R3U", "R1W", "R3W", "R1QX", "R2QX", "R1QZ", "R2QZ"):
        t[:, COL[s]] = DT * t[:, COL[s]] / H
    for s in ("R2U", "R2W", "R3QX", "R3QZ"):
        t[:, COL[s]] = DT * t[:, COL[s]]
    return t


def expand_jm(rows, mx, mz, tpml, si):
    pmll = 1 - tpml
    nx, nz = mx + 2 * tpml, mz + tpml + 1
    jm = np.zeros((nz, nx), dtype=np.int32)
    first = 2 if si else 0
    for L in range(first, mz + 1):
        jm[L, 1 - pmll: mx + 1 - pmll] = rows[L - first]
        jm[L, : 1 - pmll] = jm[L, 1 - pmll]
        jm[L, mx - pmll:] = jm[L, mx - pmll]
    if si:
        jm[1] = jm[2]
        jm[0] = jm[3]
    jm[mz + 1:] = jm[mz]
    return jm


def _profile(omg, vel, pow_, sf, wc, dtv, tpml, dt):
    f = dt
    oda = [f(1)] * (tpml + 1); odb = [f(1)] * (tpml + 1); odc = [f(0)] * (tpml + 1)
    oda2 = [f(1)] * (tpml + 2); odb2 = [f(1)] * (tpml + 2); odc2 = [f(0)] * (tpml + 2)

    def one(o):
        ap = f(f(1) + f(f(f(sf * o) * f(np.float32(0.075))) / f(np.float32(0.91))))
        denom = f(np.exp(f(f(-f(o / ap)) - f(wc * dtv))))
        a = f(f(f(denom + f(1)) / f(2)) / ap)
        with np.errstate(invalid="ignore", divide="ignore"):
            c = f(f(o / f(o + f(f(wc * ap) * dtv))) * f(denom - f(1)))
        return a, denom, c

    for j in range(1, tpml + 1):
        oda[j], odb[j], odc[j] = one(f(f(omg * vel) * f(np.power(f(np.float32(j)), pow_))))
        oda2[j], odb2[j], odc2[j] = one(f(f(omg * vel) * f(np.power(f(np.float32(j) - np.float32(0.5)), pow_))))
    j = tpml + 1
    oda2[j], odb2[j], odc2[j] = one(f(f(omg * vel) * f(np.power(f(np.float32(j) - np.float32(0.5)), pow_))))
    odd = [f(f(odc[k] + f(2)) / f(odb[k] + f(1))) for k in range(tpml + 1)]
    odd2 = [f(f(odc2[k] + f(2)) / f(odb2[k] + f(1))) for k in range(tpml + 2)]
    return (oda, odb, odc, odd), (oda2, odb2, odc2, odd2)


def ppml(jm, table, mx, mz, tpml, ktbo, r, tau, pow_, sf, wc, dt_, h_, dt):
    f = dt
    R, TAU, POW, SF, WC, DT, H = (f(v) for v in (r, tau, pow_, sf, wc, dt_, h_))
    nx, nz = mx + 2 * tpml, mz + tpml + 1
    if tpml == 0:
        omg = f(0)
    else:
        omg = f(f(f(f(f(-TAU * f(np.log(R))) * DT) / f(np.float32(tpml))) / f(np.power(f(np.float32(tpml)), POW))) / H)
    out = [np.zeros((nz, tpml + 1), dt) for _ in range(8)] + [np.zeros((nx, tpml + 1), dt) for _ in range(4)] + \
          [np.zeros((nz, tpml + 2), dt) for _ in range(8)] + [np.zeros((nx, tpml + 2), dt) for _ in range(4)]

    def vel_of(j, zdir):
        t = table[j - 1]
        if zdir:
            return calcul_velocity(t[COL["SZZ2"]], -t[COL["P2"]], -t[COL["P3"]], t[COL["MU"]],
                                   f(f(H * t[COL["R1W"]]) / DT), f(f(H * t[COL["R2QZ"]]) / DT),
                                   f(f(H * t[COL["R3W"]]) / DT), dt)
        return calcul_velocity(t[COL["SXX1"]], -t[COL["P1"]], -t[COL["P3"]], t[COL["MU"]],
                               f(f(H * t[COL["R1U"]]) / DT), f(f(H * t[COL["R2QX"]]) / DT),
                               f(f(H * t[COL["R3U"]]) / DT), dt)

    for L in range(nz):
        for side, col in ((0, 0), (1, nx - 1)):
            vs = vel_of(int(jm[L, col]), False)[2]
            p1, p2 = _profile(omg, vs, POW, SF, WC, DT, tpml, dt)
            b1, b2 = (0, 12) if side == 0 else (4, 16)
            for k in range(4):
                out[b1 + k][L, :] = p1[k]
                out[b2 + k][L, :] = p2[k]
    if ktbo != 0:
        omg = f(0)
    for x in range(nx):
        vpf = vel_of(int(jm[nz - 1, x]), True)[0]
        p1, p2 = _profile(omg, vpf, POW, SF, WC, DT, tpml, dt)
        for k in range(4):
            out[8 + k][x, :] = p1[k]
            out[20 + k][x, :] = p2[k]
    return out


def _higdon(wb, alfa, beta, dt_, h_):
    wb = float(wb)
    be1, be2 = 1.0, float(alfa) / float(beta)
    ni = float(alfa) * float(dt_) / float(h_)
    qx = (wb * (be1 + ni) - ni) / (be1 + ni) / (1.0 - wb)
    rx = (wb * (be2 + ni) - ni) / (be2 + ni) / (1.0 - wb)
    qt = (wb * (be1 + ni) - be1) / (be1 + ni) / (1.0 - wb)
    rt = (wb * (be2 + ni) - be1) / (be2 + ni) / (1.0 - wb)
    qxt = rxt = wb / (wb - 1.0)
    return _hig_coeffs(qx, rx, qt, rt, qxt, rxt)


def _hig_coeffs(qx, rx, qt, rt, qxt, rxt):
    return [-(qx + rx), -qx * rx, -(qt + rt), -(qx * rt + qt * rx + qxt + rxt), -(qx * rxt + rx * qxt),
            -qt * rt, -(qt * rxt + rt * qxt), -qxt * rxt]


def _higce(wb, alfa, beta, dt_, h_, dt):
    gp = float(dt(dt(alfa * dt_) / h_))
    gs = float(dt(dt(beta * dt_) / h_))
    gs1 = 1.0 + gs
    omw = float(dt(dt(1) - wb))
    wb = float(wb)
    h1x = (gs - wb * gs1) / (gs1 * omw)
    h1t = (1.0 - wb * gs1) / (gs1 * omw)
    hxt = wb / (1.0 - wb)
    c1t, cxt = 1.0 - gp, gp
    return [h1x, 0.0, c1t + h1t, cxt + hxt - h1x * c1t, -h1x * cxt, -h1t * c1t, -hxt * c1t - h1t * cxt, -hxt * cxt]


def _higce2(wb, velh, velce, dt_, h_):
    wb = float(wb)
    ni = float(velh) * float(dt_) / float(h_)
    g = float(velce) * float(dt_) / float(h_)
    qx = (wb * (1.0 + ni) - ni) / (1.0 + ni) / (1.0 - wb)
    rx = (1.0 - g) / (1.0 + g)
    qt = (wb * (1.0 + ni) - 1.0) / (1.0 + ni) / (1.0 - wb)
    rt = -(1.0 - g) / (1.0 + g)
    return _hig_coeffs(qx, rx, qt, rt, wb / (wb - 1.0), -1.0)


def _opt_abs_bc(gplus, gminus, dt_, dx):
    tplus, tminus = dx * math.cos(gplus), dx * math.cos(gminus)
    Rz, Iz = math.cos(dt_), math.sin(dt_)
    Rx, Ix = math.cos(tplus + tminus), math.sin(tplus + tminus)
    Ry, Iy = -(math.cos(tplus) + math.cos(tminus)), -(math.sin(tplus) + math.sin(tminus))
    t1, t2 = Rx * Rz - Ix * Iz, Rx * Iz + Rz * Ix
    t3, t4 = Ry * Rz - Iy * Iz, Ry * Iz + Rz * Iy
    delta = 1.0 / ((Ry + Iy + 2.0 * Rz) * (t1 + t2 - Rz + Iz) + (1.0 - Rx - Ix) * (2.0 + t3 + t4))
    r1 = np.zeros((3, 3)); r0 = np.zeros((3, 3))
    r1[1, 0] = (1.0 - Rz) * (t1 + t2 - Rz + Iz) * delta
    r1[0, 2] = (1.0 - Rz) * (1.0 - Rx - Ix) * delta
    r1[0, 1] = -0.5 - r1[1, 0]
    r1[1, 1] = 1.0 - 2.0 * r1[0, 2]
    r1[1, 2], r1[2, 0], r1[2, 1] = r1[1, 0], r1[0, 2], r1[0, 1]
    t5, t6 = Rx * Rz + Ix * Iz, Rx * Iz - Rz * Ix
    t7, t8 = Ry * Rz + Iy * Iz, Ry * Iz - Rz * Iy
    r0[0, 2] = (-(Rz + Iz - t5 + t6) * (Ry + Iy + 2.0 * Rz) + (1.0 + Rz + t7 - t8) * (1.0 - Rx - Ix)) * delta
    r0[1, 0] = ((1.0 + Rz + t7 - t8) * (t1 + t2 - Rz + Iz) + (Rz + Iz - t5 + t6) * (2.0 + t3 + t4)) * delta
    r0[0, 1] = 0.5 - r0[1, 0]
    r0[1, 1] = 1.0 - 2.0 * r0[0, 2]
    r0[2, 2] = -1.0
    r0[1, 2], r0[2, 0], r0[2, 1] = r0[1, 0], r0[0, 2], r0[0, 1]
    s1 = s2 = 0.0
    for i in range(3):
        for j in range(3):
            s1 += r0[i, j] * r1[i, j]
            s2 += r1[i, j] * r1[i, j]
    ratio = -s1 / s2
    a = r0 + ratio * r1
    return [a[0, 1], a[0, 2], a[1, 0], a[1, 1], a[1, 2], a[2, 0], a[2, 1], a[2, 2]]


def nonref(h_, key, vel, vels, velp, dt_, omg, wb, thpp, thss, dt):
    f = dt
    if key == 0:
        return [f(0)] * 8
    if key == 1:
        return [f(v) for v in _higdon(wb, velp, vels, dt_, h_)]
    if key == 2:
        tmp = f(f(-dt_ * vel) / h_)
        return [f(0), f(0), f(f(1) + tmp), f(f(1) - tmp), f(0), f(0), f(f(-1) - tmp), tmp]
    if key in (3, 9):
        haux = float(f(f(omg / (vel if key == 3 else vels)) * h_))
        return [f(np.float32(v)) for v in _opt_abs_bc(float(thpp), float(thss), float(f(omg * dt_)), haux)]
    if key == 4:
        hv = f(h_ / vel)
        t1 = f(f(dt_ - hv) / f(dt_ + hv))
        t2 = f(f(f(f(2) * h_) / vel) / f(dt_ + hv))
        return [t1, f(0), t2, t2, f(0), t1, f(-1), f(0)]
    if key == 5:
        t = f(f(vel * dt_) / h_)
        return [f(-f(f(1) - t) / f(f(1) + t)), f(0), f(f(f(1) - t) / f(f(1) + t)), f(1), f(0), f(0), f(0), f(0)]
    if key == 6:
        return [f(v) for v in _higce(wb, velp, vels, dt_, h_, dt)]
    if key == 7:
        return [f(v) for v in _higce2(wb, vel, vel, dt_, h_)]
    if key == 8:
        return [f(v) for v in _higce2(wb, vels, velp, dt_, h_)]
    raise ValueError(key)


def bottom_nr(jm, table, mx, mz, tpml, ktbo, dt_, h_, omg, wb, thpp, thss, dt):
    f = dt
    DT, H = f(dt_), f(h_)
    t = table[int(jm[mz, 0]) - 1]
    vpf, vps, vs = calcul_velocity(t[COL["SXX1"]], -t[COL["P1"]], -t[COL["P3"]], t[COL["MU"]],
                                   f(f(H * t[COL["R1U"]]) / DT), f(f(H * t[COL["R2QX"]]) / DT),
                                   f(f(H * t[COL["R3U"]]) / DT), dt)
    args = (DT, f(omg), f(wb), f(thpp), f(thss), dt)
    return np.array(nonref(H, ktbo, vpf, vs, vpf, *args) + nonref(H, ktbo, vs, vs, vpf, *args), dtype=dt)


def source(time, stf, mt2, dt_, h_, key_sour, qr, dt):
    f = dt
    DT, H, QR = f(dt_), f(h_), f(qr)
    x = [f(v) for v in time] + [f(f(mt2) * DT)]
    y = [f(v) for v in stf]
    y.append(y[-1])
    n = len(x)
    # spline with yp1 = ypn = 0 (open_sr_file.F90:121-154), 1-based lists
    X = [None] + x; Y = [None] + y
    a = [f(0)] * (n + 1); b = [f(0)] * (n + 1); c = [f(0)] * (n + 1); r = [f(0)] * (n + 1)
    for i in range(1, n):
        c[i] = f(X[i + 1] - X[i])
    for i in range(1, n):
        r[i] = f(f(6) * f(f(Y[i + 1] - Y[i]) / c[i]))
    rold = list(r)
    for i in range(2, n):
        r[i] = f(rold[i] - rold[i - 1])
    for i in range(2, n):
        a[i] = c[i - 1]
        b[i] = f(f(2) * f(c[i] + a[i]))
    b[1] = b[n] = f(1)
    r[1] = f(f(f(3) / f(X[2] - X[1])) * f(f(f(Y[2] - Y[1]) / f(X[2] - X[1])) - f(0)))
    c[1] = f(0.5)
    r[n] = f(f(f(-3) / f(X[n] - X[n - 1])) * f(f(f(Y[n] - Y[n - 1]) / f(X[n] - X[n - 1])) - f(0)))
    a[n] = f(0.5)
    gam = [f(0)] * (n + 1); u = [f(0)] * (n + 1)
    bet = b[1]
    u[1] = f(r[1] / bet)
    for j in range(2, n + 1):
        gam[j] = f(c[j - 1] / bet)
        bet = f(b[j] - f(a[j] * gam[j]))
        u[j] = f(f(r[j] - f(a[j] * u[j - 1])) / bet)
    for j in range(n - 1, 0, -1):
        u[j] = f(u[j] - f(gam[j + 1] * u[j + 1]))
    y2 = u

    def locate(xv):
        jl, ju = 0, n + 1
        ascnd = X[n] >= X[1]
        while ju - jl > 1:
            jm = (ju + jl) // 2
            if ascnd == (xv >= X[jm]):
                jl = jm
            else:
                ju = jm
        if xv == X[1]:
            return 1
        if xv == X[n]:
            return n - 1
        return jl

    out = np.zeros((mt2, 2), dtype=dt)
    for i in range(1, mt2 + 1):
        t = f(f(i - 1) * DT)
        if t > X[n - 1]:
            break
        klo = max(min(locate(t), n - 1), 1)
        khi = klo + 1
        hh = f(X[khi] - X[klo])
        aa = f(f(X[khi] - t) / hh)
        bb = f(f(t - X[klo]) / hh)
        s1 = f(f(f(aa * Y[klo]) + f(bb * Y[khi]))
               + f(f(f(f(f(f(aa * aa) * aa) - aa) * y2[klo]) + f(f(f(f(bb * bb) * bb) - bb) * y2[khi])) * f(hh * hh))
               / f(6))
        if key_sour == 0:
            s2 = f(f(QR * s1) / f(H * H)); s1 = f(f(f(1) - QR) * s1 / f(H * H))
        elif key_sour == 1:
            s2 = f(0); s1 = f(s1 / f(H * H))
        elif key_sour == 2:
            s2 = f(s1 / f(H * H)); s1 = f(f(QR * s1) / f(H * H))
        elif key_sour == 3:
            s2 = f(s1 / f(H * H)); s1 = f(0)
        else:
            s2 = f(0)
        out[i - 1] = (s1, s2)
    return out
