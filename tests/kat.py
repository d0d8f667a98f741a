"""Known-answer checks of the scheme, shared by the oracle tests (CPU) and the
engine tests (GPU).

* Mirror symmetry.  With MX odd, the reference's x-ranges are symmetric about
  x = (MX/2 + 1) H: the 4th-order u/qx columns 4..MX-2 (inh_qx_int.F90:40),
  w/qz columns 3..MX-2 (inh_qz_int.F90:41), the 2nd-order transition
  columns 2 and MX-1 (strain_uw_xx.F90:74-92) and the PML strips on either
  side (strain_uw_xx.F90:60, 95).  An explosive source in TXX, TZZ and PRES
  at LIN_X = (MX+1)/2 (stress_lin_nn.F90:58-63), whose TXX cell sits on that
  axis, in a homogeneous medium therefore gives fields that are mirror
  images: TXX, TZZ, PRES, W and QZ even about the axis (index map
  I -> MX+1-I), U, QX and TXZ odd (I -> MX+2-I, the half-cell staggered
  columns).  In exact arithmetic the symmetry is exact; in floating point
  only the reference's left-to-right sums (``a - b + c - d`` of mirrored
  terms, inh_qz_int.F90:47-48) round differently on the two sides, a few ulp.
  An index slip in any staggered x-stencil breaks it at order one.
* Biot wave speeds.  A plane pulse along z, uniform in x, in a homogeneous
  medium travels at the speeds CALCUL_VELOCITY gives (calcul_velocity.F90:
  16-36): the shear speed sqrt(REL1*MU) for a pulse of u, and the slow P
  speed for a pulse of p once the fast P pulse has run ahead.  Those are
  the inviscid (high-frequency) Biot speeds, so the medium is the sandstone
  with a permeability of 1e-6 m^2: Biot's characteristic frequency is then
  0.016 Hz, far below the pulse's, and the viscous coupling is negligible.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np

from fdporo import job, media

# (field, parity): +1 even about the axis, -1 odd (half-cell staggered)
MIRROR = (("UM", -1), ("WM", 1), ("QX", -1), ("QZ", 1), ("TXX", 1), ("TZZ", 1), ("PRES", 1), ("TXZ", -1))


def mirror_inputs(si: bool, prec: str = "f64", mx: int = 61, mz: int = 50, tpml: int = 8, nsteps: int = 300):
    """Homogeneous sandstone, explosive 300 Hz Ricker at LIN_X = (MX+1)/2."""
    assert mx % 2 == 1
    cfg, med = job.small_homogeneous(mx=mx, mz=mz, nsteps=nsteps, tpml=tpml, f0=300.0, n_rec=1)
    cfg.stress_imaging = si
    cfg.x_source = (mx + 1) / 2 * cfg.h
    cfg.z_source = mz * cfg.h / 2
    inp = job.prepare(cfg, med, prec)
    assert inp.lin_x == (mx + 1) // 2
    return inp


def mirror_defect(eng, inp) -> dict:
    """Largest |f(I) - parity * f(mirror I)| of each field, relative to the
    field's largest value."""
    pmll = 1 - inp.tpml
    out = {}
    for name, parity in MIRROR:
        f = eng.field(name).astype(np.float64)
        cols = np.arange(pmll, pmll + f.shape[1])
        mirror = (inp.mx + 1 - cols) if parity > 0 else (inp.mx + 2 - cols)
        ok = (mirror >= pmll) & (mirror < pmll + f.shape[1])
        a = f[:, cols[ok] - pmll]
        b = parity * f[:, mirror[ok] - pmll]
        scale = float(np.max(np.abs(f))) or 1.0
        out[name] = float(np.max(np.abs(a - b))) / scale
    return out


OPEN_SANDSTONE = replace(media.SANDSTONE, kappa=1e-6)


def plane_wave_inputs(prec: str = "f64", mx: int = 40, mz: int = 400, tpml: int = 10):
    """A column of open sandstone with no source: the pulse is an initial
    condition."""
    cfg, _ = job.small_homogeneous(mx=mx, mz=mz, nsteps=400, tpml=tpml, f0=300.0, n_rec=1)
    cfg.stf_value = np.zeros_like(cfg.stf_value)
    med = media.homogeneous(mx, cfg.n_model_rows, OPEN_SANDSTONE)
    return job.prepare(cfg, med, prec)


def calcul_velocity(inp) -> dict:
    """CALCUL_VELOCITY of the medium's one material (unscaled as ppml.F90:168
    passes it)."""
    from oracle import setup_ref
    t = np.asarray(inp.table[0], np.float64)
    c = setup_ref.COL
    vpf, vps, vs = setup_ref.calcul_velocity(t[c["SXX1"]], -t[c["P1"]], -t[c["P3"]], t[c["MU"]],
                                             inp.h * t[c["R1U"]] / inp.dt, inp.h * t[c["R2QX"]] / inp.dt,
                                             inp.h * t[c["R3U"]] / inp.dt, np.float64)
    return {"vpf": float(vpf), "vps": float(vps), "vs": float(vs)}


def _peak(col: np.ndarray, lo: int, hi: int) -> float:
    """Sub-cell position of the largest |value| in col[lo:hi] (parabola
    through the three samples around it)."""
    seg = np.abs(col[lo:hi])
    k = int(np.argmax(seg)) + lo
    y0, y1, y2 = (abs(float(col[k + d])) for d in (-1, 0, 1))
    return k + 0.5 * (y0 - y2) / (y0 - 2 * y1 + y2)


def plane_wave_speed(eng, inp, field: str, speed: float, z0: int = 200, sigma: float = 6.0,
                     levels=(100, 300)) -> float:
    """Sets a Gaussian pulse of ``field`` along z (uniform in x) at row z0,
    runs the engine, and returns the speed of the down-going pulse between
    the two levels, found near where ``speed`` would carry it."""
    shape = eng.field(field).shape
    z = np.arange(shape[0])[:, None]
    amp = 1e-3 if field in ("UM", "WM", "QX", "QZ") else 1e3
    eng.set_field(field, (amp * np.exp(-((z - z0) / sigma) ** 2) * np.ones((1, shape[1]))).astype(eng.dtype))
    col = inp.tpml + inp.mx // 2
    pos, done = [], 0
    for lev in levels:
        eng.time_loop(done + 1, lev)
        done = lev
        f = eng.field(field)[:, col].astype(np.float64)
        travel = speed * lev * inp.dt / inp.h
        pos.append(_peak(f, int(z0 + 0.7 * travel), int(z0 + 1.3 * travel) + 2))
    return (pos[1] - pos[0]) * inp.h / ((levels[1] - levels[0]) * inp.dt)
