"""Set-up of one shot, in the order of the reference's main program.

``prepare`` turns a :class:`JobConfig` (the namelist values of the
reference's ``<JOB>.IN``/``<JOB>.INM``) and a :class:`~fdporo.media.Medium`
(its ``.JMH``/``.MO`` contents) into the inputs of the time-stepping ABI,
following main.F90:60-82: READ_OPEN (grid and source cell), AUX1,
READ_MODEL (JM expansion), READ_MODEL_PAR (table scaling), OPEN_SR_FILE
(source time function), PRE_NR_COEF1 (bottom coefficients), PPML
(profiles).  The arithmetic runs in libfdp's host set-up code
(include/fdp_prep.h); ``run`` then drives any engine with the
:class:`~fdporo.engine.Engine` interface.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from dataclasses import dataclass, field

import numpy as np

from . import native
from .media import Medium
from .native import FDP_F32, FDP_F64, FDP_REC_TLP, FDP_REC_TLQ, FDP_REC_TLV, FdpError


def _f32(x: float) -> float:
    return float(np.float32(x))


def nint(x: float) -> int:
    """Fortran NINT: round half away from zero."""
    return int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


def ricker(t: np.ndarray, f0: float, t0: float | None = None) -> np.ndarray:
    t0 = 1.2 / f0 if t0 is None else t0
    a = (np.pi * f0 * (t - t0)) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


@dataclass
class JobConfig:
    mx: int
    mz: int                 # MZ as read from CONTROLDATA2, before the stress-imaging shift
    h: float
    dt: float
    mt2: int                # number of time levels (MT2 = INT(MT/DT)+1)
    tpml: int = 20
    stress_imaging: bool = True
    x_source: float = 0.0
    z_source: float = 0.0
    xbmin: float = 0.0
    key_sour: int = 1
    qr: float = 0.0
    # CONTROLDATA1 defaults (read_open.F90:118-126): default-real literals
    r: float = _f32(0.001)
    tau: float = 1.5
    pow_: float = 2.0
    sf: float = 0.0
    wc: float = 0.0
    # NONREF defaults (read_open.F90:174-184)
    ktbo: int = 0
    omg: float = 0.0        # NONREF OMG before the division by 2*pi
    wb: float = 0.4
    thpple: float = 0.19757
    thssle: float = 0.70511
    # STF.DAT samples (time, value)
    stf_time: np.ndarray = field(default_factory=lambda: np.zeros(0))
    stf_value: np.ndarray = field(default_factory=lambda: np.zeros(0))
    # REC.DAT and KEYS
    irecx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    lrecx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    irecz: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    lrecz: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    key_tlv: bool = True
    key_tlq: bool = False
    key_tlp: bool = False

    @property
    def mz_grid(self) -> int:
        return self.mz + 2 if self.stress_imaging else self.mz

    @property
    def n_model_rows(self) -> int:
        return self.mz_grid - 1 if self.stress_imaging else self.mz_grid + 1

    @property
    def rec_flags(self) -> int:
        return ((FDP_REC_TLV if self.key_tlv else 0) | (FDP_REC_TLQ if self.key_tlq else 0)
                | (FDP_REC_TLP if self.key_tlp else 0))


@dataclass
class Inputs:
    precision: int
    mx: int
    mz: int
    tpml: int
    stress_imaging: bool
    lin_x: int
    lin_z: int
    h: float
    dt: float
    jm: np.ndarray
    table: np.ndarray
    profiles: list
    ab: np.ndarray
    sourtf: np.ndarray
    irecx: np.ndarray
    lrecx: np.ndarray
    irecz: np.ndarray
    lrecz: np.ndarray
    rec_flags: int

    @property
    def nx(self) -> int:
        return self.mx + 2 * self.tpml

    @property
    def nz(self) -> int:
        return self.mz + self.tpml + 1

    @property
    def mt2(self) -> int:
        return self.sourtf.shape[0]

    @property
    def pmll(self) -> int:
        return 1 - self.tpml

    @property
    def pmlxh(self) -> int:
        return self.mx + self.tpml

    @property
    def cells(self) -> int:
        return self.nx * self.nz


def source_cell(cfg: JobConfig, h_pp: float) -> tuple[int, int]:
    """LIN_X, LIN_Z as READ_OPEN computes them (read_open.F90:163-169);
    X_SOURCE, Z_SOURCE and XBMIN are default-real variables there."""
    xs = np.float32(abs(cfg.x_source))
    zs = np.float32(abs(cfg.z_source))
    if cfg.stress_imaging:
        zs = np.float32(float(zs) + 2.0 * h_pp)
    lin_x = nint(float(np.float32(xs - np.float32(cfg.xbmin))) / h_pp)
    lin_z = nint(float(zs) / h_pp)
    return lin_x, lin_z


def prepare(cfg: JobConfig, medium: Medium, precision: str = "f32") -> Inputs:
    lib = native.load()
    prec = FDP_F64 if precision in ("f64", 8) else FDP_F32
    dt_ = np.float64 if prec == FDP_F64 else np.float32
    pp = (lambda v: float(dt_(v)))
    h, dt = pp(cfg.h), pp(cfg.dt)
    mx, mz, tpml, si = cfg.mx, cfg.mz_grid, cfg.tpml, cfg.stress_imaging
    nx, nz = mx + 2 * tpml, mz + tpml + 1
    lin_x, lin_z = source_cell(cfg, h)
    # READ_MODEL
    rows = np.ascontiguousarray(medium.jm_rows, dtype=np.int32)
    if rows.shape != (cfg.n_model_rows, mx):
        raise ValueError(f"JM rows {rows.shape} != {(cfg.n_model_rows, mx)}")
    jm = np.zeros((nz, nx), dtype=np.int32)
    rc = lib.fdp_prep_expand_jm(mx, mz, tpml, int(si), rows.ctypes.data_as(C.POINTER(C.c_int32)),
                                jm.ctypes.data_as(C.POINTER(C.c_int32)))
    if rc:
        raise FdpError(rc, "fdp_prep_expand_jm")
    # READ_MODEL_PAR: the .MO values are read in precision PP, then scaled
    table = np.array(medium.table, dtype=dt_, order="C", copy=True)  # scaled in place below
    rc = lib.fdp_prep_scale_table(prec, table.shape[0], dt, h, table.ctypes.data_as(C.c_void_p))
    if rc:
        raise FdpError(rc, "fdp_prep_scale_table")
    # OPEN_SR_FILE
    st = np.ascontiguousarray(cfg.stf_time, dtype=dt_)
    sv = np.ascontiguousarray(cfg.stf_value, dtype=dt_)
    sourtf = np.zeros((cfg.mt2, 2), dtype=dt_)
    rc = lib.fdp_prep_source(prec, len(st), st.ctypes.data_as(C.c_void_p), sv.ctypes.data_as(C.c_void_p), cfg.mt2,
                             dt, h, cfg.key_sour, pp(cfg.qr), sourtf.ctypes.data_as(C.c_void_p))
    if rc:
        raise FdpError(rc, "fdp_prep_source")
    # PRE_NR_COEF1 (bottom); OMG = OMG/(2 pi) as read_open.F90:188 does
    ab = np.zeros(16, dtype=dt_)
    omg = pp(pp(cfg.omg) / 6.283185307179586476925286766559)
    rc = lib.fdp_prep_bottom_nr(prec, mx, mz, tpml, cfg.ktbo, dt, h, omg, pp(cfg.wb), pp(cfg.thpple), pp(cfg.thssle),
                                jm.ctypes.data_as(C.POINTER(C.c_int32)), table.shape[0],
                                table.ctypes.data_as(C.c_void_p), ab.ctypes.data_as(C.c_void_p))
    if rc:
        raise FdpError(rc, "fdp_prep_bottom_nr")
    # PPML
    shapes = ([(nz, tpml + 1)] * 8 + [(nx, tpml + 1)] * 4 + [(nz, tpml + 2)] * 8 + [(nx, tpml + 2)] * 4)
    profiles = [np.zeros(s, dtype=dt_) for s in shapes]
    ptrs = (C.c_void_p * 24)(*[p.ctypes.data for p in profiles])
    rc = lib.fdp_prep_pml(prec, mx, mz, tpml, cfg.ktbo, pp(cfg.r), pp(cfg.tau), pp(cfg.pow_), pp(cfg.sf),
                          pp(cfg.wc), dt, h, jm.ctypes.data_as(C.POINTER(C.c_int32)), table.shape[0],
                          table.ctypes.data_as(C.c_void_p), ptrs)
    if rc:
        raise FdpError(rc, "fdp_prep_pml")
    return Inputs(prec, mx, mz, tpml, si, lin_x, lin_z, h, dt, jm, table, profiles, ab, sourtf,
                  np.asarray(cfg.irecx, np.int32), np.asarray(cfg.lrecx, np.int32),
                  np.asarray(cfg.irecz, np.int32), np.asarray(cfg.lrecz, np.int32), cfg.rec_flags)


def load_inputs(engine, inp: Inputs, medium_from=None) -> None:
    """Sets the module state of an engine (GPU or oracle) from prepared
    inputs; with ``medium_from`` (an engine of the same grid) the medium is
    shared with that engine instead of uploaded again."""
    if medium_from is None:
        engine.set_medium(inp.jm, inp.table)
    else:
        engine.share_medium(medium_from)
    engine.set_pml(inp.profiles)
    engine.set_bottom_nr(inp.ab)
    engine.set_source(inp.sourtf)
    engine.set_receivers(inp.irecx, inp.lrecx, inp.irecz, inp.lrecz, inp.rec_flags)


def make_engine(inp: Inputs, device: int = 0, medium_from=None):
    from .engine import Engine
    e = Engine(inp.mx, inp.mz, inp.tpml, inp.lin_x, inp.lin_z, inp.h, inp.dt,
               precision="f64" if inp.precision == FDP_F64 else "f32",
               stress_imaging=inp.stress_imaging, device=device)
    load_inputs(e, inp, medium_from)
    return e


def with_source(inp: Inputs, cfg: JobConfig, x_source: float, z_source: float) -> Inputs:
    """The same prepared job with the source moved: LIN_X and LIN_Z as
    READ_OPEN computes them for the new position; the medium, PML profiles,
    bottom coefficients, source time function and receivers stay (none of
    them depends on where the source is)."""
    c = dataclasses.replace(cfg, x_source=x_source, z_source=z_source)
    lin_x, lin_z = source_cell(c, inp.h)
    return dataclasses.replace(inp, lin_x=lin_x, lin_z=lin_z)


# ---------------------------------------------------------------------------
# the benchmark configurations (seeded synthetic stand-ins for the
# reference's own inputs, which its repository does not contain)

def small_homogeneous(mx: int = 300, mz: int = 300, nsteps: int = 1500, tpml: int = 20, f0: float = 60.0,
                      dt: float = 1e-4, h: float = 1.0, n_rec: int = 101, key_tlq: bool = False,
                      key_tlp: bool = True) -> tuple[JobConfig, Medium]:
    """300x300 homogeneous sandstone, 60 Hz Ricker at the centre, receivers at z = 50 m."""
    from .media import homogeneous
    t = np.arange(0, nsteps) * dt
    xr = np.linspace(0, mx, n_rec)
    ir = np.array([nint(x / h) for x in xr], np.int32)
    lr = np.full(n_rec, nint(50.0 / h) + 2, np.int32)
    cfg = JobConfig(mx=mx, mz=mz, h=h, dt=dt, mt2=nsteps, tpml=tpml, x_source=mx * h / 2, z_source=mz * h / 2,
                    stf_time=t, stf_value=ricker(t, f0), irecx=ir, lrecx=lr, irecz=ir, lrecz=lr,
                    key_tlq=key_tlq, key_tlp=key_tlp)
    return cfg, homogeneous(mx, cfg.n_model_rows)


def layered(mx: int = 2048, mz: int = 2048, nsteps: int = 4000, tpml: int = 20, f0: float = 20.0,
            dt: float = 1e-4, h: float = 1.0, n_rec: int = 512, seed: int = 20250, layer_depth: float | None = None,
            key_tlp: bool = True) -> tuple[JobConfig, Medium]:
    """Layered medium with a 10 % Gaussian random field (correlation 20 m),
    20 Hz Ricker explosive source at 10 m depth, receivers on row 2."""
    from .media import layered_grf
    t = np.arange(0, nsteps) * dt
    ir = np.linspace(1, mx, n_rec).round().astype(np.int32)
    lr = np.full(n_rec, 2, np.int32)
    cfg = JobConfig(mx=mx, mz=mz, h=h, dt=dt, mt2=nsteps, tpml=tpml, x_source=mx * h / 2, z_source=10.0,
                    stf_time=t, stf_value=ricker(t, f0), irecx=ir, lrecx=lr, irecz=ir, lrecz=lr, key_tlp=key_tlp)
    depth = layer_depth if layer_depth is not None else mz * h / 2
    return cfg, layered_grf(mx, cfg.n_model_rows, h, seed, layer_depth=depth)


def batch_shots(n_shots: int = 64, nsteps: int = 3000, seed: int = 20251, sides=(512, 2048, 32), tpml: int = 20,
                f0: float = 20.0, dt: float = 1e-4, h: float = 1.0, n_rec: int = 512) -> list[tuple[int, dict]]:
    """Per-shot parameters of the batched workload: each grid side drawn
    uniformly from {lo, lo+step, ..., hi}, the source uniformly in the upper
    quarter, the layered random medium of :func:`layered` with a per-shot
    seed.  Returns (shot seed, keyword arguments of :func:`batch_shot`)."""
    rng = np.random.default_rng(seed)
    lo, hi, step = sides
    choices = np.arange(lo, hi + 1, step)
    out = []
    for k in range(n_shots):
        mx, mz = (int(v) for v in rng.choice(choices, size=2))
        xs = float(rng.uniform(0.05, 0.95) * mx * h)
        zs = float(rng.uniform(0.01, 0.25) * mz * h)
        out.append((seed * 1000 + k, dict(mx=mx, mz=mz, nsteps=nsteps, tpml=tpml, f0=f0, dt=dt, h=h, n_rec=n_rec,
                                          x_source=xs, z_source=zs)))
    return out


def large_shots(n_shots: int = 16, mx: int = 8192, mz: int = 8192, nsteps: int = 10000, seed: int = 20252,
                tpml: int = 20, n_rec: int = 512) -> tuple[JobConfig, Medium, list[tuple[float, float]]]:
    """The large survey: one layered random medium of :func:`layered` shared
    by ``n_shots`` shots whose sources lie uniformly in the upper quarter;
    returns the first shot's configuration, the medium and every shot's
    (x_source, z_source)."""
    cfg, med = layered(mx=mx, mz=mz, nsteps=nsteps, tpml=tpml, n_rec=n_rec, seed=seed)
    rng = np.random.default_rng(seed + 1)
    pos = [(float(rng.uniform(0.05, 0.95) * mx * cfg.h), float(rng.uniform(0.01, 0.25) * mz * cfg.h))
           for _ in range(n_shots)]
    cfg.x_source, cfg.z_source = pos[0]
    return cfg, med, pos


def batch_shot(seed: int, mx: int, mz: int, nsteps: int, tpml: int, f0: float, dt: float, h: float, n_rec: int,
               x_source: float, z_source: float) -> tuple[JobConfig, Medium]:
    """One shot of :func:`batch_shots`."""
    cfg, med = layered(mx=mx, mz=mz, nsteps=nsteps, tpml=tpml, f0=f0, dt=dt, h=h, n_rec=min(n_rec, mx), seed=seed)
    cfg.x_source, cfg.z_source = x_source, z_source
    return cfg, med
