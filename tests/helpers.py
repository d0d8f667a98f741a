"""Shared builders for the parity tests: prepared inputs, random states, and
comparisons between the CUDA engine and the CPU oracle."""
from __future__ import annotations

import numpy as np

from fdporo import job, media
from fdporo.native import HISTORY, MEMORY_VARS, WAVEFIELD


def random_medium(cfg: job.JobConfig, n_mat: int, seed: int) -> media.Medium:
    """``n_mat`` random Biot materials scattered over the grid."""
    rng = np.random.default_rng(seed)
    base = media.SANDSTONE
    fac = lambda: 1.0 + 0.3 * (rng.random(n_mat) - 0.5)
    tab = media.biot_table(base.rho_s * fac(), base.rho_f * fac(), base.phi * fac(), base.k_s * fac(),
                           base.k_f * fac(), base.k_frame * fac(), base.mu * fac(),
                           base.kappa * 10 ** (2 * (rng.random(n_mat) - 0.5)), base.eta * fac(), 2.0 * fac())
    rows = rng.integers(1, n_mat + 1, size=(cfg.n_model_rows, cfg.mx)).astype(np.int32)
    return media.Medium(rows, tab)


def small_job(mx=40, mz=30, tpml=6, nsteps=80, si=True, f0=400.0, n_rec=7, seed=1, per_cell=False,
              key_tlq=True, key_tlp=True, ktbo=0, wc=0.0):
    dt, h = 1e-4, 1.0
    t = np.arange(nsteps) * dt
    rng = np.random.default_rng(seed)
    ir = rng.integers(-tpml + 1, mx + tpml, n_rec).astype(np.int32)
    lr = rng.integers(0, mz + tpml + (3 if si else 1), n_rec).astype(np.int32)
    iz = rng.integers(-tpml + 1, mx + tpml, n_rec).astype(np.int32)
    lz = rng.integers(0, mz + tpml + (3 if si else 1), n_rec).astype(np.int32)
    ir[0], lr[0] = mx // 2, 3  # one receiver on the free-surface rows
    iz[0], lz[0] = mx // 2 + 1, 1
    cfg = job.JobConfig(mx=mx, mz=mz, h=h, dt=dt, mt2=nsteps, tpml=tpml, stress_imaging=si,
                        x_source=mx * h / 2 + 0.3, z_source=mz * h / 3, stf_time=t,
                        stf_value=job.ricker(t, f0), irecx=ir, lrecx=lr, irecz=iz, lrecz=lz,
                        key_tlq=key_tlq, key_tlp=key_tlp, ktbo=ktbo, wc=wc)
    if per_cell:
        med = media.layered_grf(mx, cfg.n_model_rows, h, seed, layer_depth=mz * h / 2, corr_len=4.0)
    else:
        med = random_medium(cfg, 5, seed)
    return cfg, med


def randomize_state(engines, inp, seed: int, scale: float = 1e-3):
    """Writes the same random wavefield, memory variables and bottom history
    into every engine.  For the oracle the old-q copies QXP/QZP are set to the
    q fields, the invariant the reference keeps between levels."""
    rng = np.random.default_rng(seed)
    vals = {}
    for name in WAVEFIELD + MEMORY_VARS + HISTORY:
        lx, ux, lz, uz = engines[0].bounds(name)
        vals[name] = (scale * rng.standard_normal((uz - lz + 1, ux - lx + 1))).astype(engines[0].dtype)
    for e in engines:
        for n, v in vals.items():
            e.set_field(n, v)
        if hasattr(e, "lib") and e.__class__.__name__ == "Oracle":
            e.set_field("QXP", vals["QX"])
            e.set_field("QZP", vals["QZ"])
    return vals


def compare_state(a, b, names=None, exact=True, rtol=0.0):
    """Returns a dict name -> max abs difference; asserts equality (bitwise
    when ``exact``) on every field."""
    names = names or (WAVEFIELD + MEMORY_VARS + HISTORY)
    out = {}
    for n in names:
        x, y = a.field(n), b.field(n)
        d = float(np.max(np.abs(x.astype(np.float64) - y.astype(np.float64)))) if x.size else 0.0
        out[n] = d
        if exact:
            assert np.array_equal(x, y), f"{n}: max |diff| = {d}"
        else:
            scale = float(np.max(np.abs(y))) or 1.0
            assert d <= rtol * scale, f"{n}: max |diff| = {d} vs scale {scale}"
    return out
