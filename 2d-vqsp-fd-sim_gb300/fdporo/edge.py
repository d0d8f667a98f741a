"""Learned absorbing edge: the ctypes wrapper of include/fdp_edge.h and the
training and evaluation drivers.

A *pair* is one medium simulated twice with the same source: ``ext``, a wide
grid with the reference's 20-cell PML far from the region of interest (the
reflection-free target), and ``trunc``, the region of interest itself with
a thin PML whose strip cells the edge corrects.  Training advances both one
level at a time and lets fdp_edge_train_level fit the correction and reset
``trunc`` to the target (teacher forcing).  Evaluation runs ``trunc`` with
the edge attached, with the thin PML alone, and with the reference's PML,
against the target.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import job, media, native
from .engine import Engine, _iptr, _ptr
from .native import FdpError

SETS, SET_PARAMS, IN, OUT = 12, 10888, 96, 8


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Edge:
    """The networks of one learned edge on one GPU."""

    def __init__(self, device: int = 0, scale=None, seed: int = 0):
        self.lib = native.load()
        self._e = C.c_void_p()
        sc = None if scale is None else np.ascontiguousarray(scale, np.float32)
        rc = self.lib.fdp_edge_create(device, None if sc is None else _fptr(sc), C.c_uint64(seed), C.byref(self._e))
        if rc != 0:
            raise FdpError(rc, self.lib.fdp_edge_last_error(None).decode())

    def close(self) -> None:
        if self._e:
            self.lib.fdp_edge_destroy(self._e)
            self._e = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise FdpError(rc, self.lib.fdp_edge_last_error(self._e).decode())

    def set_output(self, kind: str) -> None:
        """"correct" (add y * scale) or "damp" (multiply by 1 - sigmoid(y - 4))."""
        self._check(self.lib.fdp_edge_set_output(self._e, {"correct": 0, "damp": 1}[kind]))

    def params(self) -> np.ndarray:
        p = np.zeros(SETS * SET_PARAMS, np.float32)
        self._check(self.lib.fdp_edge_get_params(self._e, _fptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == SETS * SET_PARAMS
        self._check(self.lib.fdp_edge_set_params(self._e, _fptr(p)))

    def scale(self) -> np.ndarray:
        s = np.zeros(8, np.float32)
        self._check(self.lib.fdp_edge_get_scale(self._e, _fptr(s)))
        return s

    def set_scale(self, s) -> None:
        s = np.ascontiguousarray(s, np.float32)
        self._check(self.lib.fdp_edge_set_scale(self._e, _fptr(s)))

    @staticmethod
    def _arrays(sets, x, t=None):
        sets = np.ascontiguousarray(sets, np.int32)
        x = np.ascontiguousarray(x, np.float32).reshape(len(sets), IN)
        t = None if t is None else np.ascontiguousarray(t, np.float32).reshape(len(sets), OUT)
        return sets, x, t

    def forward(self, sets, x) -> np.ndarray:
        sets, x, _ = self._arrays(sets, x)
        y = np.zeros((len(sets), OUT), np.float32)
        self._check(self.lib.fdp_edge_forward(self._e, len(sets), _iptr(sets), _fptr(x), _fptr(y)))
        return y

    def gradients(self, sets, x, target) -> tuple[np.ndarray, float]:
        sets, x, t = self._arrays(sets, x, target)
        g = np.zeros(SETS * SET_PARAMS, np.float32)
        loss = C.c_double()
        self._check(self.lib.fdp_edge_gradients(self._e, len(sets), _iptr(sets), _fptr(x), _fptr(t), _fptr(g),
                                                C.byref(loss)))
        return g, loss.value

    def train_batch(self, sets, x, target, lr: float) -> float:
        sets, x, t = self._arrays(sets, x, target)
        loss = C.c_double()
        self._check(self.lib.fdp_edge_train_batch(self._e, len(sets), _iptr(sets), _fptr(x), _fptr(t), C.c_float(lr),
                                                  C.byref(loss)))
        return loss.value

    def train_level(self, trunc: Engine, ext: Engine, ox: int, level: int, lr: float, teacher: bool = True,
                    want_loss: bool = False):
        loss = C.c_double()
        self._check(self.lib.fdp_edge_train_level(self._e, trunc._ctx, ext._ctx, ox, level, C.c_float(lr),
                                                  int(bool(teacher)), C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def attach(self, engine: Engine) -> None:
        self._check(self.lib.fdp_edge_attach(engine._ctx, self._e))

    def detach(self, engine: Engine) -> None:
        self._check(self.lib.fdp_edge_attach(engine._ctx, None))


# ---------------------------------------------------------------------------
# pairs of runs


def crop_medium(med: media.Medium, x0: int, nx: int, n_rows: int) -> media.Medium:
    """Columns x0 .. x0+nx-1 and the first n_rows model rows of a medium,
    with the materials renumbered."""
    rows = np.asarray(med.jm_rows)[:n_rows, x0:x0 + nx]
    used, inv = np.unique(rows, return_inverse=True)
    return media.Medium((inv.reshape(rows.shape) + 1).astype(np.int32), np.asarray(med.table)[used - 1])


@dataclass
class Pair:
    trunc: job.Inputs
    ext: job.Inputs
    ox: int
    cfg: job.JobConfig      # the region's job (thin PML)
    medium: media.Medium    # the region's medium


def plain_strip(inp: job.Inputs) -> job.Inputs:
    """The same inputs with every PML profile made transparent (ODA = ODD =
    1, ODB = ODC = 0: the strip cells take plain 2nd-order derivatives and
    the memory variables stay zero), so the strip absorbs nothing by itself."""
    from dataclasses import replace
    prof = []
    for k, p in enumerate(inp.profiles):
        which = k % 4  # A, B, C, D of each group of four (ppml.F90:60-83)
        prof.append(np.full_like(p, 1.0 if which in (0, 3) else 0.0))
    return replace(inp, profiles=prof)


def make_pair(seed: int, n: int = 512, margin: int = 256, depth_margin: int = 512, tpml_thin: int = 4,
              tpml_ext: int = 20, nsteps: int = 1500, f0: float = 20.0, n_rec: int = 101,
              source: tuple[float, float] | None = None, strip: str = "pml") -> Pair:
    """A seeded layered random medium on an (n + 2 margin) x (n + depth_margin)
    target grid with the reference PML, and its top-centre n x n region with
    a thin strip of tpml_thin cells on the sides and bottom: a PML
    (strip="pml") or transparent cells that absorb nothing by themselves
    (strip="plain"); both share the source (default: seeded, upper quarter
    of the region) and n_rec receivers on row 2 of the region."""
    rng = np.random.default_rng(seed)
    mx_e, mz_e = n + 2 * margin, n + depth_margin
    cfg_e, med_e = job.layered(mx=mx_e, mz=mz_e, nsteps=nsteps, tpml=tpml_ext, f0=f0, n_rec=n_rec, seed=seed,
                               layer_depth=0.5 * n)
    xs, zs = source if source is not None else (float(rng.uniform(0.2, 0.8) * n), float(rng.uniform(0.03, 0.25) * n))
    ir = np.linspace(1, n, n_rec).round().astype(np.int32)
    lr = np.full(n_rec, 2, np.int32)
    cfg_t = job.JobConfig(mx=n, mz=n, h=cfg_e.h, dt=cfg_e.dt, mt2=nsteps, tpml=tpml_thin, x_source=xs, z_source=zs,
                          stf_time=cfg_e.stf_time, stf_value=cfg_e.stf_value, irecx=ir, lrecx=lr, irecz=ir, lrecz=lr,
                          key_tlp=True)
    cfg_e.x_source, cfg_e.z_source = xs + margin * cfg_e.h, zs
    cfg_e.irecx = cfg_e.irecz = (ir + margin).astype(np.int32)
    cfg_e.lrecx = cfg_e.lrecz = lr
    med_t = crop_medium(med_e, margin, n, cfg_t.n_model_rows)
    trunc = job.prepare(cfg_t, med_t, "f32")
    if strip == "plain":
        trunc = plain_strip(trunc)
    return Pair(trunc, job.prepare(cfg_e, med_e, "f32"), margin, cfg_t, med_t)


def field_scales(pair: Pair, levels: int = 600, every: int = 50) -> np.ndarray:
    """RMS of each of the 8 fields over the region's strip cells of the
    target run, sampled every `every` levels (the edge's input/output
    scales)."""
    from .native import WAVEFIELD
    ext = job.make_engine(pair.ext)
    t = pair.trunc
    acc = np.zeros(8)
    cnt = 0
    for lo in range(1, levels + 1, every):
        ext.time_loop(lo, min(lo + every - 1, levels))
        for f, name in enumerate(WAVEFIELD):
            a = ext.field(name)
            x0 = pair.ox + t.pmll - ext.pmll
            x1 = pair.ox + t.pmlxh - ext.pmll
            sub = a[: t.nz, x0:x1 + 1]
            strip = np.concatenate([sub[:, :8].ravel(), sub[:, -8:].ravel(), sub[-8:, :].ravel()])
            acc[f] += float(np.mean(strip.astype(np.float64) ** 2))
        cnt += 1
    ext.close()
    s = np.sqrt(acc / max(cnt, 1))
    return np.where(s > 0, s, 1.0).astype(np.float32)


def train_pair(edge: Edge, pair: Pair, levels: int, lr: float, report_every: int = 0, free_every: int = 0,
               free_run: int = 0) -> list[float]:
    """Training over the first `levels` levels of one pair: teacher forcing,
    except that every `free_every` levels the region runs `free_run` levels
    on its own with the edge's corrections (what it meets when attached)."""
    ext, trunc = job.make_engine(pair.ext), job.make_engine(pair.trunc)
    losses = []
    for n in range(1, levels + 1):
        ext.time_loop(n, n)
        trunc.time_loop(n, n)
        want = bool(report_every) and n % report_every == 0
        free = bool(free_every) and (n % free_every) < free_run
        loss = edge.train_level(trunc, ext, pair.ox, n, lr, teacher=not free, want_loss=want)
        if want:
            losses.append(loss)
    ext.synchronize()
    trunc.synchronize()
    ext.close()
    trunc.close()
    return losses


def evaluate(pair: Pair, levels: int, edge: Edge | None = None, tpml: int | None = None, every: int = 25) -> dict:
    """Error of the region's run against the target: the error energy of u
    and w over the region's interior (columns 1..MX, rows 0..MZ) summed over
    snapshots every `every` levels, relative to the target's energy there,
    and the relative L2 error of the seismograms (u, -w, p, -txx).  `tpml`
    replaces the thin PML (the reference's PML when 20); `edge` is attached."""
    t = pair.trunc
    inp = t
    if tpml is not None and tpml != t.tpml:
        inp = _with_pml(pair, tpml)
    ext, run = job.make_engine(pair.ext), job.make_engine(inp)
    if edge is not None:
        edge.attach(run)
    err = ref = 0.0
    for lo in range(1, levels + 1, every):
        hi = min(lo + every - 1, levels)
        ext.time_loop(lo, hi)
        run.time_loop(lo, hi)
        se, sr = ext.snapshot(3), run.snapshot(3)
        x0 = pair.ox + 1 - ext.pmll
        xr = 1 - run.pmll
        mz = t.mz + 1
        a = se[:, :mz, x0:x0 + t.mx].astype(np.float64)
        b = sr[:, :mz, xr:xr + t.mx].astype(np.float64)
        err += float(np.sum((a - b) ** 2))
        ref += float(np.sum(a * a))
    cols = [0, 1, 8, 9]
    re_, rr = ext.receivers(1, levels)[:, :, cols], run.receivers(1, levels)[:, :, cols]
    seis = float(np.linalg.norm(rr.astype(np.float64) - re_) / max(np.linalg.norm(re_.astype(np.float64)), 1e-300))
    if edge is not None:
        edge.detach(run)
    ext.close()
    run.close()
    return {"reflected_energy": err / max(ref, 1e-300), "seismogram_rel_l2": seis}


def _with_pml(pair: Pair, tpml: int) -> job.Inputs:
    """The region's inputs prepared with another PML width."""
    from dataclasses import replace
    return job.prepare(replace(pair.cfg, tpml=tpml), pair.medium, "f32")
