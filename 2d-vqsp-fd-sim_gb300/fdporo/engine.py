"""Python host mirror of the time-stepping interface.

:class:`Engine` wraps one ``fdp_ctx`` (one shot resident on one GPU).  Its
methods follow the reference's seam: the module state that TIME_LOOP reads
(medium, PML profiles, bottom coefficients, source, receivers) is set once,
then :meth:`time_loop` advances levels ``it_begin..it_end`` as
``DO ITILE = MT1, MT2`` does (time_loop.F90:65).

Array convention: every 2-D array is a C-ordered numpy array of shape
``(nz, nx)`` -- x fastest, i.e. exactly the reference's column-major layout
of ``A(lx:ux, lz:uz)`` -- with the Fortran bounds available from
:meth:`bounds`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .native import FIELD_ID, FDP_F32, FDP_F64, FdpError


def _dtype(precision: int):
    return np.float64 if precision == FDP_F64 else np.float32


def _ptr(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Engine:
    """One shot of the GB300 engine.  ``precision`` is ``"f32"`` or ``"f64"``."""

    def __init__(self, mx: int, mz: int, tpml: int, lin_x: int, lin_z: int, h: float, dt: float,
                 precision: str = "f32", stress_imaging: bool = True, tau_eps: float = 0.0, device: int = 0):
        self.lib = native.load()
        self.precision = FDP_F64 if precision in ("f64", "double", 8) else FDP_F32
        self.dtype = _dtype(self.precision)
        self.mx, self.mz, self.tpml = mx, mz, tpml
        self.pmll, self.pmlxh, self.pmlzh = 1 - tpml, mx + tpml, mz + tpml
        self.nx, self.nz = mx + 2 * tpml, mz + tpml + 1
        g = native.fdp_grid(mx=mx, mz=mz, tpml=tpml, stress_imaging=int(bool(stress_imaging)), lin_x=lin_x,
                            lin_z=lin_z, precision=self.precision, device=device, h=h, dt=dt, tau_eps=tau_eps)
        self._ctx = C.c_void_p()
        rc = self.lib.fdp_create(C.byref(g), C.byref(self._ctx))
        if rc != 0:
            raise FdpError(rc, self.lib.fdp_last_error(None).decode())
        self.mr = 0
        self.mt2 = 0

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if self._ctx:
            self.lib.fdp_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise FdpError(rc, self.lib.fdp_last_error(self._ctx).decode())

    def _real(self, a) -> np.ndarray:
        return np.ascontiguousarray(a, dtype=self.dtype)

    # -- module state -------------------------------------------------------
    def set_medium(self, jm: np.ndarray, table24: np.ndarray) -> None:
        """JM (nz, nx) int32 and the scaled material table (jmnum, 24)."""
        jm = np.ascontiguousarray(jm, dtype=np.int32)
        tab = self._real(table24)
        assert jm.shape == (self.nz, self.nx), (jm.shape, (self.nz, self.nx))
        assert tab.ndim == 2 and tab.shape[1] == 24
        self._check(self.lib.fdp_set_medium(self._ctx, _iptr(jm), self.nx, self.nz, tab.shape[0], _ptr(tab)))

    def share_medium(self, other: "Engine") -> None:
        """Uses ``other``'s device medium instead of a copy of its own
        (``fdp_share_medium``): same grid, precision and device."""
        self._check(self.lib.fdp_share_medium(self._ctx, other._ctx))

    def set_pml(self, profiles: list[np.ndarray]) -> None:
        arrs = [self._real(p) for p in profiles]
        assert len(arrs) == 24
        ptrs = (C.c_void_p * 24)(*[a.ctypes.data for a in arrs])
        self._check(self.lib.fdp_set_pml(self._ctx, ptrs))

    def set_pml_arrays(self, profiles: list[np.ndarray]) -> None:
        """The 24 profiles as separate arguments (fdp_set_pml_arrays, the
        form the Fortran binding uses)."""
        arrs = [self._real(p) for p in profiles]
        assert len(arrs) == 24
        self._check(self.lib.fdp_set_pml_arrays(self._ctx, *[C.c_void_p(a.ctypes.data) for a in arrs]))

    def set_bottom_nr(self, ab16: np.ndarray) -> None:
        ab = self._real(ab16).reshape(16)
        self._check(self.lib.fdp_set_bottom_nr(self._ctx, _ptr(ab)))

    def set_source(self, sourtf: np.ndarray) -> None:
        """SOURTF_A as an (mt2, 2) array (row it-1 = solid, fluid)."""
        s = self._real(sourtf).reshape(-1, 2)
        self.mt2 = s.shape[0]
        self._check(self.lib.fdp_set_source(self._ctx, _ptr(s), self.mt2))

    def set_receivers(self, irecx, lrecx, irecz, lrecz, flags: int) -> None:
        a = [np.ascontiguousarray(v, dtype=np.int32) for v in (irecx, lrecx, irecz, lrecz)]
        self.mr = len(a[0])
        self._check(self.lib.fdp_set_receivers(self._ctx, *[_iptr(v) for v in a], self.mr, flags))

    # -- time stepping --------------------------------------------------------
    def time_loop(self, it_begin: int, it_end: int) -> None:
        self._check(self.lib.fdp_run(self._ctx, it_begin, it_end))

    def prepare_run(self, n_levels: int) -> None:
        """Captures the graphs a run of ``n_levels`` levels replays (fdp_prepare_run)."""
        self._check(self.lib.fdp_prepare_run(self._ctx, n_levels))

    def synchronize(self) -> None:
        self._check(self.lib.fdp_synchronize(self._ctx))

    def receivers(self, it_first: int, n_levels: int) -> np.ndarray:
        """(n_levels, MR, 10) values in STORE_SEISMOGRAMS column order."""
        # fdp_get_receivers writes every value (zeros where a flag is off)
        out = np.empty((n_levels, self.mr, native.FDP_REC_VALUES), dtype=self.dtype)
        self._check(self.lib.fdp_get_receivers(self._ctx, it_first, n_levels, _ptr(out)))
        return out

    def kernel_launches(self) -> int:
        return int(self.lib.fdp_kernel_launches(self._ctx))

    def stream(self) -> int:
        """The engine's cudaStream_t as an integer handle."""
        s = C.c_void_p()
        self._check(self.lib.fdp_get_stream(self._ctx, C.byref(s)))
        return int(s.value or 0)

    def medium_info(self) -> dict:
        """Device representation of the medium: mode ("table", "planes", or
        "biot" -- planes whose aliases follow Biot's relations) and the
        per-cell coefficient planes each phase reads."""
        v = [C.c_int32() for _ in range(3)]
        self._check(self.lib.fdp_medium_info(self._ctx, *[C.byref(x) for x in v]))
        return {"mode": {0: "table", 1: "planes", 2: "biot"}[v[0].value], "planes_stress": v[1].value,
                "planes_velocity": v[2].value}

    def core_info(self) -> dict:
        """Core rectangles {phase: (x0, x1, z0, z1)} of the frame/core split
        (all zero when another kernel variant runs)."""
        r = np.zeros(8, np.int32)
        self._check(self.lib.fdp_core_info(self._ctx, _iptr(r)))
        return {"stress": tuple(int(v) for v in r[:4]), "velocity": tuple(int(v) for v in r[4:])}

    def march_info(self) -> dict | None:
        """Region and launch shape of the march kernel (fdp_march_info), or
        None when the levels do not run as march levels."""
        r, sh = np.zeros(8, np.int32), np.zeros(4, np.int32)
        self._check(self.lib.fdp_march_info(self._ctx, _iptr(r), _iptr(sh)))
        if not sh[0]:
            return None
        return {"region": tuple(int(v) for v in r[:4]), "stress_writes": tuple(int(v) for v in r[4:]),
                "strips": int(sh[0]), "band_rows": int(sh[1]), "ctas": int(sh[2]), "warps": int(sh[3])}

    def profile(self, it_begin: int, it_end: int) -> dict:
        """Device time (ms) and launch counts over levels it_begin..it_end of
        each phase (frame and core together), of the row-1/receiver kernel,
        and of each phase's core kernel alone."""
        ms = (C.c_double * 5)()
        n = (C.c_int64 * 5)()
        self._check(self.lib.fdp_profile_run(self._ctx, it_begin, it_end, ms, n))
        return {k: (ms[i], n[i]) for i, k in enumerate(("stress", "velocity", "edge", "stress_core",
                                                            "velocity_core"))}

    # -- state ----------------------------------------------------------------
    def bounds(self, name: str) -> tuple[int, int, int, int]:
        b = np.zeros(4, dtype=np.int32)
        self._check(self.lib.fdp_field_bounds(self._ctx, FIELD_ID[name], _iptr(b)))
        return tuple(int(v) for v in b)

    def field(self, name: str) -> np.ndarray:
        lx, ux, lz, uz = self.bounds(name)
        out = np.zeros((uz - lz + 1, ux - lx + 1), dtype=self.dtype)
        self._check(self.lib.fdp_get_field(self._ctx, FIELD_ID[name], _ptr(out)))
        return out

    def set_field(self, name: str, values: np.ndarray) -> None:
        lx, ux, lz, uz = self.bounds(name)
        v = self._real(values)
        assert v.shape == (uz - lz + 1, ux - lx + 1), (name, v.shape)
        self._check(self.lib.fdp_set_field(self._ctx, FIELD_ID[name], _ptr(v)))

    def snapshot(self, mask: int = 3) -> np.ndarray:
        n = bin(mask & 15).count("1")
        out = np.zeros((n, self.nz, self.nx), dtype=self.dtype)
        self._check(self.lib.fdp_get_snapshot(self._ctx, mask, _ptr(out)))
        return out


class Batch:
    """Many prepared :class:`Engine` shots advanced together (``fdp_batch``).

    The engines stay usable for reading results (:meth:`Engine.receivers`,
    :meth:`Engine.field`, ...) after :meth:`synchronize`; while the batch
    exists they are advanced only through it.  Every shot's values are
    bit-identical to running it alone."""

    def __init__(self, engines: list[Engine]):
        if not engines:
            raise ValueError("a batch needs at least one shot")
        self.lib = native.load()
        self.engines = list(engines)
        arr = (C.c_void_p * len(engines))(*[e._ctx.value for e in engines])
        self._b = C.c_void_p()
        rc = self.lib.fdp_batch_create(arr, len(engines), C.byref(self._b))
        if rc != 0:
            raise FdpError(rc, self.lib.fdp_batch_last_error(None).decode())

    def close(self) -> None:
        if self._b:
            self.lib.fdp_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise FdpError(rc, self.lib.fdp_batch_last_error(self._b).decode())

    def time_loop(self, it_begin: int, it_end: int) -> None:
        """Advances every shot over levels it_begin..it_end (asynchronous)."""
        self._check(self.lib.fdp_batch_run(self._b, it_begin, it_end))

    def synchronize(self) -> None:
        self._check(self.lib.fdp_batch_synchronize(self._b))

    def set_shape(self, units_per_item: int, waves: int) -> None:
        """Fixes the tile shape (``units_per_item = 0``: tune on the next run;
        ``native.FDP_BATCH_SHOTS``: every shot's own kernels side by side)."""
        self._check(self.lib.fdp_batch_set_shape(self._b, units_per_item, waves))

    def shape(self) -> tuple[int, int]:
        m, w = C.c_int32(), C.c_int32()
        self._check(self.lib.fdp_batch_get_shape(self._b, C.byref(m), C.byref(w)))
        return m.value, w.value

    def kernel_launches(self) -> int:
        return int(self.lib.fdp_batch_kernel_launches(self._b))

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.fdp_batch_get_stream(self._b, C.byref(s)))
        return int(s.value or 0)
