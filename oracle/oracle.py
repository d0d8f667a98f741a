"""TEST INFRASTRUCTURE ONLY -- Python handle on the CPU oracle.

Builds and loads ``fdp_oracle.cpp`` (the C++ restatement of the reference's
time loop) and exposes it through the same methods as
``fdporo.engine.Engine`` so a test can drive the oracle and the CUDA engine
with identical calls.  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg use this module; the product never does.

PARITY UNPINNED: the reference has no tests or golden vectors and cannot be
compiled here (no Fortran compiler); see the header of fdp_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
SRC = ORACLE_DIR / "fdp_oracle.cpp"
BUILD_DIR = ORACLE_DIR / "_build"
LIB_CHECKED = BUILD_DIR / "liboracle_fdp.so"      # bounds-checked, single thread
LIB_OMP = BUILD_DIR / "liboracle_fdp_omp.so"      # unchecked, OpenMP over rows
# bounds-checked, with a deliberate x-index slip in the u update: only the
# test showing that the known-answer tests catch such a slip loads it
LIB_PLANTED = BUILD_DIR / "liboracle_fdp_planted.so"

FIELD_NAMES = [
    "UM", "WM", "QX", "QZ", "TXX", "TZZ", "TXZ", "PRES",
    "PZXL", "PZXH", "PXXL", "PXXH", "OXXL", "OXXH", "PXZH", "PZZH", "OZZH",
    "RXXL", "RXXH", "SXXL", "SXXH", "RZXL", "RZXH", "GXXL", "GXXH", "HXXL", "HXXH",
    "GZXL", "GZXH", "RXZH", "GXZH", "RZZH", "SZZH", "GZZH", "HZZH",
    "SZ_U", "SZ_W", "SZ_QX", "SZ_QZ", "QXP", "QZP",
]
FIELD_ID = {n: i for i, n in enumerate(FIELD_NAMES)}

_FLAGS = ["-std=c++17", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force: bool = False, planted: bool = False) -> None:
    """Compiles both oracle libraries (and, with ``planted``, the variant
    with a planted index slip) if missing or older than the source."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    jobs = [(LIB_CHECKED, ["-O2", "-DORACLE_CHECK"]), (LIB_OMP, ["-O3", "-fopenmp"])]
    if planted:
        jobs.append((LIB_PLANTED, ["-O2", "-DORACLE_CHECK", "-DORACLE_PLANT_X_SLIP"]))
    procs = []
    for lib, extra in jobs:
        if force or not lib.exists() or lib.stat().st_mtime < SRC.stat().st_mtime:
            tmp = lib.with_suffix(f".tmp{os.getpid()}")
            cmd = ["g++", *extra, *_FLAGS, "-o", str(tmp), str(SRC)]
            procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True),
                          tmp, lib, cmd))
    for p, tmp, lib, cmd in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{out}")
        os.replace(tmp, lib)


_libs: dict[str, C.CDLL] = {}


def _load(which: str = "checked") -> C.CDLL:
    if which in _libs:
        return _libs[which]
    build(planted=which == "planted")
    lib = C.CDLL(str({"checked": LIB_CHECKED, "omp": LIB_OMP, "planted": LIB_PLANTED}[which]))
    vp, i32, d = C.c_void_p, C.c_int32, C.c_double
    pi32 = C.POINTER(C.c_int32)
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, d, d, d, C.c_int, C.c_int]
    lib.orc_destroy.argtypes = [vp]
    lib.orc_error.restype = C.c_char_p
    lib.orc_error.argtypes = [vp]
    lib.orc_set_threads.argtypes = [vp, C.c_int]
    lib.orc_set_medium.argtypes = [vp, pi32, C.c_int, vp]
    lib.orc_set_profiles.argtypes = [vp, C.POINTER(vp)]
    lib.orc_set_bottom_nr.argtypes = [vp, vp]
    lib.orc_set_source.argtypes = [vp, vp, C.c_int]
    lib.orc_set_receivers.argtypes = [vp, pi32, pi32, pi32, pi32, C.c_int, C.c_int]
    lib.orc_run.argtypes = [vp, C.c_int, C.c_int, vp]
    lib.orc_field_bounds.argtypes = [vp, C.c_int, pi32]
    lib.orc_field.argtypes = [vp, C.c_int, vp, C.c_int]
    lib.orc_run_ascii.restype = C.c_longlong
    lib.orc_run_ascii.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int]
    for fn in ("orc_set_medium", "orc_set_profiles", "orc_set_bottom_nr", "orc_set_source", "orc_set_receivers",
               "orc_run", "orc_field_bounds", "orc_field", "orc_set_threads"):
        getattr(lib, fn).restype = C.c_int
    _libs[which] = lib
    return lib


class Oracle:
    """CPU restatement with the interface of ``fdporo.engine.Engine``."""

    def __init__(self, mx, mz, tpml, lin_x, lin_z, h, dt, precision="f32", stress_imaging=True, tau_eps=0.0,
                 threads: int = 0, planted: bool = False):
        which = "planted" if planted else ("omp" if threads else "checked")
        self.lib = _load(which)
        self.prec = 8 if precision in ("f64", 8) else 4
        self.dtype = np.float64 if self.prec == 8 else np.float32
        self.mx, self.mz, self.tpml = mx, mz, tpml
        self.nx, self.nz = mx + 2 * tpml, mz + tpml + 1
        self.h = self.dtype(h)
        self.dt = self.dtype(dt)
        self._h = self.lib.orc_create(self.prec, mx, mz, tpml, int(bool(stress_imaging)), float(self.h),
                                      float(self.dt), float(tau_eps), lin_x, lin_z)
        if threads:
            self.lib.orc_set_threads(self._h, int(threads))
        self.mr = 0
        self.rec_flags = 0
        self._raw: dict[int, np.ndarray] = {}

    def close(self):
        if self._h:
            self.lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.orc_error(self._h).decode())

    def _real(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def set_medium(self, jm, table24):
        jm = np.ascontiguousarray(jm, dtype=np.int32)
        tab = self._real(table24)
        self._check(self.lib.orc_set_medium(self._h, jm.ctypes.data_as(C.POINTER(C.c_int32)), tab.shape[0],
                                            tab.ctypes.data_as(C.c_void_p)))

    def set_pml(self, profiles):
        self._keep = [self._real(p) for p in profiles]
        ptrs = (C.c_void_p * 24)(*[a.ctypes.data for a in self._keep])
        self._check(self.lib.orc_set_profiles(self._h, ptrs))

    def set_bottom_nr(self, ab16):
        ab = self._real(ab16).reshape(16)
        self._check(self.lib.orc_set_bottom_nr(self._h, ab.ctypes.data_as(C.c_void_p)))

    def set_source(self, sourtf):
        s = self._real(sourtf).reshape(-1, 2)
        self.mt2 = s.shape[0]
        self._check(self.lib.orc_set_source(self._h, s.ctypes.data_as(C.c_void_p), self.mt2))

    def set_receivers(self, irecx, lrecx, irecz, lrecz, flags):
        a = [np.ascontiguousarray(v, dtype=np.int32) for v in (irecx, lrecx, irecz, lrecz)]
        self.mr = len(a[0])
        self.rec_flags = int(flags)
        self._check(self.lib.orc_set_receivers(self._h, *[v.ctypes.data_as(C.POINTER(C.c_int32)) for v in a],
                                               self.mr, int(bool(flags & 2))))

    def time_loop(self, it_begin, it_end):
        n = it_end - it_begin + 1
        if n <= 0:
            return
        rec = np.zeros((n, max(self.mr, 1), 10), dtype=self.dtype)
        self._check(self.lib.orc_run(self._h, it_begin, it_end, rec.ctypes.data_as(C.c_void_p) if self.mr else None))
        for k in range(n):
            self._raw[it_begin + k] = rec[k, : self.mr].copy()

    def time_loop_ascii(self, it_begin, it_end, directory) -> int:
        """Levels it_begin..it_end followed, each, by the reference's receiver
        output: per receiver an OPEN/WRITE/CLOSE of REC_UW_<j>.asc, REC_Q_<j>.asc
        (KEY_TLQ) and REC_STRESS_<j>.asc (KEY_TLP) in ``directory``.  Returns
        the number of files opened."""
        n = self.lib.orc_run_ascii(self._h, it_begin, it_end, str(directory).encode(), int(bool(self.rec_flags & 1)),
                                   int(bool(self.rec_flags & 2)), int(bool(self.rec_flags & 4)))
        if n < 0:
            raise RuntimeError("oracle: " + self.lib.orc_error(self._h).decode())
        return int(n)

    def synchronize(self):
        pass

    def receivers(self, it_first, n_levels):
        """Values exactly as STORE_SEISMOGRAMS(_PRESSURE) would write them;
        columns of a disabled KEY_* flag are zero, as in the ABI."""
        out = np.stack([self._raw[it_first + k] for k in range(n_levels)])
        if not self.rec_flags & 1:
            out[:, :, 0:8] = 0
        if not self.rec_flags & 4:
            out[:, :, 8:10] = 0
        return out

    def bounds(self, name):
        b = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_field_bounds(self._h, FIELD_ID[name], b.ctypes.data_as(C.POINTER(C.c_int32))))
        return tuple(int(v) for v in b)

    def field(self, name):
        lx, ux, lz, uz = self.bounds(name)
        out = np.zeros((uz - lz + 1, ux - lx + 1), dtype=self.dtype)
        self._check(self.lib.orc_field(self._h, FIELD_ID[name], out.ctypes.data_as(C.c_void_p), 0))
        return out

    def set_field(self, name, values):
        lx, ux, lz, uz = self.bounds(name)
        v = self._real(values)
        assert v.shape == (uz - lz + 1, ux - lx + 1)
        self._check(self.lib.orc_field(self._h, FIELD_ID[name], v.ctypes.data_as(C.c_void_p), 1))


def make_oracle(inp, threads: int = 0, planted: bool = False) -> Oracle:
    """An oracle loaded with the same prepared inputs as a GPU engine
    (``planted``: the variant with a deliberate index slip, for the test
    that shows the known-answer tests catch one)."""
    o = Oracle(inp.mx, inp.mz, inp.tpml, inp.lin_x, inp.lin_z, inp.h, inp.dt,
               precision="f64" if inp.precision == 8 else "f32", stress_imaging=inp.stress_imaging,
               threads=threads, planted=planted)
    o.set_medium(inp.jm, inp.table)
    o.set_pml(inp.profiles)
    o.set_bottom_nr(inp.ab)
    o.set_source(inp.sourtf)
    o.set_receivers(inp.irecx, inp.lrecx, inp.irecz, inp.lrecz, inp.rec_flags)
    return o
