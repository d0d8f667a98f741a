"""The reference's file formats: writing job directories and reading output.

A job directory as the reference's driver reads it (read_open.F90:-53-178,
read_model.F90, read_model_par.F90, open_sr_file.F90):
``HF_2DFD_VS_PORO`` (the job name), ``<JOB>.IN`` and ``<JOB>.INM``
(namelists), ``<JOB>.JMH`` and ``<JOB>.MO`` (gfortran unformatted sequential
records), ``STF.DAT`` and ``REC.DAT`` (list-directed text).  The record and
namelist primitives are libfdp's C++ code (include/fdp_io.h), which the
drop-in host ``fdp_host`` uses too.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import native
from .job import JobConfig
from .media import Medium

def _lib():
    return native.load()


def format_e(value: float, w: int = 13, d: int = 6) -> str:
    """Fortran Ew.d as gfortran writes it."""
    buf = C.create_string_buffer(w + 1)
    rc = _lib().fdp_io_format_e(float(value), w, d, buf)
    if rc:
        raise ValueError("bad edit descriptor")
    return buf.value.decode()


def namelist_get(text: str, group: str, name: str) -> str | None:
    buf = C.create_string_buffer(512)
    rc = _lib().fdp_io_namelist_get(text.encode(), group.encode(), name.encode(), buf, 512)
    return buf.value.decode() if rc == 0 else None


def read_record(path, index: int) -> bytes:
    lib = _lib()
    n = C.c_int64()
    if lib.fdp_io_read_record(str(path).encode(), index, None, 0, C.byref(n)) != 0:
        raise IOError(f"record {index} of {path}")
    buf = C.create_string_buffer(max(n.value, 1))
    if lib.fdp_io_read_record(str(path).encode(), index, buf, n.value, C.byref(n)) != 0:
        raise IOError(f"record {index} of {path}")
    return buf.raw[: n.value]


def append_record(path, data: bytes) -> None:
    if _lib().fdp_io_append_record(str(path).encode(), data, len(data)) != 0:
        raise IOError(f"cannot append to {path}")


def _fmt(v) -> str:
    if isinstance(v, bool):
        return ".TRUE." if v else ".FALSE."
    if isinstance(v, str):
        return "'" + v.replace("'", "''") + "'"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


def namelist(group: str, **values) -> str:
    body = ",\n".join(f"  {k.upper()} = {_fmt(v)}" for k, v in values.items())
    return f"&{group.upper()}\n{body}\n/\n"


def write_job(directory, job: str, cfg: JobConfig, medium: Medium, precision: str = "f32",
              key_snv: bool = False, ipas2: int = 1000) -> Path:
    """Writes a job directory the reference's driver (and fdp_host) can run.
    MT is chosen so that MT2 = INT(MT/DT)+1 equals cfg.mt2."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    (d / "HF_2DFD_VS_PORO").write_text(job + "\n")
    mt = (cfg.mt2 - 1 + 0.5) * cfg.dt
    text = namelist("CONTROLDATA", TPML=cfg.tpml, PROCX=1, PROCZ=1, STRESS_IMAGING=bool(cfg.stress_imaging))
    text += namelist("CONTROLDATA1", MT=mt, R=cfg.r, TAU=cfg.tau, POW=cfg.pow_, SF=cfg.sf, WC=cfg.wc,
                     TAU_EPS=0.0, IPAS2=ipas2)
    text += namelist("NAMES_SR_REC", SR_FILE_NAME="STF.DAT", REC_FILE_NAME="REC.DAT")
    text += namelist("KEYS", KEY_TLV=bool(cfg.key_tlv), KEY_SNV=bool(key_snv), KEY_TLQ=bool(cfg.key_tlq),
                     KEY_TLP=bool(cfg.key_tlp))
    text += namelist("SOURCE", X_SOURCE=cfg.x_source, Z_SOURCE=cfg.z_source, KEY_SOUR=cfg.key_sour, QR=cfg.qr)
    text += namelist("NONREF", OMG=cfg.omg, WB=cfg.wb, KTLE=0, KTRI=0, KTBO=cfg.ktbo, THPPBO=cfg.thpple,
                     THSSBO=cfg.thssle)
    text += namelist("TXT", TEXT="synthetic job")
    text += namelist("REC", MR=len(cfg.irecx))
    (d / f"{job}.IN").write_text(text)
    (d / f"{job}.INM").write_text(
        namelist("NAMES", MO_FILE_NAME=f"{job}.MO", JMH_FILE_NAME=f"{job}.JMH")
        + namelist("CONTROLDATA2", MX=cfg.mx, MZ=cfg.mz, H=cfg.h, DT_VS=cfg.dt, XBMIN=cfg.xbmin))
    real = np.float64 if precision == "f64" else np.float32
    for name in (f"{job}.JMH", f"{job}.MO"):
        (d / name).unlink(missing_ok=True)
    for row in np.asarray(medium.jm_rows, np.int32):
        append_record(d / f"{job}.JMH", row.tobytes())
    append_record(d / f"{job}.MO", np.int32(medium.jmnum).tobytes())
    append_record(d / f"{job}.MO", np.ascontiguousarray(medium.table, dtype=real).tobytes())
    (d / "STF.DAT").write_text("".join(f"{t!r} {v!r}\n" for t, v in zip(map(float, cfg.stf_time),
                                                                          map(float, cfg.stf_value))))
    (d / "REC.DAT").write_text("".join(f"R{j:04d} {a} {b} {c} {e}\n" for j, (a, b, c, e) in enumerate(
        zip(cfg.irecx, cfg.lrecx, cfg.irecz, cfg.lrecz), 1)))
    return d


def seismogram_lines(level_values: np.ndarray, dt: float, it_first: int, cols) -> list[str]:
    """Lines of one receiver's file as STORE_SEISMOGRAMS writes them:
    DT*(IT) and the selected columns, each as 1X,E13.6."""
    dtp = level_values.dtype.type
    out = []
    for k, row in enumerate(level_values):
        t = dtp(dtp(dt) * dtp(it_first + k))
        out.append("".join(" " + format_e(float(v)) for v in [t, *row[list(cols)]]))
    return out
