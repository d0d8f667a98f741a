"""The drop-in host fdp_host on a job directory in the reference's formats:
its seismogram files must equal, line for line, the engine's receiver
values written with the reference's format, and its snapshots the engine's
wavefield."""
import subprocess

import numpy as np
import pytest

from fdporo import build, formats, job

@pytest.mark.gpu
@pytest.mark.parametrize("si", [True, False])
def test_fdp_host_runs_a_job_directory(tmp_path, si):
    cfg, med = job.small_homogeneous(mx=60, mz=40, nsteps=120, tpml=8, f0=250.0, n_rec=4, key_tlq=True,
                                     key_tlp=True)
    cfg.stress_imaging = si
    med = type(med)(np.ones((cfg.n_model_rows, cfg.mx), np.int32), med.table)
    d = formats.write_job(tmp_path / "job", "JOB", cfg, med, "f32", key_snv=True, ipas2=50)
    build.build()
    r = subprocess.run([str(build.HOST_EXE), "--dir", str(d)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp = job.prepare(cfg, med, "f32")
    eng = job.make_engine(inp)
    eng.time_loop(1, 100)
    snap = np.frombuffer(formats.read_record(d / "SNAP.V000100", 0), np.float32).reshape(2, inp.nz, inp.nx)
    np.testing.assert_array_equal(snap[0], eng.field("UM"))
    np.testing.assert_array_equal(snap[1], eng.field("WM"))
    eng.time_loop(101, cfg.mt2)
    rec = eng.receivers(1, cfg.mt2)
    for j in range(len(cfg.irecx)):
        for name, cols in ((f"REC_UW_{j + 1}.asc", (0, 1, 2, 3)), (f"REC_Q_{j + 1}.asc", (4, 5, 6, 7)),
                           (f"REC_STRESS_{j + 1}.asc", (8, 9))):
            lines = (d / name).read_text().splitlines()
            assert lines == formats.seismogram_lines(rec[:, j, :], cfg.dt, 1, cols), name
    assert (d / "SNAP.Q000050").exists()


def test_fdp_host_reports_missing_input(tmp_path):
    build.build()
    (tmp_path / "HF_2DFD_VS_PORO").write_text("NOPE\n")
    r = subprocess.run([str(build.HOST_EXE), "--dir", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode != 0
    assert "NOPE.IN NOT FOUND" in r.stderr


@pytest.mark.gpu
def test_fdp_host_stops_on_a_stop_file(tmp_path):
    """time_loop.F90:79-86: a file named STOP ends the run before the next
    level and receives that level's number; nothing is written for the
    levels not run."""
    cfg, med = job.small_homogeneous(mx=40, mz=30, nsteps=60, tpml=6, f0=250.0, n_rec=3)
    med = type(med)(np.ones((cfg.n_model_rows, cfg.mx), np.int32), med.table)
    d = formats.write_job(tmp_path / "job", "JOB", cfg, med, "f32")
    (d / "STOP").write_text("")
    build.build()
    r = subprocess.run([str(build.HOST_EXE), "--dir", str(d)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (d / "STOP").read_text().split() == ["1"]
    assert not (d / "REC_UW_1.asc").exists() or (d / "REC_UW_1.asc").read_text() == ""
