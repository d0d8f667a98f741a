"""The march variant against the oracle.

By default on grids whose levels outgrow 1.5x L2 (or with
FDP_KERNEL_VARIANT=march on any grid large enough), an FP32 context runs
each level's deep interior as one kernel pass (the stress phase, then the
velocity phase, from bands of rows staged in shared memory by bulk tensor
copies), beside the frame kernels on the side stream, and the levels
alternate between two buffers of each wavefield array.  Every field, PML
memory variable, the bottom history and every receiver value must equal
the oracle's bit for bit: from random states and from rest, both
free-surface modes, grids whose width leaves a partial strip, sources
inside the march region, runs of odd length (which end in the other
buffers), any split of the rows among the CTAs, every medium
representation (Biot planes, material table, generic planes, constants)
and the full 2048^2 layered grid.
"""
import os

import numpy as np
import pytest

from helpers import compare_state, randomize_state, small_job

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def march(monkeypatch):
    monkeypatch.setenv("FDP_KERNEL_VARIANT", "march")


def _pair(cfg, med, prec="f32"):
    from fdporo import job
    from oracle.oracle import make_oracle
    inp = job.prepare(cfg, med, prec)
    return inp, job.make_engine(inp), make_oracle(inp)


@pytest.mark.parametrize("si", [True, False])
@pytest.mark.parametrize("mx,mz", [(72, 56), (160, 100), (251, 90), (300, 40)])
def test_random_state(si, mx, mz):
    cfg, med = small_job(mx=mx, mz=mz, tpml=6, nsteps=40, si=si, per_cell=True, seed=mx + mz)
    inp, eng, orc = _pair(cfg, med)
    info = eng.march_info()
    assert info is not None
    assert info["strips"] == -(-((info["region"][1] - info["region"][0]) // 4) // 30)
    randomize_state([eng, orc], inp, seed=7)
    for a, b in ((1, 1), (2, 9), (10, 40)):
        eng.time_loop(a, b)
        orc.time_loop(a, b)
        compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 40), orc.receivers(1, 40))


@pytest.mark.parametrize("si", [True, False])
def test_shot_from_rest_with_the_source_inside(si):
    cfg, med = small_job(mx=160, mz=120, tpml=8, nsteps=70, si=si, per_cell=True, seed=77, n_rec=9)
    inp, eng, orc = _pair(cfg, med)
    x0, x1, z0, z1 = eng.march_info()["region"]
    assert x0 <= inp.lin_x < x1 and z0 <= inp.lin_z < z1
    eng.time_loop(1, 70)
    orc.time_loop(1, 70)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 70), orc.receivers(1, 70))
    assert np.abs(orc.field("PRES")).max() > 0


@pytest.mark.parametrize("ctas", [1, 2, 5, 13, 152])
def test_any_split_of_the_rows_among_ctas(ctas, monkeypatch):
    monkeypatch.setenv("FDP_MARCH_CTAS", str(ctas))
    cfg, med = small_job(mx=200, mz=70, tpml=5, nsteps=12, si=True, per_cell=True, seed=90 + ctas)
    inp, eng, orc = _pair(cfg, med)
    info = eng.march_info()
    assert info["ctas"] == min(ctas, info["strips"] * (info["region"][3] - info["region"][2]))
    randomize_state([eng, orc], inp, seed=91)
    eng.time_loop(1, 12)
    orc.time_loop(1, 12)
    compare_state(eng, orc)


@pytest.mark.parametrize("sms", [1, 2, 3])
def test_whole_strips_per_cta(sms, monkeypatch):
    """With more strips than CTA slots (planned here for 1-3 SMs) every CTA
    takes the same number of whole strips, the last one the rest."""
    monkeypatch.setenv("FDP_MARCH_SMS", str(sms))
    cfg, med = small_job(mx=600, mz=60, tpml=5, nsteps=13, si=True, per_cell=True, seed=70 + sms)
    inp, eng, orc = _pair(cfg, med)
    info = eng.march_info()
    strips = info["strips"]
    assert strips == 5
    slots = sms * (2 if info["band_rows"] == 4 else 1)
    per = -(-strips // slots)
    assert info["ctas"] == -(-strips // per)
    randomize_state([eng, orc], inp, seed=71)
    eng.time_loop(1, 13)
    orc.time_loop(1, 13)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 13), orc.receivers(1, 13))


@pytest.mark.parametrize("rows", [4, 6, 8])
@pytest.mark.parametrize("ctas", [3, 152])
def test_band_rows(rows, ctas, monkeypatch):
    """Bands of four rows (two CTAs per SM), six and eight."""
    monkeypatch.setenv("FDP_MARCH_ROWS", str(rows))
    monkeypatch.setenv("FDP_MARCH_CTAS", str(ctas))
    cfg, med = small_job(mx=251, mz=97, tpml=6, nsteps=21, si=True, per_cell=True, seed=60 + rows)
    inp, eng, orc = _pair(cfg, med)
    info = eng.march_info()
    assert info["band_rows"] == rows and info["warps"] == rows
    randomize_state([eng, orc], inp, seed=61)
    eng.time_loop(1, 21)
    orc.time_loop(1, 21)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 21), orc.receivers(1, 21))


def test_launch_count():
    """Per level the stress and the velocity frame kernel and the march
    kernel; per captured run (32, 32 and 6 levels) one k_edge and one
    level-counter update; one level-counter reset per run of fdp_run."""
    cfg, med = small_job(mx=72, mz=56, tpml=6, nsteps=70, per_cell=True, seed=31)
    inp, eng, _ = _pair(cfg, med)
    assert eng.march_info() is not None
    n0 = eng.kernel_launches()
    eng.time_loop(1, 70)
    eng.synchronize()
    assert eng.kernel_launches() - n0 == 70 * 3 + 3 * 2 + 1


@pytest.mark.parametrize("variant,march", [(None, False), ("", False), ("split", False), ("march", True)])
def test_variant_choice_on_a_small_grid(variant, march, monkeypatch):
    """Without FDP_KERNEL_VARIANT an FP32 context runs march levels only
    where its levels outgrow one and a half times L2 (the 2048^2 parity
    test of test_gpu_configs.py runs them so); this small grid keeps the
    split unless march levels are named.  Every choice equals the oracle
    bit for bit."""
    if variant is None:
        monkeypatch.delenv("FDP_KERNEL_VARIANT", raising=False)
    else:
        monkeypatch.setenv("FDP_KERNEL_VARIANT", variant)
    cfg, med = small_job(mx=120, mz=64, tpml=6, nsteps=9, per_cell=True, seed=41)
    inp, eng, orc = _pair(cfg, med)
    assert (eng.march_info() is not None) == march
    randomize_state([eng, orc], inp, seed=42)
    eng.time_loop(1, 9)
    orc.time_loop(1, 9)
    compare_state(eng, orc)


def test_default_on_a_large_grid(monkeypatch):
    """A 2048^2 layered FP32 context runs march levels by default, with the
    same number of CTAs on every strip."""
    from fdporo import job
    monkeypatch.delenv("FDP_KERNEL_VARIANT", raising=False)
    cfg, med = job.layered(mx=2048, mz=2048, nsteps=10)
    eng = job.make_engine(job.prepare(cfg, med, "f32"))
    info = eng.march_info()
    assert info is not None
    assert info["ctas"] % info["strips"] == 0
    assert info["band_rows"] in (4, 8)


def test_fp64_keeps_the_split():
    cfg, med = small_job(mx=72, mz=56, tpml=6, nsteps=10, per_cell=True, seed=5)
    _, e64, _ = _pair(cfg, med, "f64")
    assert e64.march_info() is None


def _planes_medium(med):
    """The medium with an anisotropic perturbation: SIG_ZZ_1 no longer
    equals SIG_XX_2, so the engine holds it as generic coefficient planes
    rather than the ten Biot planes."""
    from fdporo import media
    t = np.array(med.table, copy=True)
    t[:, media.COL["SIG_ZZ_1"]] *= 1.0 + 0.05 * np.linspace(0.0, 1.0, t.shape[0])
    return media.Medium(med.jm_rows, t)


@pytest.mark.parametrize("kind", ["table", "planes", "homogeneous"])
@pytest.mark.parametrize("rows", [4, 8])
@pytest.mark.parametrize("si", [True, False])
def test_other_media(kind, rows, si, monkeypatch):
    """March levels for a medium held as a material table (a material index
    per cell), as generic coefficient planes, and as constants (one
    material): the coefficients come through the kernels' lookup instead of
    staged planes.  Random states and a source inside the march region,
    against the oracle bit for bit."""
    from fdporo import job, media
    monkeypatch.setenv("FDP_MARCH_ROWS", str(rows))
    cfg, med = small_job(mx=251, mz=90, tpml=6, nsteps=17, si=si, per_cell=(kind == "planes"), seed=80 + rows,
                         n_rec=7)
    if kind == "planes":
        med = _planes_medium(med)
    elif kind == "homogeneous":
        med = media.Medium(np.ones_like(np.asarray(med.jm_rows)), np.asarray(med.table)[:1])
    inp, eng, orc = _pair(cfg, med)
    want = {"table": "table", "planes": "planes", "homogeneous": "planes"}[kind]
    assert eng.medium_info()["mode"] == want
    info = eng.march_info()
    assert info is not None and info["band_rows"] == rows
    randomize_state([eng, orc], inp, seed=81)
    for a, b in ((1, 5), (6, 17)):
        eng.time_loop(a, b)
        orc.time_loop(a, b)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 17), orc.receivers(1, 17))


def test_layered_2048_full_grid():
    from fdporo import job
    from oracle.oracle import make_oracle
    cfg, med = job.layered(mx=2048, mz=2048, nsteps=101)
    inp = job.prepare(cfg, med, "f32")
    eng, orc = job.make_engine(inp), make_oracle(inp, threads=min(16, os.cpu_count() or 1))
    assert eng.march_info() is not None
    eng.time_loop(1, 101)
    orc.time_loop(1, 101)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 101), orc.receivers(1, 101))
