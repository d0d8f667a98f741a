"""Parity of the CUDA engine (through the C ABI) with the CPU oracle.

The kernels evaluate each reference expression in the reference's order
without FMA contraction, and the derived per-material coefficients are
computed on the host with the same C library as the oracle, so the bar here
is bit-for-bit equality of every wavefield array, every PML memory variable,
the bottom-row history and every receiver value, in FP32 and in FP64.
"""
import numpy as np
import pytest

from helpers import compare_state, randomize_state, small_job

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True, params=["split", "fused", "global", "tma", "coretma", "march"])
def kernel_variant(request, monkeypatch):
    """Runs every test with each kernel variant fdp_create can select through
    FDP_KERNEL_VARIANT: the frame/core split on two streams or in one
    launch per phase, the unit kernels over the whole grid, the TMA-staged
    kernels, the split with TMA-staged persistent core kernels (FP32 Biot
    media; the others keep the per-thread-load core), and the march kernel
    doing both phases of the deep interior in one pass (the default on
    grids whose levels outgrow L2; FP32, FP64 keeps the split)."""
    monkeypatch.setenv("FDP_KERNEL_VARIANT", request.param)
    return request.param


def _pair(cfg, med, prec):
    from fdporo import job
    from oracle.oracle import make_oracle
    inp = job.prepare(cfg, med, prec)
    return inp, job.make_engine(inp), make_oracle(inp)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
def test_one_step_from_random_state(prec, si):
    cfg, med = small_job(si=si, seed=3)
    inp, eng, orc = _pair(cfg, med, prec)
    randomize_state([eng, orc], inp, seed=11)
    eng.time_loop(1, 1)
    orc.time_loop(1, 1)
    compare_state(eng, orc)
    eng.time_loop(2, 6)
    orc.time_loop(2, 6)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 6), orc.receivers(1, 6))


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
def test_shot_from_rest(prec, si):
    # 80 levels: two graph replays of 32 levels plus one graph of 16 levels
    cfg, med = small_job(si=si, nsteps=80, seed=5)
    inp, eng, orc = _pair(cfg, med, prec)
    eng.time_loop(1, 80)
    orc.time_loop(1, 80)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 80), orc.receivers(1, 80))
    assert np.abs(orc.field("PRES")).max() > 0


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_resume_matches_single_run(prec):
    cfg, med = small_job(nsteps=90, seed=7)
    inp, eng, orc = _pair(cfg, med, prec)
    for a, b in ((1, 1), (2, 37), (38, 40), (41, 90)):
        eng.time_loop(a, b)
    orc.time_loop(1, 90)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 90), orc.receivers(1, 90))
    np.testing.assert_array_equal(eng.receivers(40, 51), orc.receivers(40, 51))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_per_cell_medium(prec):
    cfg, med = small_job(mx=48, mz=40, tpml=8, nsteps=40, per_cell=True, seed=9)
    inp, eng, orc = _pair(cfg, med, prec)
    assert inp.table.shape[0] == 48 * cfg.n_model_rows
    eng.time_loop(1, 40)
    orc.time_loop(1, 40)
    compare_state(eng, orc)


@pytest.mark.parametrize("ktbo", [1, 2, 3, 4, 5, 6, 7, 8, 9])
def test_bottom_conditions(ktbo):
    # KTBO != 0 zeroes the bottom damping constant; WC > 0 keeps the
    # profiles finite (with WC = 0 ppml.F90:283 divides 0 by 0)
    cfg, med = small_job(nsteps=40, seed=13, ktbo=ktbo, wc=200.0)
    cfg.omg = 60.0
    inp, eng, orc = _pair(cfg, med, "f64")
    assert np.any(inp.ab != 0)
    randomize_state([eng, orc], inp, seed=17)
    eng.time_loop(1, 40)
    orc.time_loop(1, 40)
    compare_state(eng, orc)


@pytest.mark.parametrize("tpml", [1, 2, 20])
def test_pml_widths(tpml):
    cfg, med = small_job(mx=36, mz=28, tpml=tpml, nsteps=34, seed=19)
    inp, eng, orc = _pair(cfg, med, "f32")
    randomize_state([eng, orc], inp, seed=23)
    eng.time_loop(1, 34)
    orc.time_loop(1, 34)
    compare_state(eng, orc)


def test_snapshot_matches_fields():
    cfg, med = small_job(nsteps=10, seed=29)
    inp, eng, orc = _pair(cfg, med, "f32")
    eng.time_loop(1, 10)
    snap = eng.snapshot(15)
    for k, n in enumerate(("UM", "WM", "QX", "QZ")):
        np.testing.assert_array_equal(snap[k], eng.field(n))


def test_kernel_launch_count(kernel_variant):
    """Exact launches of a 70-level run, replayed as captured runs of 32, 32
    and 6 levels, each ending with a level-counter update, after one
    level-counter reset.  The frame/core split (also with TMA-staged cores)
    launches a frame and a core kernel per phase and level, with the row-1
    and receiver step folded into the next level's stress frame kernel and
    one k_edge for the last level of each run (march levels: the march kernel
    and the two frame kernels per level); the other variants one kernel per
    phase and a k_edge per level."""
    cfg, med = small_job(mx=72, mz=56, tpml=6, nsteps=70, seed=31)
    inp, eng, _ = _pair(cfg, med, "f32")
    n0 = eng.kernel_launches()
    eng.time_loop(1, 70)
    eng.synchronize()
    runs = 3
    if kernel_variant == "march":
        # per level the march kernel and the two frame kernels
        assert eng.march_info() is not None
        expected = 70 * 3 + runs * 2 + 1
    elif kernel_variant in ("split", "coretma"):
        core = eng.core_info()
        assert all(x1 > x0 and z1 > z0 for x0, x1, z0, z1 in core.values())
        expected = 70 * 4 + runs * 2 + 1
    else:
        expected = 70 * 3 + runs + 1
    assert eng.kernel_launches() - n0 == expected
