"""Batched shots (fdp_batch_*) against the CPU oracle, shot by shot.

Shots of different grid sizes, PML widths, media, sources and receivers are
advanced together; every shot's wavefield, memory variables, bottom history
and receiver values must equal the oracle's bit for bit, whatever the tile
shape of the work queue, including the shape the batch tunes for itself on
the run's own levels.
"""
import numpy as np
import pytest

from helpers import compare_state, randomize_state, small_job

pytestmark = pytest.mark.gpu

# (mx, mz, tpml, seed): uneven sizes, including grids wide enough for the
# interior fast paths and one narrower than a warp's 32 columns
SHOTS = [(40, 30, 6, 61), (160, 100, 8, 62), (72, 56, 4, 63), (24, 20, 3, 64)]


def _shots(prec, si, per_cell, nsteps):
    from fdporo import job
    from oracle.oracle import make_oracle
    engs, orcs = [], []
    for k, (mx, mz, tpml, seed) in enumerate(SHOTS):
        cfg, med = small_job(mx=mx, mz=mz, tpml=tpml, nsteps=nsteps, si=si, per_cell=per_cell, seed=seed,
                             n_rec=3 + k)
        inp = job.prepare(cfg, med, prec)
        engs.append(job.make_engine(inp))
        orcs.append(make_oracle(inp))
        randomize_state([engs[-1], orcs[-1]], inp, seed=seed + 100)
    return engs, orcs


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
@pytest.mark.parametrize("shape", [(1, 0), (2, 1), (4, 2), (3, 1), (-1, 0)])
def test_batch_matches_oracle(prec, si, shape):
    from fdporo.engine import Batch
    engs, orcs = _shots(prec, si, per_cell=True, nsteps=40)
    with Batch(engs) as b:
        b.set_shape(*shape)
        b.time_loop(1, 5)
        b.time_loop(6, 40)  # one graph replay of 32 levels plus direct levels
        b.synchronize()
        assert b.shape() == shape
    for e, o in zip(engs, orcs):
        o.time_loop(1, 40)
        compare_state(e, o)
        np.testing.assert_array_equal(e.receivers(1, 40), o.receivers(1, 40))


@pytest.mark.parametrize("per_cell", [True, False])
def test_batch_tuned_shape(per_cell):
    from fdporo.engine import Batch
    engs, orcs = _shots("f32", True, per_cell=per_cell, nsteps=70)
    with Batch(engs) as b:
        # the first 18 levels time the 9 queue shapes, the next 32 the
        # shots mode (every shot's own kernels side by side)
        b.time_loop(1, 70)
        b.synchronize()
        m, w = b.shape()
        assert (m in (1, 2, 4) and w in (0, 1, 2)) or (m, w) == (-1, 0)
        assert b.kernel_launches() >= 3 * 70
    for e, o in zip(engs, orcs):
        o.time_loop(1, 70)
        compare_state(e, o)
        np.testing.assert_array_equal(e.receivers(1, 70), o.receivers(1, 70))


def test_batch_equals_single_runs():
    from fdporo import job
    from fdporo.engine import Batch
    runs = []
    for _ in range(2):
        engs = []
        for mx, mz, tpml, seed in SHOTS:
            cfg, med = small_job(mx=mx, mz=mz, tpml=tpml, nsteps=36, per_cell=True, seed=seed)
            engs.append(job.make_engine(job.prepare(cfg, med, "f32")))
        runs.append(engs)
    with Batch(runs[0]) as b:
        b.set_shape(2, 1)
        b.time_loop(1, 36)
        b.synchronize()
    for e in runs[1]:
        e.time_loop(1, 36)
    for a, c in zip(*runs):
        compare_state(a, c)
        np.testing.assert_array_equal(a.receivers(1, 36), c.receivers(1, 36))


def test_batch_mixed_groups():
    """Shots with different free-surface modes and medium representations
    (table, per-cell Biot planes) in one batch: one launch per group."""
    from fdporo import job
    from fdporo.engine import Batch
    from oracle.oracle import make_oracle
    engs, orcs = [], []
    # per-cell media of more than 4096 cells are held as Biot planes, the
    # others through the material table
    cases = [(True, True, 160, 100, 8), (False, False, 40, 30, 6), (True, False, 72, 56, 4), (False, True, 120, 60, 5)]
    for k, (si, per_cell, mx, mz, tpml) in enumerate(cases):
        cfg, med = small_job(mx=mx, mz=mz, tpml=tpml, nsteps=40, si=si, per_cell=per_cell, seed=80 + k)
        inp = job.prepare(cfg, med, "f64")
        engs.append(job.make_engine(inp))
        orcs.append(make_oracle(inp))
    assert {e.medium_info()["mode"] for e in engs} == {"table", "biot"}
    with Batch(engs) as b:
        b.set_shape(2, 1)
        b.time_loop(1, 40)
        b.synchronize()
        assert b.kernel_launches() >= 4 * 3 * 40 // 2
    for e, o in zip(engs, orcs):
        o.time_loop(1, 40)
        compare_state(e, o)
        np.testing.assert_array_equal(e.receivers(1, 40), o.receivers(1, 40))


def test_batch_rejects_bad_shots():
    from fdporo import job
    from fdporo.engine import Batch
    from fdporo.native import FdpError
    cfg, med = small_job(per_cell=True, seed=71)
    a = job.make_engine(job.prepare(cfg, med, "f32"))
    b = job.make_engine(job.prepare(cfg, med, "f64"))
    with pytest.raises(FdpError) as err:
        Batch([a, b])
    assert err.value.code == -5
    with pytest.raises(FdpError) as err:
        Batch([a, a])
    assert err.value.code == -1


def test_shots_mode_march_levels_between_queue_levels(monkeypatch):
    """In the shots mode a shot with march levels runs them in pairs and an
    odd last level in place, so the work-queue kernels, which update the
    buffers they were given in place, can take over between runs: shots
    mode and queue runs of odd and even lengths, then levels alone, equal
    the oracle bit for bit."""
    from fdporo.engine import Batch
    monkeypatch.setenv("FDP_KERNEL_VARIANT", "march")
    engs, orcs = _shots("f32", True, per_cell=True, nsteps=80)
    assert engs[1].march_info() is not None
    with Batch(engs) as b:
        lo = 1
        for shape, n in (((-1, 0), 7), ((2, 1), 5), ((-1, 0), 33), ((1, 0), 2), ((-1, 0), 4)):
            b.set_shape(*shape)
            b.time_loop(lo, lo + n - 1)
            lo += n
        b.synchronize()
    for e in engs:
        e.time_loop(lo, 61)
    for e, o in zip(engs, orcs):
        o.time_loop(1, 61)
        compare_state(e, o)
        np.testing.assert_array_equal(e.receivers(1, 61), o.receivers(1, 61))


def test_march_shots_in_and_out_of_a_batch(monkeypatch):
    """Contexts made with the march variant alternate between two buffers of
    each field when run alone; a batch holding them updates them in place.
    Levels run alone (an odd number, so the current buffers are the second
    ones), then in a batch, then alone again equal the oracle bit for bit."""
    from fdporo.engine import Batch
    monkeypatch.setenv("FDP_KERNEL_VARIANT", "march")
    engs, orcs = _shots("f32", True, per_cell=True, nsteps=60)
    assert engs[1].march_info() is not None
    for e in engs:
        e.time_loop(1, 7)
    with Batch(engs) as b:
        assert engs[1].march_info() is None  # the batch holds it: in-place levels
        b.set_shape(-1, 0)
        b.time_loop(8, 45)
        b.synchronize()
    assert engs[1].march_info() is not None
    for e in engs:
        e.time_loop(46, 60)
    for e, o in zip(engs, orcs):
        o.time_loop(1, 60)
        compare_state(e, o)
        np.testing.assert_array_equal(e.receivers(1, 60), o.receivers(1, 60))
