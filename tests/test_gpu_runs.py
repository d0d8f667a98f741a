"""Runs of levels split at every kind of boundary.

Inside a run of levels the engine folds each level's row-1 and receiver
step into the next level's stress frame kernel (and the stress samples into
the level's velocity frame kernel), and ends every run -- a 32-level graph
replay or the graph of the levels left after the last one -- with its own
k_edge.
Splitting a shot into runs of 1, 2, 31, 32, 33 ... levels, reading the
receivers and the state between runs, must give the oracle's values bit for
bit at every split, with and without stress imaging and receivers.
"""
import numpy as np
import pytest

from helpers import compare_state, randomize_state, small_job

pytestmark = pytest.mark.gpu

# run boundaries (inclusive level ranges) of a 100-level shot
SPLITS = [(1, 1), (2, 3), (4, 34), (35, 66), (67, 67), (68, 100)]


@pytest.fixture(params=["split", "march"])
def variant(request, monkeypatch):
    """The frame/core split and the march variant, whose levels alternate
    between two buffers of each field (runs of odd length end in the other
    buffers)."""
    monkeypatch.setenv("FDP_KERNEL_VARIANT", request.param)
    return request.param


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
@pytest.mark.parametrize("n_rec", [9, 0])
def test_split_runs_match_oracle(prec, si, n_rec, variant):
    from fdporo import job
    from oracle.oracle import make_oracle
    cfg, med = small_job(mx=72, mz=56, tpml=6, nsteps=100, si=si, per_cell=True, seed=81, n_rec=max(n_rec, 1))
    if n_rec == 0:
        empty = np.zeros(0, np.int32)
        cfg.irecx = cfg.lrecx = cfg.irecz = cfg.lrecz = empty
    inp = job.prepare(cfg, med, prec)
    eng, orc = job.make_engine(inp), make_oracle(inp)
    randomize_state([eng, orc], inp, seed=82)
    for a, b in SPLITS:
        eng.time_loop(a, b)
        orc.time_loop(a, b)
        compare_state(eng, orc)
        if n_rec:
            np.testing.assert_array_equal(eng.receivers(1, b), orc.receivers(1, b))


def test_one_long_run_equals_split_runs(variant):
    from fdporo import job
    cfg, med = small_job(mx=72, mz=56, tpml=6, nsteps=100, si=True, per_cell=True, seed=83, n_rec=11)
    inp = job.prepare(cfg, med, "f32")
    whole, split = job.make_engine(inp), job.make_engine(inp)
    whole.time_loop(1, 100)
    for a, b in SPLITS:
        split.time_loop(a, b)
    compare_state(whole, split)
    np.testing.assert_array_equal(whole.receivers(1, 100), split.receivers(1, 100))


def test_prepared_graphs_give_the_same_levels(variant):
    """fdp_prepare_run captures the graphs of a run length ahead of the run;
    the prepared run, later runs of the same length (graph replays of an
    already captured graph) and the oracle agree bit for bit, and preparing
    launches nothing."""
    from fdporo import job
    from oracle.oracle import make_oracle
    cfg, med = small_job(mx=72, mz=56, tpml=6, nsteps=100, si=True, per_cell=True, seed=84, n_rec=7)
    inp = job.prepare(cfg, med, "f32")
    eng, orc = job.make_engine(inp), make_oracle(inp)
    randomize_state([eng, orc], inp, seed=85)
    n0 = eng.kernel_launches()
    eng.prepare_run(20)
    eng.prepare_run(52)
    assert eng.kernel_launches() == n0
    for a, b in ((1, 20), (21, 40), (41, 92), (93, 100)):
        eng.time_loop(a, b)
    orc.time_loop(1, 100)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 100), orc.receivers(1, 100))


def test_prepared_graphs_of_both_buffers(variant):
    """With march levels a run of odd length leaves the other buffers
    current; fdp_prepare_run captures the graphs of both, so a prepared
    length run after an odd run replays a graph captured for the other
    buffers.  Every level agrees with the oracle bit for bit."""
    from fdporo import job
    from oracle.oracle import make_oracle
    cfg, med = small_job(mx=96, mz=60, tpml=6, nsteps=90, si=False, per_cell=True, seed=86, n_rec=5)
    inp = job.prepare(cfg, med, "f32")
    eng, orc = job.make_engine(inp), make_oracle(inp)
    randomize_state([eng, orc], inp, seed=87)
    eng.prepare_run(37)
    for a, b in ((1, 3), (4, 40), (41, 41), (42, 78), (79, 90)):
        eng.time_loop(a, b)
    orc.time_loop(1, 90)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 90), orc.receivers(1, 90))
