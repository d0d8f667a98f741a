"""Shots sharing one device medium (fdp_share_medium).

A survey's shots differ only in where the source is; the medium is the same
module state for all of them.  A context that shares another's medium must
give, bit for bit, what it gives with its own copy (and what the oracle
gives), alone and batched; the shared arrays must outlive the context that
built them; a context that takes a medium of its own afterwards must leave
the others untouched; and a batch must refuse to run a shot whose device
parameters changed after the batch was made.
"""
import numpy as np
import pytest

from helpers import compare_state, small_job

pytestmark = pytest.mark.gpu


def _survey(prec, n, seed=71, mx=160, mz=100, tpml=8, nsteps=40):
    from fdporo import job
    cfg, med = small_job(mx=mx, mz=mz, tpml=tpml, nsteps=nsteps, si=True, per_cell=True, seed=seed)
    inp = job.prepare(cfg, med, prec)
    rng = np.random.default_rng(seed)
    moved = [job.with_source(inp, cfg, float(rng.uniform(0.2, 0.8) * mx * cfg.h),
                             float(rng.uniform(0.05, 0.3) * mz * cfg.h)) for _ in range(n)]
    return inp, moved


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_shared_equals_own_copy_and_oracle(prec):
    from fdporo import job
    from oracle.oracle import make_oracle
    inp, moved = _survey(prec, 2)
    owner = job.make_engine(inp)
    shared = [job.make_engine(m, medium_from=owner) for m in moved]
    own = [job.make_engine(m) for m in moved]
    assert shared[0].medium_info() == own[0].medium_info()
    for e in shared + own:
        e.time_loop(1, 40)
    for s, o, m in zip(shared, own, moved):
        compare_state(s, o)
        np.testing.assert_array_equal(s.receivers(1, 40), o.receivers(1, 40))
    orc = make_oracle(moved[0])
    orc.time_loop(1, 40)
    compare_state(shared[0], orc)
    np.testing.assert_array_equal(shared[0].receivers(1, 40), orc.receivers(1, 40))


def test_shared_medium_outlives_its_builder():
    from fdporo import job
    inp, moved = _survey("f32", 1, seed=72)
    owner = job.make_engine(inp)
    shared = job.make_engine(moved[0], medium_from=owner)
    owner.close()  # the share keeps the arrays
    ref = job.make_engine(moved[0])
    shared.time_loop(1, 40)
    ref.time_loop(1, 40)
    compare_state(shared, ref)


def test_own_medium_after_sharing_leaves_others():
    from fdporo import job
    inp, moved = _survey("f32", 1, seed=73)
    _, other = _survey("f32", 1, seed=74)
    owner = job.make_engine(inp)
    sharer = job.make_engine(moved[0], medium_from=owner)
    # the sharer takes a different medium of its own; the owner keeps the first
    sharer.set_medium(other[0].jm, other[0].table)
    owner.time_loop(1, 40)
    ref = job.make_engine(inp)
    ref.time_loop(1, 40)
    compare_state(owner, ref)


def test_batch_of_shared_shots_equals_single_runs():
    from fdporo import job
    from fdporo.engine import Batch
    inp, moved = _survey("f32", 3, seed=75)
    owner = job.make_engine(inp)
    batched = [owner] + [job.make_engine(m, medium_from=owner) for m in moved]
    alone = [job.make_engine(m) for m in [inp] + moved]
    with Batch(batched) as b:
        b.set_shape(2, 1)
        b.time_loop(1, 40)
        b.synchronize()
    for a in alone:
        a.time_loop(1, 40)
    for s, a in zip(batched, alone):
        compare_state(s, a)
        np.testing.assert_array_equal(s.receivers(1, 40), a.receivers(1, 40))


def test_batch_refuses_a_shot_changed_after_creation():
    from fdporo import job
    from fdporo.engine import Batch
    from fdporo.native import FDP_ERR_STATE, FdpError
    inp, moved = _survey("f32", 1, seed=76)
    owner = job.make_engine(inp)
    other = job.make_engine(moved[0], medium_from=owner)
    with Batch([owner, other]) as b:
        b.time_loop(1, 2)
        b.synchronize()
        other.set_source(moved[0].sourtf)  # new device parameters
        with pytest.raises(FdpError) as ex:
            b.time_loop(3, 4)
        assert ex.value.code == FDP_ERR_STATE


def test_share_needs_the_same_grid():
    from fdporo import job
    from fdporo.native import FDP_ERR_ARG, FDP_ERR_STATE, FdpError
    from fdporo.engine import Engine
    inp, _ = _survey("f32", 1, seed=77)
    cfg2, med2 = small_job(mx=120, mz=100, tpml=8, nsteps=40, si=True, per_cell=True, seed=78)
    small = job.make_engine(job.prepare(cfg2, med2, "f32"))
    owner = job.make_engine(inp)
    with pytest.raises(FdpError) as ex:
        small.share_medium(owner)
    assert ex.value.code == FDP_ERR_ARG
    bare = Engine(inp.mx, inp.mz, inp.tpml, inp.lin_x, inp.lin_z, inp.h, inp.dt, precision="f32")
    with pytest.raises(FdpError) as ex:
        owner.share_medium(bare)  # no medium to share yet
    assert ex.value.code == FDP_ERR_STATE
