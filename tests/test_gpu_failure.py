"""The failure path of the bounded device waits, without faulting the GPU.

Every wait in the engine's kernels (the TMA-staged variants wait for their
tile copies on an mbarrier) has an iteration limit; a wait that runs out
records itself in the context's status word, the host reports
FDP_ERR_DEVICE at its next synchronisation, and the context stays usable.
fdp_diag_wait_timeout makes such a wait run out on purpose: a kernel polls,
a bounded number of times, a word nothing sets.
"""
import numpy as np
import pytest

from helpers import compare_state, small_job

pytestmark = pytest.mark.gpu


def test_expired_wait_is_reported_once_and_the_context_stays_usable():
    from fdporo import job
    from fdporo.native import FDP_ERR_DEVICE, FdpError
    from oracle.oracle import make_oracle
    cfg, med = small_job(mx=40, mz=30, tpml=6, nsteps=40, seed=91)
    inp = job.prepare(cfg, med, "f32")
    eng, orc = job.make_engine(inp), make_oracle(inp)
    eng.time_loop(1, 5)
    assert eng.lib.fdp_diag_wait_timeout(eng._ctx, 2000) == 0
    with pytest.raises(FdpError) as ex:
        eng.synchronize()
    assert ex.value.code == FDP_ERR_DEVICE
    eng.synchronize()  # reported once
    eng.time_loop(6, 40)
    orc.time_loop(1, 40)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 40), orc.receivers(1, 40))
