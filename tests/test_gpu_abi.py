"""Entry points in the form a Fortran caller binds them.

The ISO_C_BINDING shim passes the reference's module arrays by reference
(assumed-size dummies), so the PML profiles reach the library through
fdp_set_pml_arrays, 24 separate arguments, instead of fdp_set_pml's array
of pointers.  Both must leave the engine in the same state: a shot loaded
either way runs bit-identical to the oracle.
"""
import numpy as np
import pytest

from helpers import compare_state, small_job

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_pml_arrays_entry_point_matches_the_oracle(prec):
    from fdporo import job
    from fdporo.engine import Engine
    from oracle.oracle import make_oracle
    cfg, med = small_job(mx=48, mz=40, tpml=8, nsteps=40, seed=91)
    inp = job.prepare(cfg, med, prec)
    eng = Engine(inp.mx, inp.mz, inp.tpml, inp.lin_x, inp.lin_z, inp.h, inp.dt, precision=prec,
                 stress_imaging=inp.stress_imaging)
    eng.set_medium(inp.jm, inp.table)
    eng.set_pml_arrays(inp.profiles)
    eng.set_bottom_nr(inp.ab)
    eng.set_source(inp.sourtf)
    eng.set_receivers(inp.irecx, inp.lrecx, inp.irecz, inp.lrecz, inp.rec_flags)
    orc = make_oracle(inp)
    eng.time_loop(1, 40)
    orc.time_loop(1, 40)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 40), orc.receivers(1, 40))
    assert np.abs(orc.field("PRES")).max() > 0
