"""Known-answer tests (tests/kat.py) run on the engine through the C ABI.

The engine matches the oracle bit for bit elsewhere; these checks hold the
engine itself to properties the reference's scheme must have, at a larger
size than the oracle tests use: exact-to-rounding mirror symmetry of an
explosive source on a wide grid in both precisions and both free-surface
modes, and the shear and slow P plane-wave speeds of CALCUL_VELOCITY.
"""
import pytest

import kat

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 1e-4)])
@pytest.mark.parametrize("si", [True, False])
def test_engine_explosive_source_is_mirror_symmetric(prec, tol, si):
    from fdporo import job
    inp = kat.mirror_inputs(si, prec=prec, mx=511, mz=300, tpml=20, nsteps=600)
    eng = job.make_engine(inp)
    for k in range(0, 600, 200):
        eng.time_loop(k + 1, k + 200)
        defect = kat.mirror_defect(eng, inp)
        assert max(defect.values()) < tol, (k + 200, defect)


@pytest.mark.parametrize("field,which", [("UM", "vs"), ("PRES", "vps")])
def test_engine_plane_wave_speeds(field, which):
    from fdporo import job
    inp = kat.plane_wave_inputs()
    v = kat.calcul_velocity(inp)
    speed = kat.plane_wave_speed(job.make_engine(inp), inp, field, v[which])
    assert abs(speed / v[which] - 1) < 3e-3, (speed, v[which])
