"""Parity of the interior fast paths with the CPU oracle.

A warp takes the straight-line interior path only when its 32 columns and
all the rows its threads update lie in the 4th-order interior, so these
grids are wide enough (MX = 160) to hold several such warps per row; the
rows around the PML edges, the free surface and the source row keep the
per-cell path.  Each of the three device representations of the medium is
exercised: the material table indexed through JM, generic per-cell planes,
and the ten planes of an isotropic Biot medium with the aliases resolved at
compile time.  The bar is bit-for-bit equality, as in the other parity
tests.
"""
import numpy as np
import pytest

from helpers import compare_state, randomize_state, small_job

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True, params=["split", "fused", "global", "tma", "coretma", "march"])
def kernel_variant(request, monkeypatch):
    monkeypatch.setenv("FDP_KERNEL_VARIANT", request.param)
    return request.param


def _case(medium: str, si: bool, seed: int):
    from fdporo import media
    cfg, med = small_job(mx=160, mz=100, tpml=8, nsteps=40, si=si, per_cell=(medium != "table"), seed=seed)
    if medium == "planes":
        # an anisotropic perturbation: SIG_ZZ_1 no longer equals SIG_XX_2
        t = np.array(med.table, copy=True)
        t[:, media.COL["SIG_ZZ_1"]] *= 1.0 + 0.05 * np.linspace(0.0, 1.0, t.shape[0])
        med = media.Medium(med.jm_rows, t)
    return cfg, med


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
@pytest.mark.parametrize("medium", ["biot", "planes", "table"])
def test_interior_from_random_state(prec, si, medium):
    from fdporo import job
    from oracle.oracle import make_oracle
    cfg, med = _case(medium, si, seed=41)
    inp = job.prepare(cfg, med, prec)
    eng, orc = job.make_engine(inp), make_oracle(inp)
    assert eng.medium_info()["mode"] == medium
    randomize_state([eng, orc], inp, seed=43)
    eng.time_loop(1, 3)
    orc.time_loop(1, 3)
    compare_state(eng, orc)
    eng.time_loop(4, 40)
    orc.time_loop(4, 40)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 40), orc.receivers(1, 40))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_interior_shot_from_rest(prec):
    from fdporo import job
    from oracle.oracle import make_oracle
    cfg, med = _case("biot", True, seed=47)
    inp = job.prepare(cfg, med, prec)
    eng, orc = job.make_engine(inp), make_oracle(inp)
    eng.time_loop(1, 40)
    orc.time_loop(1, 40)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, 40), orc.receivers(1, 40))
    assert np.abs(orc.field("PRES")).max() > 0
