"""Size-independent properties at the benchmark's full size, on the GPU.

The 2048^2 layered per-cell medium of the benchmark (4.3 M cells with the
PML), FP32: no source gives exactly zero everywhere; every operation of
the scheme is linear in the wavefield, so a source scaled by 4 scales every
field and seismogram by 4 -- to within 1e-5 of the peak: each cell's value
starts as the numerical precursor ahead of the front, in subnormal numbers
(below 1.2e-38, where rounding is not scale-free), and the linear recursion
carries those roundings up with the precursor's growth (a few ulp of the
wavefield after 300 levels; the CPU oracle, bit-identical to the engine,
does the same); and the 20-cell PML of a small region reflects little
against a wide run of the same medium.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LEVELS = 300


@pytest.fixture(scope="module")
def full_size():
    from fdporo import job
    cfg, med = job.layered(mx=2048, mz=2048, nsteps=LEVELS, tpml=20, n_rec=512, seed=20250, layer_depth=1024.0)
    return job.prepare(cfg, med, "f32")


def _run(inp, scale):
    import dataclasses
    from fdporo import job
    src = dataclasses.replace(inp, sourtf=np.ascontiguousarray(inp.sourtf * np.float32(scale)))
    eng = job.make_engine(src)
    eng.time_loop(1, LEVELS)
    return eng


def test_no_source_leaves_every_field_zero(full_size):
    from fdporo.native import MEMORY_VARS, WAVEFIELD
    eng = _run(full_size, 0.0)
    for n in WAVEFIELD + MEMORY_VARS:
        assert not np.any(eng.field(n)), n
    assert not np.any(eng.receivers(1, LEVELS))


def test_source_scaled_by_four_scales_everything_by_four(full_size):
    from fdporo.native import MEMORY_VARS, WAVEFIELD
    a, b = _run(full_size, 1.0), _run(full_size, 4.0)
    for n in WAVEFIELD + MEMORY_VARS:
        x, y = a.field(n), b.field(n)
        peak = float(np.max(np.abs(x))) if x.size else 0.0
        np.testing.assert_allclose(y, 4 * x, rtol=0, atol=4e-5 * peak + 1e-30, err_msg=n)
    ra, rb = a.receivers(1, LEVELS), b.receivers(1, LEVELS)
    np.testing.assert_allclose(rb, 4 * ra, rtol=0, atol=4e-5 * float(np.max(np.abs(ra))))


def test_pml_reflects_little_against_a_wide_run():
    from fdporo import edge
    pair = edge.make_pair(7, n=128, margin=96, depth_margin=160, nsteps=700, f0=100.0, n_rec=33)
    res = edge.evaluate(pair, 700, tpml=20)
    assert res["reflected_energy"] < 1e-3, res
    assert res["seismogram_rel_l2"] < 0.05, res
