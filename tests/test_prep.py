"""Host set-up (libfdp's C++ restatement of PPML, PRE_NR_COEF1/NONREF,
OPEN_SR_FILE, READ_MODEL, READ_MODEL_PAR) against the independent numpy
restatement in oracle/setup_ref.py.  Runs on the CPU."""
import numpy as np
import pytest

from fdporo import job, media
from oracle import setup_ref

# numpy's exp/log/pow may differ from the C library's by an ulp
RTOL = {"f32": 2e-6, "f64": 1e-13}


def _dt(prec):
    return np.float64 if prec == "f64" else np.float32


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
def test_jm_expansion_and_scaling(prec, si):
    cfg, _ = job.small_homogeneous(mx=30, mz=20, nsteps=10, tpml=5)
    cfg.stress_imaging = si
    rng = np.random.default_rng(1)
    rows = rng.integers(1, 6, size=(cfg.n_model_rows, cfg.mx)).astype(np.int32)
    tab = media.biot_table(2650, 1000, 0.2 + 0.01 * np.arange(5), 37e9, 2.25e9, 10e9, 9e9, 1e-12, 1e-3, 2.0)
    med = media.Medium(rows, tab)
    inp = job.prepare(cfg, med, prec)
    ref = setup_ref.expand_jm(rows, cfg.mx, cfg.mz_grid, cfg.tpml, si)
    np.testing.assert_array_equal(inp.jm, ref)
    np.testing.assert_array_equal(inp.table, setup_ref.scale_table(tab, cfg.dt, cfg.h, _dt(prec)))


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("ktbo,wc,sf", [(0, 0.0, 0.0), (0, 30.0, 0.5), (2, 40.0, 0.0)])
def test_pml_profiles(prec, ktbo, wc, sf):
    cfg, med = job.layered(mx=24, mz=18, nsteps=10, tpml=6, n_rec=4, seed=3, layer_depth=9.0)
    cfg.ktbo, cfg.wc, cfg.sf = ktbo, wc, sf
    inp = job.prepare(cfg, med, prec)
    ref = setup_ref.ppml(inp.jm, inp.table, cfg.mx, cfg.mz_grid, cfg.tpml, ktbo, cfg.r, cfg.tau, cfg.pow_, sf, wc,
                         cfg.dt, cfg.h, _dt(prec))
    # ODC = ...*(DENOM-1) cancels: an ulp of DENOM is an absolute ulp of 1
    atol = 4 * np.finfo(_dt(prec)).eps
    for k, (a, b) in enumerate(zip(inp.profiles, ref)):
        np.testing.assert_allclose(a, b, rtol=RTOL[prec], atol=atol, err_msg=f"profile {k}")
    # the damping grows into the layer and ODA(0) = ODB(0) = 1, ODC(0) = 0
    assert np.all(inp.profiles[0][:, 0] == 1) and np.all(inp.profiles[2][:, 0] == 0)
    if ktbo == 0:
        assert np.all(np.diff(inp.profiles[1][:, :], axis=1) <= 0)


def test_pml_zero_over_zero_when_damping_is_switched_off():
    # KTBO /= 0 sets OMG = 0 (ppml.F90:262); with WC = 0 the coefficient
    # OMGPDT/(OMGPDT+WC*AP*DT) of ppml.F90:283 is 0/0
    cfg, med = job.small_homogeneous(mx=20, mz=16, nsteps=10, tpml=4)
    cfg.ktbo = 1
    inp = job.prepare(cfg, med, "f64")
    assert np.all(np.isnan(inp.profiles[10][:, 1:]))


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("ktbo", list(range(10)))
def test_bottom_coefficients(prec, ktbo):
    cfg, med = job.small_homogeneous(mx=20, mz=16, nsteps=10, tpml=4)
    cfg.ktbo, cfg.omg, cfg.wc = ktbo, 60.0, 10.0
    inp = job.prepare(cfg, med, prec)
    dt = _dt(prec)
    omg = dt(dt(cfg.omg) / 6.283185307179586476925286766559)
    ref = setup_ref.bottom_nr(inp.jm, inp.table, cfg.mx, cfg.mz_grid, cfg.tpml, ktbo, cfg.dt, cfg.h, omg, cfg.wb,
                              cfg.thpple, cfg.thssle, dt)
    np.testing.assert_allclose(inp.ab, ref, rtol=RTOL[prec] * 10, atol=1e-15)
    if ktbo == 0:
        assert np.all(inp.ab == 0)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("key_sour,qr", [(0, 0.3), (1, 0.0), (2, 0.25), (3, 0.0)])
def test_source_spline(prec, key_sour, qr):
    dt = _dt(prec)
    rng = np.random.default_rng(7)
    t = np.sort(rng.random(40)) * 0.01
    v = rng.standard_normal(40)
    out = np.zeros((150, 2), dtype=dt)
    import ctypes as C
    from fdporo import native
    lib = native.load()
    tt, vv = t.astype(dt), v.astype(dt)
    rc = lib.fdp_prep_source(8 if prec == "f64" else 4, 40, tt.ctypes.data_as(C.c_void_p),
                             vv.ctypes.data_as(C.c_void_p), 150, 1e-4, 2.0, key_sour, qr,
                             out.ctypes.data_as(C.c_void_p))
    assert rc == 0
    ref = setup_ref.source(tt, vv, 150, 1e-4, 2.0, key_sour, qr, dt)
    np.testing.assert_allclose(out, ref, rtol=RTOL[prec] * 50, atol=1e-12 if prec == "f64" else 1e-5)
    # levels past the last sample are zero (open_sr_file.F90:86)
    last = int(np.floor(float(tt[-1]) / 1e-4)) + 1
    assert np.all(out[last + 1:] == 0)


def test_spline_reproduces_samples_on_the_grid():
    cfg, _ = job.small_homogeneous(mx=20, mz=16, nsteps=200, tpml=4, f0=100.0)
    inp = job.prepare(cfg, media.homogeneous(cfg.mx, cfg.n_model_rows), "f64")
    expect = job.ricker(np.arange(200) * 1e-4, 100.0) / (cfg.h * cfg.h)
    np.testing.assert_allclose(inp.sourtf[:, 0], expect, rtol=0, atol=1e-12)
    assert np.all(inp.sourtf[:, 1] == 0)


def test_velocities_of_sandstone():
    # fast P, slow P and S speeds of the brine-saturated sandstone
    t = media.rock_table(media.SANDSTONE)
    c = setup_ref.COL
    vpf, vps, vs = setup_ref.calcul_velocity(t[c["SXX1"]], -t[c["P1"]], -t[c["P3"]], t[c["MU"]], t[c["R1U"]],
                                             t[c["R2QX"]], t[c["R3U"]], np.float64)
    assert 3300 < vpf < 3600 and 1900 < vs < 2100 and 500 < vps < 1200
    import ctypes as C
    from fdporo import native
    out = [C.c_double(), C.c_double(), C.c_double()]
    native.load().fdp_prep_velocities(8, t[c["SXX1"]], -t[c["P1"]], -t[c["P3"]], t[c["MU"]], t[c["R1U"]],
                                      t[c["R2QX"]], t[c["R3U"]], *[C.byref(o) for o in out])
    np.testing.assert_allclose([o.value for o in out], [vpf, vps, vs], rtol=1e-14)
