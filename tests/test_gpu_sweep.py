"""A seeded sweep of small configurations against the oracle.

Each case draws its grid (including sizes where a core rectangle is empty
or a single column group), PML width, free-surface mode, bottom key,
medium kind, source position, receivers, precision, kernel variant and run
split from a fixed seed, starts from a random state and must match the
oracle bit for bit in every field, memory variable, the bottom history and
every receiver value.
"""
import numpy as np
import pytest

from helpers import compare_state, randomize_state, small_job

pytestmark = pytest.mark.gpu

VARIANTS = ["split", "fused", "global", "tma", "coretma"]


def _case(k: int):
    rng = np.random.default_rng(1000 + k)
    mx = int(rng.integers(8, 140))
    mz = int(rng.integers(8, 100))
    tpml = int(rng.choice([1, 2, 3, 6, 10, 20]))
    si = bool(rng.integers(0, 2))
    ktbo = int(rng.choice([0, 0, 0, 1, 3, 5, 9]))
    per_cell = bool(rng.integers(0, 2))
    prec = "f64" if rng.random() < 0.3 else "f32"
    levels = int(rng.integers(3, 70))
    split = int(rng.integers(1, levels + 1))
    n_rec = int(rng.integers(1, 12))
    variant = VARIANTS[int(rng.integers(0, len(VARIANTS)))]
    return dict(mx=mx, mz=mz, tpml=tpml, si=si, ktbo=ktbo, per_cell=per_cell, prec=prec, levels=levels,
                split=split, n_rec=n_rec, variant=variant, seed=2000 + k)


@pytest.mark.parametrize("k", range(160))
def test_random_case_matches_oracle(k, monkeypatch):
    from fdporo import job
    from oracle.oracle import make_oracle
    c = _case(k)
    monkeypatch.setenv("FDP_KERNEL_VARIANT", c["variant"])
    cfg, med = small_job(mx=c["mx"], mz=c["mz"], tpml=c["tpml"], nsteps=c["levels"], si=c["si"],
                         per_cell=c["per_cell"], seed=c["seed"], n_rec=c["n_rec"], ktbo=c["ktbo"],
                         wc=200.0 if c["ktbo"] else 0.0)
    if c["ktbo"]:
        cfg.omg = 60.0
    # the source row must lie in 2..MZ-2 (fdp_create rejects others)
    lo, hi = 2, c["mz"] - 2
    try:
        inp = job.prepare(cfg, med, c["prec"])
    except Exception as ex:  # a geometry the set-up itself refuses
        pytest.skip(f"set-up refuses {c}: {ex}")
    if not (lo <= inp.lin_z <= hi):
        pytest.skip(f"source row {inp.lin_z} outside 2..MZ-2 for {c}")
    eng, orc = job.make_engine(inp), make_oracle(inp)
    randomize_state([eng, orc], inp, seed=c["seed"] + 1)
    for a, b in ((1, c["split"]), (c["split"] + 1, c["levels"])):
        if a > b:
            continue
        eng.time_loop(a, b)
        orc.time_loop(a, b)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, c["levels"]), orc.receivers(1, c["levels"]))


@pytest.mark.parametrize("k", range(80))
def test_random_case_matches_oracle_march(k, monkeypatch):
    """Other draws with the march variant and any number of CTAs (FP64,
    table media and grids too small for its region run the split)."""
    from fdporo import job
    from oracle.oracle import make_oracle
    c = _case(500 + k)
    monkeypatch.setenv("FDP_KERNEL_VARIANT", "march")
    monkeypatch.setenv("FDP_MARCH_CTAS", str(1 + k % 13))
    cfg, med = small_job(mx=c["mx"], mz=c["mz"], tpml=c["tpml"], nsteps=c["levels"], si=c["si"],
                         per_cell=True, seed=c["seed"], n_rec=c["n_rec"], ktbo=c["ktbo"],
                         wc=200.0 if c["ktbo"] else 0.0)
    if c["ktbo"]:
        cfg.omg = 60.0
    try:
        inp = job.prepare(cfg, med, c["prec"])
    except Exception as ex:
        pytest.skip(f"set-up refuses {c}: {ex}")
    if not (2 <= inp.lin_z <= c["mz"] - 2):
        pytest.skip(f"source row {inp.lin_z} outside 2..MZ-2 for {c}")
    eng, orc = job.make_engine(inp), make_oracle(inp)
    randomize_state([eng, orc], inp, seed=c["seed"] + 1)
    for a, b in ((1, c["split"]), (c["split"] + 1, c["levels"])):
        if a > b:
            continue
        eng.time_loop(a, b)
        orc.time_loop(a, b)
    compare_state(eng, orc)
    np.testing.assert_array_equal(eng.receivers(1, c["levels"]), orc.receivers(1, c["levels"]))
