"""Generates the regression fixtures in this directory from the CPU oracle.

The reference ships no golden vectors and cannot be built here (no Fortran
compiler), so these fixtures pin the oracle and the engine to the values
this commit's oracle produces: small seeded jobs run through the oracle,
their receiver values and final wavefields stored as .npz.  The test
`tests/test_golden.py` checks the oracle (CPU) and the engine (GPU) against
them.  Regenerate only when a deliberate change of the arithmetic is made:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (str(ROOT), str(ROOT / "2d-vqsp-fd-sim_gb300"), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

# (name, small_job keyword arguments, precision, levels)
CASES = [
    ("si_table_f64", dict(mx=40, mz=30, tpml=6, nsteps=80, si=True, seed=101), "f64", 80),
    ("si_table_f32", dict(mx=40, mz=30, tpml=6, nsteps=80, si=True, seed=101), "f32", 80),
    ("nosi_table_f64", dict(mx=36, mz=28, tpml=5, nsteps=60, si=False, seed=102), "f64", 60),
    ("si_percell_f64", dict(mx=72, mz=56, tpml=6, nsteps=60, si=True, per_cell=True, seed=103), "f64", 60),
    ("si_bottom_ktbo3_f64", dict(mx=40, mz=30, tpml=6, nsteps=50, si=True, seed=104, ktbo=3, wc=200.0), "f64", 50),
]
FIELDS = ["UM", "WM", "QX", "QZ", "TXX", "TZZ", "TXZ", "PRES"]


def run_case(engine_factory, kw: dict, precision: str, levels: int) -> dict:
    from fdporo import job
    from helpers import small_job
    cfg, med = small_job(**kw)
    if kw.get("ktbo"):
        cfg.omg = 60.0
    inp = job.prepare(cfg, med, precision)
    e = engine_factory(inp)
    e.time_loop(1, levels)
    out = {"receivers": e.receivers(1, levels)}
    for f in FIELDS:
        out[f] = e.field(f)
    return out


def main() -> None:
    import platform
    from oracle.oracle import make_oracle
    for name, kw, prec, levels in CASES:
        out = run_case(make_oracle, kw, prec, levels)
        # the C library's exp and log may differ in the last bit between
        # machines; the fixtures record where they were made
        out["machine"] = np.array(platform.machine())
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, {k: v.shape for k, v in out.items()}, float(np.abs(out["receivers"]).max()))


if __name__ == "__main__":
    main()
