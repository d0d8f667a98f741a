"""The committed regression fixtures (tests/golden, made by
tests/golden/make_golden.py from the CPU oracle) against the oracle on the
CPU and the engine on the GPU.  On the machine type the fixtures were made
on the comparison is bit for bit; elsewhere the C library's exp/log may
differ in the last bit, so it allows a relative 1e-9 (FP64) or 1e-4 (FP32)
of each array's largest value."""
import platform
from pathlib import Path

import numpy as np
import pytest

from golden.make_golden import CASES, FIELDS, run_case

HERE = Path(__file__).resolve().parent / "golden"


def _check(out: dict, ref, prec: str) -> None:
    exact = str(ref["machine"]) == platform.machine()
    tol = 1e-9 if prec == "f64" else 1e-4
    for k in ["receivers"] + FIELDS:
        a, b = np.asarray(out[k]), ref[k]
        if exact:
            np.testing.assert_array_equal(a, b, err_msg=k)
        else:
            scale = max(float(np.abs(b).max()), 1e-30)
            assert float(np.abs(a.astype(np.float64) - b).max()) <= tol * scale, k


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_golden(case):
    from oracle.oracle import make_oracle
    name, kw, prec, levels = case
    _check(run_case(make_oracle, kw, prec, levels), np.load(HERE / f"{name}.npz"), prec)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_engine_matches_golden(case):
    from fdporo import job
    name, kw, prec, levels = case
    _check(run_case(job.make_engine, kw, prec, levels), np.load(HERE / f"{name}.npz"), prec)
