"""The no-allocation receiver entry point (fdp_receivers_noalloc).

It is for callers that cannot allocate device memory -- a host whose device
arrays come from a memory pool it manages itself, a runtime that forbids
allocation once running -- so everything it reads and writes is the
caller's device memory.  Here the test itself provides that memory
(torch tensors), runs the engine one level at a time, hands the engine's
wavefield after each level to the entry point, and checks that its output
equals the engine's own fdp_get_receivers values for that level, bit for
bit, over many consecutive calls.  This file is collected last so that a
run stopping at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import small_job

pytestmark = pytest.mark.gpu

FIELDS = ("UM", "WM", "QX", "QZ", "PRES", "TXX")


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("si", [True, False])
def test_noalloc_matches_engine_receivers(prec, si):
    import torch
    from fdporo import job, native
    lib = native.load()
    cfg, med = small_job(si=si, nsteps=12, seed=41)
    inp = job.prepare(cfg, med, prec)
    eng = job.make_engine(inp)
    mr = len(inp.irecx)
    dtype = torch.float64 if prec == "f64" else torch.float32
    rec = torch.from_numpy(np.stack([inp.irecx, inp.lrecx, inp.irecz, inp.lrecz], axis=1)
                           .astype(np.int32).reshape(-1).copy()).cuda()
    out = torch.zeros((mr, native.FDP_REC_VALUES), dtype=dtype, device="cuda")
    for level in range(1, 13):
        eng.time_loop(level, level)
        dev = {n: torch.from_numpy(eng.field(n)).cuda() for n in FIELDS}
        torch.cuda.synchronize()
        rc = lib.fdp_receivers_noalloc(inp.precision, *[_ptr(dev[n]) for n in FIELDS], inp.nx, inp.nz, inp.nx,
                                       1 - inp.tpml, _ptr(rec), mr, inp.rec_flags, inp.dt, level, _ptr(out), None)
        assert rc == 0, lib.fdp_last_error(None)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), eng.receivers(level, 1)[0])
    assert np.abs(out.cpu().numpy()).max() > 0
    eng.close()


def test_noalloc_rejects_more_receivers_than_its_capacity():
    import torch
    from fdporo import native
    lib = native.load()
    too_many = 16385  # FDP_NOALLOC_MAX_RECEIVERS + 1
    f = torch.zeros(64, device="cuda")
    rc = lib.fdp_receivers_noalloc(4, *[_ptr(f)] * 6, 8, 8, 8, 1, _ptr(f), too_many, 7, 1e-4, 1, _ptr(f), None)
    assert rc == -1
    assert b"capacity" in lib.fdp_last_error(None)


def test_noalloc_resumed_run_primed_at_the_level_before():
    """A run resumed at level k > 1 calls the entry point once with level
    k-1's wavefield (output discarded); from level k on, its output equals
    the engine's.  A call with no receivers only looks the device state up."""
    import torch
    from fdporo import job, native
    lib = native.load()
    rc = lib.fdp_receivers_noalloc(4, *[None] * 6, 8, 8, 8, 1, None, 0, 7, 1e-4, 1, None, None)
    assert rc == 0, lib.fdp_last_error(None)
    cfg, med = small_job(si=True, nsteps=12, seed=43)
    inp = job.prepare(cfg, med, "f32")
    eng = job.make_engine(inp)
    mr = len(inp.irecx)
    rec = torch.from_numpy(np.stack([inp.irecx, inp.lrecx, inp.irecz, inp.lrecz], axis=1)
                           .astype(np.int32).reshape(-1).copy()).cuda()
    out = torch.zeros((mr, native.FDP_REC_VALUES), dtype=torch.float32, device="cuda")
    eng.time_loop(1, 6)
    for level in range(6, 10):
        if level > 6:
            eng.time_loop(level, level)
        dev = {n: torch.from_numpy(eng.field(n)).cuda() for n in FIELDS}
        torch.cuda.synchronize()
        rc = lib.fdp_receivers_noalloc(inp.precision, *[_ptr(dev[n]) for n in FIELDS], inp.nx, inp.nz, inp.nx,
                                       1 - inp.tpml, _ptr(rec), mr, inp.rec_flags, inp.dt, level, _ptr(out), None)
        assert rc == 0, lib.fdp_last_error(None)
        torch.cuda.synchronize()
        if level > 6:
            np.testing.assert_array_equal(out.cpu().numpy(), eng.receivers(level, 1)[0])
    eng.close()
