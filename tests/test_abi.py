"""The C ABI library loads, exports every entry point the headers declare,
and validates its arguments on the host.  No kernel runs here."""
import ctypes as C
import re
from pathlib import Path

import pytest

from conftest import gpu_present

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fdp_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_headers_declare_the_abi():
    names = declared_functions()
    for must in ("fdp_create", "fdp_set_medium", "fdp_set_pml", "fdp_set_bottom_nr", "fdp_set_source",
                 "fdp_set_receivers", "fdp_run", "fdp_get_receivers", "fdp_get_snapshot", "fdp_destroy",
                 "fdp_prep_pml", "fdp_prep_bottom_nr", "fdp_prep_source"):
        assert must in names


def test_library_exports_every_declared_symbol(fdp_lib):
    from fdporo import native
    for name in declared_functions():
        assert hasattr(fdp_lib, name), f"{name} is declared but not exported"
        assert name in native.SIGNATURES, f"{name} has no ctypes signature"


def _grid(**kw):
    from fdporo import native
    g = dict(mx=32, mz=24, tpml=4, stress_imaging=1, lin_x=16, lin_z=10, precision=4, device=0, h=1.0, dt=1e-4,
             tau_eps=0.0)
    g.update(kw)
    return native.fdp_grid(**g)


@pytest.mark.parametrize("bad", [dict(precision=2), dict(mx=4), dict(mz=5), dict(tpml=-1), dict(lin_z=1),
                                 dict(lin_z=23), dict(h=0.0), dict(dt=-1.0)])
def test_create_rejects_bad_geometry(fdp_lib, bad):
    ctx = C.c_void_p()
    rc = fdp_lib.fdp_create(C.byref(_grid(**bad)), C.byref(ctx))
    assert rc == -1
    assert not ctx.value
    assert fdp_lib.fdp_last_error(None)


def test_null_context_is_rejected(fdp_lib):
    assert fdp_lib.fdp_run(None, 1, 1) == -1
    assert fdp_lib.fdp_synchronize(None) == -1
    assert fdp_lib.fdp_share_medium(None, None) == -1
    assert fdp_lib.fdp_diag_wait_timeout(None, 10) == -1
    fdp_lib.fdp_destroy(None)


@pytest.mark.skipif(gpu_present(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_cleanly(fdp_lib):
    ctx = C.c_void_p()
    rc = fdp_lib.fdp_create(C.byref(_grid()), C.byref(ctx))
    assert rc == -2  # FDP_ERR_CUDA
    assert not ctx.value
    assert b"cuda" in fdp_lib.fdp_last_error(None).lower()


def test_engine_raises_without_gpu():
    if gpu_present():
        pytest.skip("GPU present")
    from fdporo import Engine, FdpError
    with pytest.raises(FdpError):
        Engine(32, 24, 4, 16, 10, 1.0, 1e-4)


def test_errors_without_a_context_are_per_thread(fdp_lib):
    """fdp_last_error(NULL) reports the calling thread's own last failure:
    two threads failing at once each read their own message."""
    import threading
    bar = threading.Barrier(2)
    seen = {}

    def worker(tag, bad):
        ctx = C.c_void_p()
        bar.wait()
        for _ in range(200):
            rc = fdp_lib.fdp_create(C.byref(_grid(**bad)), C.byref(ctx))
            assert rc == -1
            seen.setdefault(tag, set()).add(fdp_lib.fdp_last_error(None))

    ts = [threading.Thread(target=worker, args=("precision", dict(precision=2))),
          threading.Thread(target=worker, args=("h", dict(h=0.0)))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert len(seen["precision"]) == 1 and len(seen["h"]) == 1
    assert seen["precision"] != seen["h"]
