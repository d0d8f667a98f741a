"""In-tree build of the native engine library ``libfdp.so``.

Compiles the CUDA kernels and C ABI (``csrc/fdp_engine.cu``) for sm_103a and
the host set-up code (``csrc/fdp_prep.cpp``), each translation unit in
parallel, and links them into ``lib/libfdp.so`` next to this package.  The
CUDA runtime is linked statically, so the library loads on a machine without
a GPU (its entry points then fail with FDP_ERR_CUDA).

Floating-point flags: ``--fmad=false`` and ``-ffp-contract=off`` keep every
multiply and add separately rounded, so the kernels evaluate the
reference's expressions exactly as written.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # 2d-vqsp-fd-sim_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
INCLUDE = REPO_ROOT / "include"
LIB_DIR = PKG_ROOT / "lib"
LIB_PATH = LIB_DIR / "libfdp.so"
OBJ_DIR = PKG_ROOT / "build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "--fmad=false", "-std=c++17",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]

SOURCES = ["fdp_engine.cu", "fdp_edge.cu", "fdp_noalloc.cu", "fdp_prep.cpp", "fdp_io.cpp"]
HOST_EXE = LIB_DIR / "fdp_host"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfdp.so")


def _inputs() -> list[Path]:
    files = [CSRC / s for s in SOURCES] + [CSRC / "fdp_host.cpp"]
    files += sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    return files


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Builds ``lib/libfdp.so`` if any source is newer; returns its path."""
    deps = _inputs()
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    nvcc = _nvcc()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)

    def compile_one(src: str) -> Path:
        s = CSRC / src
        obj = OBJ_DIR / (s.stem + ".o")
        if s.suffix == ".cu":
            cmd = [nvcc, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(s), "-o", str(obj)]
        else:
            cmd = ["g++", *CXX_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(s), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(SOURCES), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    # the drop-in host executable, linked against the library next to it
    exe_tmp = HOST_EXE.with_suffix(".tmp")
    cmd = ["g++", *CXX_FLAGS, f"-I{INCLUDE}", str(CSRC / "fdp_host.cpp"), "-o", str(exe_tmp),
           f"-L{LIB_DIR}", "-lfdp", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(exe_tmp, HOST_EXE)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
