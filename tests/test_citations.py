"""Every reference citation in the project's files resolves.

The oracle's fidelity, and the parity claims of the kernels, rest on
file:line citations of the reference's Fortran (``name.F90:N``,
``name.F90:N-M``, ``name.F90:N,M-K``).  This test reads the reference's
source tree (``FDP_REFERENCE_DIR``, default the reference checkout) and
checks that each cited file exists, each cited range lies inside it and
holds at least one statement (not only blank or comment lines), and that a
set of anchor citations on the hot path holds the statement it names.
The project's files are every tracked file in a subdirectory, the Python
files at the top, and the top-level documents whose title names the GB300
engine (records kept beside them, such as measurement logs, are not
sources).  Skipped where the reference's sources are absent.
"""
import os
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("FDP_REFERENCE_DIR", "/root/reference"))

CITE = re.compile(r"\b([A-Za-z_][A-Za-z0-9_]*\.(?:F90|F)):(\d+(?:-\d+)?(?:,\d+(?:-\d+)?)*)")

# citations of code the reference keeps commented out, on purpose
COMMENTED = {"read_model_par.F90:78-87"}

# citation -> text that the cited lines must contain (whitespace-insensitive)
ANCHORS = {
    "inh_qx_int.F90:44-52": "EXP(-REL3_QXT(JM1))*QXT(I,L)",
    "inh_v_uv_int.F90:45-54": "(REL2_UT(JM1)/REL3_QXT(JM1))*(1._PP-EXP(-REL3_QXT(JM1)))",
    "inh_qz_int.F90:45-53": "EXP(-REL3_QZT(JM1))*QZT(I,L)",
    "strain_uw_xz.F90:81-84": "A*(UTM(I,LP1)-UTM(I,L2)",
    "strain_uw_zz.F90:51,58-59": "A*(WTM(I,LP2)-WTM(I,LM1))",
    "strain_q_zz.F90:48,55-56": "A*(QZT(I,LP2)-QZT(I,LM1))",
    "strain_uw_xx.F90:82-83": "A*(UTM(I+2,L)-UTM(I-1,L))",
    "strain_q_xx.F90:77-78": "A*(QXT(I+2,L)-QXT(I-1,L))",
    "stress_xz.F90:44-46": "TXZ=MU(JM1)*EXZT(I)",
    "stress_nn.F90:53-59": "SIG_XX_1(JM1)*EXXT(I)",
    "read_model_par.F90:63-74": "REL1_U=DT*REL1_U/H",
    "read_open.F90:149-151": "MZ=MZ+2",
    "read_open.F90:165-169": "LIN_Z=NINT(Z_SOURCE/H)",
    "tl_alloc.F90:24-36": "ALLOCATE(UM(",
    "store_seismograms.F90:65-66": "SPU(J)=(S-SSU(J))/DT",
    "hplane_0_stress.F90:49-53": "TXZ(:,0)=-TXZ(:,4)",
    "hplane_1_stress.F90:45-53": "TXZ(:,2)=0.",
    "time_loop.F90:79-86": "INQUIRE(FILE='STOP',EXIST=EX)",
    "mod_auxil.F90:20": "A=-1./24.,B=9./8.",
}


def _project_file(t: str) -> bool:
    if "/" in t or t.endswith(".py"):
        return True
    if not t.endswith(".md"):
        return False
    with open(ROOT / t, errors="replace") as f:
        return "GB300" in f.readline()


def _tracked():
    out = subprocess.run(["git", "ls-files"], cwd=ROOT, capture_output=True, text=True).stdout.split()
    return [ROOT / t for t in out if _project_file(t)]


def _ranges(spec):
    for piece in spec.split(","):
        a, _, b = piece.partition("-")
        yield int(a), int(b or a)


def _lines(name, cache={}):
    if name not in cache:
        hits = list(REF.rglob(name))
        cache[name] = hits[0].read_text(errors="replace").splitlines() if hits else None
    return cache[name]


def _is_statement(line):
    s = line.strip()
    return bool(s) and not s.startswith("!")


pytestmark = pytest.mark.skipif(not REF.is_dir(), reason="reference sources not present")


def test_every_citation_resolves():
    bad, n = [], 0
    for path in _tracked():
        if not path.is_file():
            continue
        try:
            text = path.read_text()
        except UnicodeDecodeError:
            continue
        for ln, line in enumerate(text.splitlines(), 1):
            for m in CITE.finditer(line):
                name, spec = m.group(1), m.group(2)
                lines = _lines(name)
                where = f"{path.relative_to(ROOT)}:{ln}: {m.group(0)}"
                if lines is None:
                    bad.append(f"{where} (no such reference file)")
                    continue
                for a, b in _ranges(spec):
                    n += 1
                    if not 1 <= a <= b <= len(lines):
                        bad.append(f"{where} (file has {len(lines)} lines)")
                    elif m.group(0) not in COMMENTED and not any(_is_statement(x) for x in lines[a - 1:b]):
                        bad.append(f"{where} (only blank or comment lines)")
    assert n > 200
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("cite", sorted(ANCHORS))
def test_anchor_citation_holds_its_statement(cite):
    name, spec = cite.split(":")
    lines = _lines(name)
    assert lines is not None
    text = "".join("".join(lines[a - 1:b]) for a, b in _ranges(spec))
    squeeze = lambda s: re.sub(r"[\s&]", "", s)
    assert squeeze(ANCHORS[cite]) in squeeze(text), f"{cite} does not hold {ANCHORS[cite]!r}"
