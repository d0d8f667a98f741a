"""The reference's file formats (CPU): the E13.6 edit descriptor of the
seismogram files, namelist input, and gfortran unformatted records."""
import numpy as np
import pytest

from fdporo import formats, job


@pytest.mark.parametrize("value,text", [
    (1.0, " 0.100000E+01"),
    (-1.0, "-0.100000E+01"),
    (0.0, " 0.000000E+00"),
    (-0.0, "-0.000000E+00"),
    (123456.7, " 0.123457E+06"),
    (1e-5, " 0.100000E-04"),
    (0.9999995, " 0.100000E+01"),
    (3.14159265, " 0.314159E+01"),
    (-2.5e-37, "-0.250000E-36"),
    (1e100, " 0.100000+101"),
    (1e-101, " 0.100000-100"),
    (1e-99, " 0.100000E-98"),
])
def test_e13_6(value, text):
    assert formats.format_e(value) == text
    assert len(text) == 13


def test_e_format_overflow_and_specials():
    assert formats.format_e(1.0, 8, 6) == "********"
    assert formats.format_e(1.0, 12, 6) == "0.100000E+01"   # no room for the optional blank
    assert formats.format_e(-1.0, 12, 6) == "-.100000E+01"  # nor for the leading zero
    assert formats.format_e(float("nan")).strip() == "NaN"
    assert formats.format_e(float("-inf")).strip() == "-Infinity"


def test_float32_values_are_formatted_exactly():
    v = np.float32(0.1)
    assert formats.format_e(float(v)) == " 0.100000E+00"
    assert formats.format_e(float(np.float32(1.2345675))) == " 0.123457E+01"


NML = """
&CONTROLDATA  TPML = 20, PROCX=1 PROCZ = 1,
   STRESS_IMAGING = .TRUE. /   ! trailing comment
&CONTROLDATA1 MT=0.15, R=1.0D-3, IPAS2 = 500 /
&NAMES_SR_REC SR_FILE_NAME='STF.DAT', REC_FILE_NAME = "R E C.DAT" /
&keys key_tlv=T, KEY_SNV=.false. /
"""


def test_namelist_parsing():
    g = formats.namelist_get
    assert g(NML, "CONTROLDATA", "TPML") == "20"
    assert g(NML, "controldata", "procz") == "1"
    assert g(NML, "CONTROLDATA", "STRESS_IMAGING") == ".TRUE."
    assert g(NML, "CONTROLDATA1", "R") == "1.0D-3"
    assert g(NML, "CONTROLDATA1", "IPAS2") == "500"
    assert g(NML, "NAMES_SR_REC", "REC_FILE_NAME") == "R E C.DAT"
    assert g(NML, "KEYS", "KEY_SNV") == ".false."
    assert g(NML, "KEYS", "KEY_TLQ") is None
    assert g(NML, "MISSING", "X") is None
    # a group name that is a prefix of another is not matched
    assert g(NML, "CONTROLDATA", "MT") is None


def test_records_round_trip(tmp_path):
    p = tmp_path / "f.bin"
    recs = [np.arange(7, dtype=np.int32).tobytes(), b"", np.linspace(0, 1, 1000).tobytes()]
    for r in recs:
        formats.append_record(p, r)
    raw = p.read_bytes()
    # gfortran layout: 4-byte length, payload, 4-byte length
    assert raw[:4] == np.int32(28).tobytes() and raw[32:36] == np.int32(28).tobytes()
    for k, r in enumerate(recs):
        assert formats.read_record(p, k) == r
    with pytest.raises(IOError):
        formats.read_record(p, 3)


def test_job_directory_round_trip(tmp_path):
    cfg, med = job.small_homogeneous(mx=40, mz=30, nsteps=50, tpml=6, n_rec=5)
    d = formats.write_job(tmp_path / "job", "TEST", cfg, med, "f32")
    text = (d / "TEST.IN").read_text()
    assert formats.namelist_get(text, "CONTROLDATA", "TPML") == "6"
    mt = float(formats.namelist_get(text, "CONTROLDATA1", "MT"))
    assert int(np.float32(mt) / np.float32(cfg.dt)) + 1 == cfg.mt2
    rows = [np.frombuffer(formats.read_record(d / "TEST.JMH", r), np.int32) for r in range(cfg.n_model_rows)]
    np.testing.assert_array_equal(np.stack(rows), med.jm_rows)
    assert np.frombuffer(formats.read_record(d / "TEST.MO", 0), np.int32)[0] == med.jmnum
    tab = np.frombuffer(formats.read_record(d / "TEST.MO", 1), np.float32).reshape(-1, 24)
    np.testing.assert_array_equal(tab, med.table.astype(np.float32))


def test_oracle_ascii_output_matches_the_writer(tmp_path):
    """The CPU baseline's per-level receiver output (the reference's
    OPEN/WRITE/CLOSE per receiver and level) writes the same lines as the
    drop-in host's seismogram writer."""
    from helpers import small_job
    from oracle.oracle import make_oracle
    cfg, med = small_job(nsteps=15, seed=12, n_rec=4)
    inp = job.prepare(cfg, med, "f32")
    a, b = make_oracle(inp), make_oracle(inp)
    opened = a.time_loop_ascii(1, 15, tmp_path)
    b.time_loop(1, 15)
    rec = b.receivers(1, 15)
    assert opened == 15 * 4 * 3
    for j in range(4):
        for stem, cols in (("REC_UW_", [0, 1, 2, 3]), ("REC_Q_", [4, 5, 6, 7]), ("REC_STRESS_", [8, 9])):
            text = (tmp_path / f"{stem}{j + 1}.asc").read_text().splitlines()
            assert text == formats.seismogram_lines(rec[:, j, :], inp.dt, 1, cols), (stem, j)
