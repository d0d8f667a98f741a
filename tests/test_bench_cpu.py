"""The measurement code of bench.py on the CPU: the algorithmic byte counts
behind the roofline figures and the clock-sample summary."""
from types import SimpleNamespace

import pytest


def _inp(mx=2048, mz=2048, tpml=20, lin_z=12):
    return SimpleNamespace(nx=mx + 2 * tpml, nz=mz + tpml + 1, tpml=tpml, lin_z=lin_z,
                           cells=(mx + 2 * tpml) * (mz + tpml + 1))


@pytest.mark.parametrize("s,per_cell", [(4, 68), (8, 136)])
def test_core_bytes_per_cell(s, per_cell):
    import bench
    inp = _inp()
    medium = {"mode": "biot", "planes_stress": 5, "planes_velocity": 5}
    core = {"stress": (5, 2045, 5, 2047), "velocity": (5, 2045, 2, 2047)}
    b = bench.algorithmic_bytes(inp, s, medium, core)
    ns = (2045 - 5) * (2047 - 5) - (2045 - 5)  # the source row is not a core row
    nv = (2045 - 5) * (2047 - 2)
    assert b["core_cells"] == {"stress": ns, "velocity": nv}
    assert b["stress_core"] == ns * per_cell and b["velocity_core"] == nv * per_cell
    # a whole phase adds the PML memory variables and (velocity) the bottom history
    assert b["stress"] > inp.cells * per_cell and b["velocity"] > b["stress"]


def test_table_mode_reads_one_index_per_cell():
    import bench
    inp = _inp(mx=100, mz=80, tpml=5)
    b = bench.algorithmic_bytes(inp, 4, {"mode": "table", "planes_stress": 0, "planes_velocity": 0})
    mem = b["stress"] - inp.cells * (12 * 4 + 4)
    assert mem > 0 and mem % 8 == 0  # memory variables: read and written, 4 bytes each


def test_clock_summary_flags_throttling():
    import bench
    c = bench.ClockSampler(0)
    c.lines = ["2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
               "2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    s = c.summary()
    assert s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    assert s["sm_mhz"] == 2070.0
