"""Output formats: the OpenFOAM ASCII volScalarField writer and the
single-cell trace file (name, header and row formatting against the
reference's own trace file, read as text)."""
import numpy as np

from cardiacfoam_gb300 import api, io
from pathlib import Path

GOLDEN = Path(__file__).parent / "golden"


def test_time_name_like_openfoam():
    assert io.time_name(0.01) == "0.01"
    assert io.time_name(0.0001) == "0.0001"
    assert io.time_name(1e-05) == "1e-05"
    assert io.time_name(0.05) == "0.05"
    assert io.time_name(1.0) == "1"


def test_vol_scalar_field_roundtrip(tmp_path):
    v = np.array([-0.084, -0.0839999, 0.0123456789, 1e-7])
    p = tmp_path / "0.01" / "Vm"
    io.write_vol_scalar_field(p, "Vm", v, io.DIM_VM, "0.01",
                              patches=[("left", "zeroGradient"), ("right", "zeroGradient")])
    text = p.read_text()
    assert "class       volScalarField;" in text and "object      Vm;" in text
    assert 'location    "0.01";' in text and "dimensions      [1 2 -3 0 0 -1 0];" in text
    body = text.split("nonuniform List<scalar>")[1].split("(", 1)[1].split(")", 1)[0].split()
    assert np.allclose([float(x) for x in body], v, rtol=1e-5, atol=0)   # 6 digits
    assert "left" in text and "right" in text and text.count("zeroGradient") == 2
    io.write_vol_scalar_field(tmp_path / "u", "Vm", np.full(5, -0.084), io.DIM_VM, "0")
    assert "internalField   uniform -0.084;" in (tmp_path / "u").read_text()


def test_trace_file_name_and_protocol_suffix():
    s = api.stimulus_desc(20, 1000, 1, 0.4, 3)
    assert io.trace_file_name("AlievPanfilov", "myocyte", s) == "AlievPanfilov_myocyte_S1_1000.txt"
    assert io.protocol_suffix(0.0, 0) == "noStim"
    assert io.protocol_suffix(600.0, 8, 300.0, 1) == "S1_600_S2_300"


def test_row_format_matches_the_reference_trace():
    """The reference's AlievPanfilov trace (time and Vm, fixed 7 decimals)
    reproduced from its values by the same formatting the library uses."""
    g = np.load(GOLDEN / "aliev_panfilov_singlecell.npz")
    vm = g["vm_1e7"].astype(np.int64)
    dt = 5e-5
    # the first reference rows, as text: "0.0000500 -75.0073648"
    for k, expect in ((0, "0.0000500 -75.0073648"), (1, "0.0001000 -75.0147304")):
        t = (k + 1) * dt
        assert f"{t:.7f} {vm[k] * 1e-7:.7f}" == expect
