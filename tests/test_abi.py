"""The C ABI library: loads without a GPU, exports every declared symbol,
and rejects invalid descriptions before touching the device."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    txt = (ROOT / "include" / "cardiac_gpu.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cfg_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(gpu_lib):
    names = declared_functions()
    assert set(names) == set(lib.EXPORTS)
    for n in names:
        assert hasattr(gpu_lib, n), n


def _desc(**kw):
    kw.setdefault("model", "TNNP")
    kw.setdefault("tissue", "epicardialCells")
    return api.ionic_desc(kw["model"], kw["tissue"], 8, 1e-5)


@pytest.mark.parametrize("model,tissue,code", [
    ("NoSuchModel", "epicardialCells", lib.CFG_ERR_INVALID),
    ("ORd", "epicardialCells", lib.CFG_ERR_INVALID),      # ORd accepts myocyte only
    ("TNNP", "myocyte", lib.CFG_ERR_INVALID),
    ("TNNP", "", lib.CFG_ERR_INVALID),
])
def test_ionic_selection_errors(gpu_lib, model, tissue, code):
    d = api.ionic_desc(model, tissue, 8, 1e-5)
    if not tissue:
        d.tissue = None
    h = C.c_void_p()
    rc = gpu_lib.cfg_ionic_create(C.byref(d), C.byref(h))
    assert rc == code
    assert gpu_lib.cfg_last_error().decode()


def test_unsupported_solver(gpu_lib):
    d = api.ionic_desc("TNNP", "epicardialCells", 8, 1e-5, ode=api.ode_desc(solver="Rosenbrock34"))
    h = C.c_void_p()
    assert gpu_lib.cfg_ionic_create(C.byref(d), C.byref(h)) == lib.CFG_ERR_UNSUPPORTED


DICT = """
FoamFile { version 2.0; format ascii; class dictionary; object electroProperties; }
myocardiumSolver  %s;
monodomainSolverCoeffs
{
    conductivity [-1 -3 3 0 0 2 0] (0.1334 0 0 0.0176 0 0.0176);
    chi   [0 -1 0 0 0 0 0] 140000;   // surface-to-volume ratio
    cm    [-1 -4 4 0 0 2 0] 0.01;
    ionicModel    %s;
    tissue    epicardialCells;
    solver RKF45;
    /* stimulus */
    externalStimulus
    {
        stimulusLocationMin (0 0 0);
        stimulusLocationMax (1.5e-3 1.5e-3 1.5e-3);
        stimulusDuration [0 0 1 0 0 0 0] 2e-3;
        stimulusIntensity [0 -3 0 0 0 1 0] 50000;
    }
}
"""


def _create_from_dict(gpu_lib, text):
    from cardiacfoam_gb300.mesh import box_mesh
    m = box_mesh(4, 3, 2, 4e-3, 3e-3, 2e-3)
    md, keep = api.mesh_desc(m)
    h = C.c_void_p()
    return gpu_lib.cfg_monodomain_create_from_dict(text.encode(), C.byref(md), 1e-5, 0, C.byref(h))


def test_dictionary_selection_errors(gpu_lib):
    assert _create_from_dict(gpu_lib, DICT % ("bidomainSolver", "TNNP")) == lib.CFG_ERR_UNSUPPORTED
    assert _create_from_dict(gpu_lib, DICT % ("monodomainSolver", "Nope")) == lib.CFG_ERR_INVALID
    assert "Unknown ionicModel" in gpu_lib.cfg_last_error().decode()
    assert _create_from_dict(gpu_lib, "myocardiumSolver monodomainSolver;") == lib.CFG_ERR_INVALID
