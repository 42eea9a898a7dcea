"""The reference's NiedererEtAl2012 regression case
(tutorials/regressionTests/NiedererEtAl2012): its mesh, stimulus, probes and
pinned activation times, shared by the oracle pin and the GPU pin."""
import json
from pathlib import Path

from cardiacfoam_gb300 import mesh as M

GOLDEN = Path(__file__).parent / "golden"

# system/blockMeshDict:17-51: one block (100 15 35) over (20 3 7) x scale
# 0.001; the walls patch lists the block faces (3 7 6 2) (0 4 7 3) (2 6 5 1)
# (1 5 4 0) (0 3 2 1) (4 5 6 7)
BLOCK = dict(ni=100, nj=15, nk=35, extent=(20.0, 3.0, 7.0), scale=1e-3,
             patch_order=("y-max", "x-min", "x-max", "y-min", "z-min", "z-max"))
LENGTHS = tuple(e * BLOCK["scale"] for e in BLOCK["extent"])
SIGMA = (0.1334177215, 0, 0, 0.01760617761, 0, 0.01760617761)
CHI_CM = 140000 * 0.01
# constant/electroProperties: externalStimulus
BOX = ((0, 0, 5.5e-3), (1.5e-3, 1.5e-3, 7e-3))
STIMULUS = (0.0, 2e-3, 5e4)
END_TIME = 0.04
# system/Niedererpoints: probeLocations
PROBES = [(0, 0, 0.007), (0, 0, 0), (0.019999, 0, 0.007), (0.019999, 0, 0), (0, 0.003, 0.007),
          (0, 0.003, 0), (0.019999, 0.003, 0.007), (0.019999, 0.003, 0),
          (0.01, 0.0015, 0.0035)]


def explicit_dt(max_co=0.1):
    """electroModel::setDeltaT -> MyocardiumDomain::suggestExplicitDeltaT."""
    n = (BLOCK["ni"], BLOCK["nj"], BLOCK["nk"])
    dx = [LENGTHS[d] / n[d] for d in range(3)]
    return max_co * min(dx[d] ** 2 / (SIGMA[(0, 3, 5)[d]] / CHI_CM) for d in range(3))


def openfoam_mesh(oracle, contract):
    """The case's mesh with its full geometry and the cell centres OpenFOAM's
    geometry code computes for it (with the given fma contractions)."""
    b = BLOCK
    m = M.with_box_geometry(M.box_mesh(b["ni"], b["nj"], b["nk"], *LENGTHS), *LENGTHS)
    m.centres = oracle.blockmesh_centres(b["ni"], b["nj"], b["nk"], b["extent"], b["scale"],
                                         b["patch_order"], contract)
    return m


def probe_cell(p):
    """The cell holding a probe location (the corner cells at the walls)."""
    n = (BLOCK["ni"], BLOCK["nj"], BLOCK["nk"])
    i, j, k = (min(int(p[d] / (LENGTHS[d] / n[d])), n[d] - 1) for d in range(3))
    return (k * n[1] + j) * n[0] + i


def pins():
    """NiedererEtAl2012.reference:8-13 as (probe index, activation, tolerance)."""
    pts = json.loads((GOLDEN / "regression_pins.json").read_text())["NiedererEtAl2012"]["points"]
    return [(p["column"] - 2, p["activation"], p["tol"]) for p in pts]
