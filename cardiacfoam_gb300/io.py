"""Output in the reference's formats.

* OpenFOAM ASCII ``volScalarField`` files of the myocardium fields at write
  times (what ``runTime.write()`` produces for ``Vm`` and ``activationTime``
  in ``MyocardiumDomain``: ``<case>/<timeName>/<field>``), so a GPU run can be
  diffed against an OpenFOAM case or read by its post-processing.
* The single-cell trace of ``SingleCellSolver`` (``ionicModelIO::write``):
  ``postProcessing/<model>_<tissue>_<protocol>.txt`` with a ``time <names>``
  header and fixed 7-decimal rows; the rows are formatted by the library
  (``cfg_ionic_trace_row``).
* The pseudo-ECG time series of ``ECGDomain`` (``ecgModelIO::openTimeSeries``
  / ``writeRow``): ``postProcessing/pseudoECG.dat`` with a ``# time <names>``
  header and rows in scientific notation with 8 decimals.
"""
from __future__ import annotations

import os
from pathlib import Path
from typing import Iterable, Optional, Sequence, Tuple

import numpy as np

DIM_VM = "[1 2 -3 0 0 -1 0]"          # V = kg m^2 s^-3 A^-1
DIM_TIME = "[0 0 1 0 0 0 0]"


def time_name(t: float, precision: int = 6) -> str:
    """Time::timeName: the value in general format with `precision`
    significant digits (controlDict timePrecision, default 6)."""
    return f"{t:.{precision}g}"


def _scalar(v: float, precision: int) -> str:
    return f"{v:.{precision}g}"


def write_vol_scalar_field(path, name: str, values: np.ndarray, dimensions: str,
                           location: str, patches: Sequence[Tuple[str, str]] = (("walls",
                                                                                  "zeroGradient"),),
                           precision: int = 6):
    """One ASCII volScalarField file (uniform when every value is equal);
    each patch gets `type <t>;` (zeroGradient for the myocardium fields,
    myocardiumDomain.C:207)."""
    v = np.asarray(values, dtype=np.float64).ravel()
    L = ["/*--------------------------------*- C++ -*----------------------------------*\\",
         "  written by cardiacfoam_gb300",
         "\\*---------------------------------------------------------------------------*/",
         "FoamFile", "{", "    version     2.0;", "    format      ascii;",
         "    class       volScalarField;", f'    location    "{location}";',
         f"    object      {name};", "}",
         "// * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * //",
         "", f"dimensions      {dimensions};", ""]
    if v.size and np.all(v == v[0]):
        L.append(f"internalField   uniform {_scalar(v[0], precision)};")
    else:
        L.append("internalField   nonuniform List<scalar> ")
        L.append(str(v.size))
        L.append("(")
        L.extend(_scalar(x, precision) for x in v)
        L.append(")")
        L.append(";")
    L += ["", "boundaryField", "{"]
    for pname, ptype in patches:
        L += [f"    {pname}", "    {", f"        type            {ptype};", "    }"]
    L += ["}", "", "", "// " + "*" * 73 + " //", ""]
    Path(path).parent.mkdir(parents=True, exist_ok=True)
    Path(path).write_text("\n".join(L))


def write_monodomain_fields(md, case_dir, patches=(("walls", "zeroGradient"),),
                            precision: int = 6, time_precision: int = 6):
    """Vm and activationTime of a Monodomain context at its current time."""
    t = md.time()
    tn = time_name(t, time_precision)
    d = Path(case_dir) / tn
    write_vol_scalar_field(d / "Vm", "Vm", md.vm(), DIM_VM, tn, patches, precision)
    write_vol_scalar_field(d / "activationTime", "activationTime", md.activation(), DIM_TIME,
                           tn, patches, precision)
    return d


def protocol_suffix(stim_period_s1: float, nstim1: int, stim_period_s2: float = 0.0,
                    nstim2: int = 0) -> str:
    """stimulusIO::protocolSuffix (stimulusIO.C:392-423): noStim, S1_<s1> or
    S1_<s1>_S2_<s2> (Foam::name: general format, 6 digits)."""
    small = 1e-15
    if stim_period_s1 <= small or nstim1 <= 0:
        return "noStim"
    out = f"S1_{stim_period_s1:.6g}"
    if nstim2 > 0:
        out += f"_S2_{stim_period_s2:.6g}"
    return out


def trace_file_name(model: str, tissue: str, stim) -> str:
    """<ionicModel type>_<tissueName>_<protocol>.txt (singleCellSolver.C:100-112)."""
    return f"{model}_{tissue}_{protocol_suffix(stim.stim_period_s1, stim.nstim1, stim.stim_period_s2, stim.nstim2)}.txt"


class SingleCellTrace:
    """SingleCellSolver's output file for an IonicModel: the header on
    creation, one row per write(t) for integration point `cell`."""

    def __init__(self, ionic, path, columns: Optional[Iterable[str]] = None, cell: int = 0):
        self.ionic = ionic
        self.cell = cell
        self.columns = " ".join(columns) if columns else None
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        self.fh = open(path, "w")
        self.fh.write(ionic.trace_header(self.columns))

    def write(self, t: float):
        self.fh.write(self.ionic.trace_row(self.cell, t, self.columns))

    def close(self):
        if self.fh:
            self.fh.close()
            self.fh = None


def ecg_header(names: Sequence[str]) -> str:
    """ecgModelIO::openTimeSeries (ecgModelIO.C:30-52): '# time' and the
    electrode names, two spaces apart."""
    return "# time" + "".join("  " + n for n in names) + "\n"


def ecg_row(t: float, values: Sequence[float]) -> str:
    """ecgModelIO::writeRow (ecgModelIO.C:55-68) on the scientific,
    precision-8 stream."""
    return f"{t:.8e}" + "".join(f"  {v:.8e}" for v in values) + "\n"


def write_pseudo_ecg(case_dir, names: Sequence[str], times: Sequence[float], values,
                     file_name: str = "pseudoECG.dat") -> Path:
    """<case>/postProcessing/pseudoECG.dat with the given rows (ECGDomain
    writes the rows of output times, ecgDomain.C:167-190)."""
    out = Path(case_dir) / "postProcessing"
    out.mkdir(parents=True, exist_ok=True)
    path = out / file_name
    v = np.asarray(values, dtype=np.float64).reshape(len(times), len(names))
    with open(path, "w") as fh:
        fh.write(ecg_header(names))
        for t, row in zip(times, v):
            fh.write(ecg_row(float(t), row))
    return path


def read_purkinje_graph(text: str) -> dict:
    """The conduction graph file a purkinjeGraphModel names (graphFile, read by
    conductionSystemDomain.C:100-165 and conductionGraph::readFromDict):
    ``rootNode``, ``pvjNodes N(...)``, ``pvjLocations N((x y z) ...)`` and
    ``conductionEdges N(4(a b length conductance) ...)`` in OpenFOAM list
    syntax (the size prefixes are optional).  Returns edges [n][4], root,
    pvj_nodes and pvj_locations [n][3]."""
    import re
    body = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    body = re.sub(r"//[^\n]*", " ", body)
    body = re.sub(r"FoamFile\s*\{[^}]*\}", " ", body)

    def entry(key):
        m = re.search(r"\b" + key + r"\b\s*(.*?);", body, flags=re.S)
        if not m:
            raise ValueError(f"keyword {key} is undefined")
        return m.group(1)

    def numbers(s):
        # drop OpenFOAM list-size prefixes: an integer directly before "("
        s = re.sub(r"\b\d+\s*\(", "(", s)
        return [float(v) for v in re.findall(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?", s)]

    out = {"root": int(numbers(entry("rootNode"))[0]) if re.search(r"\brootNode\b", body) else 0}
    e = numbers(entry("conductionEdges"))
    if len(e) % 4:
        raise ValueError("each entry in 'conductionEdges' must have 4 values: "
                         "(nodeA nodeB length conductance)")
    out["edges"] = np.array(e, dtype=np.float64).reshape(-1, 4)
    if re.search(r"\bpvjNodes\b", body):
        out["pvj_nodes"] = np.array(numbers(entry("pvjNodes")), dtype=np.int64)
        loc = numbers(entry("pvjLocations"))
        out["pvj_locations"] = np.array(loc, dtype=np.float64).reshape(-1, 3)
        if len(out["pvj_locations"]) != len(out["pvj_nodes"]):
            raise ValueError("pvjNodes and pvjLocations differ in length")
    else:
        out["pvj_nodes"] = np.zeros(0, dtype=np.int64)
        out["pvj_locations"] = np.zeros((0, 3))
    return out


def synthetic_purkinje_tree(depth: int, segment: int, h: float, origin=(0.0, 0.0, 0.0),
                            spread=(1.0, 0.0, 0.0), conductance: float = 1.0, seed: int = 0):
    """A binary branching network for tests and benchmarks: a trunk of
    `segment` edges of length h from node 0, then at every branch point two
    branches of `segment` edges, `depth` generations deep; branches turn by a
    seeded angle in the x-y plane.  Returns (edges [n][4], node positions
    [n][3], leaf nodes)."""
    rng = np.random.default_rng(seed)
    pos = [np.array(origin, dtype=np.float64)]
    edges = []
    d0 = np.array(spread, dtype=np.float64)
    d0 /= np.linalg.norm(d0)

    def grow(start, direction, k):
        prev = start
        for _ in range(k):
            pos.append(pos[prev] + h * direction)
            edges.append((prev, len(pos) - 1, h, conductance))
            prev = len(pos) - 1
        return prev

    tips = [(grow(0, d0, segment), d0)]
    for _ in range(depth):
        nxt = []
        for node, d in tips:
            for sgn in (-1.0, 1.0):
                a = sgn * rng.uniform(0.3, 0.8)
                rot = np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0],
                                [0.0, 0.0, 1.0]])
                nd = rot @ d
                nxt.append((grow(node, nd, segment), nd))
        tips = nxt
    return np.array(edges, dtype=np.float64), np.array(pos), np.array([t for t, _ in tips])
