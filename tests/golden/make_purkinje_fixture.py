"""Generate niederer_purkinje_graph.npz from the reference's Purkinje tutorial.

Run where a cardiacFoam checkout is available ($CARDIACFOAM_REFERENCE, or the
location oracle/build.py knows):

    python tests/golden/make_purkinje_fixture.py

reads tutorials/Niederer/NiedererEtAl2011MonodomainPurkinje/constant/
purkinjeGraph (the graphFile of that tutorial's purkinjeGraphModel) with this
package's graph reader and stores its conduction edges (node a, node b,
length, conductance), root node, PVJ nodes and PVJ locations.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from cardiacfoam_gb300 import io  # noqa: E402
from oracle.build import reference_dir  # noqa: E402

GRAPH = "tutorials/Niederer/NiedererEtAl2011MonodomainPurkinje/constant/purkinjeGraph"

if __name__ == "__main__":
    ref = reference_dir()
    if ref is None:
        sys.exit("no cardiacFoam checkout found: set CARDIACFOAM_REFERENCE")
    g = io.read_purkinje_graph((Path(ref) / GRAPH).read_text())
    np.savez_compressed(HERE / "niederer_purkinje_graph.npz", edges=g["edges"],
                        root=np.int64(g["root"]), pvj_nodes=g["pvj_nodes"],
                        pvj_locations=g["pvj_locations"])
    print(f"{len(g['edges'])} edges, {len(g['pvj_nodes'])} PVJs")
