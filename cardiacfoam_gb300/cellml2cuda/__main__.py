"""Regenerate the CUDA and oracle forms of the ionic models.

    python -m cardiacfoam_gb300.cellml2cuda --ionic-models <cardiacFoam>/src/ionicModels

reads each ``<Model>_<Year>.H`` that cellML2foam produced and writes
``cardiacfoam_gb300/csrc/models/<model>.cuh`` and ``oracle/models/<model>.h``,
and for the models of ``ADJOINT_MODELS`` the reverse-mode derivative of the
right-hand side, ``cardiacfoam_gb300/csrc/models/<model>_adjoint.cuh``.
"""
import argparse
from pathlib import Path

import json

from .adjoint import emit_adjoint_header
from .emit import TISSUE_FLAGS, emit_c, emit_cuda, ident
from .model import WRAPPERS, load_model
from .opcount import count_rhs

REPO = Path(__file__).resolve().parents[2]
# models whose right-hand side is differentiated for the adjoint step
ADJOINT_MODELS = ["TNNP"]


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ionic-models", required=True,
                    help="cardiacFoam src/ionicModels directory")
    ap.add_argument("--models", nargs="*", default=list(WRAPPERS))
    args = ap.parse_args(argv)
    cu_dir = REPO / "cardiacfoam_gb300" / "csrc" / "models"
    c_dir = REPO / "oracle" / "models"
    cu_dir.mkdir(parents=True, exist_ok=True)
    c_dir.mkdir(parents=True, exist_ok=True)
    counts = {}
    for name in args.models:
        m = load_model(args.ionic_models, name)
        tissue = TISSUE_FLAGS[m.tissues[0]]
        counts[name] = count_rhs(m, tissue)
        rel = f"src/ionicModels/{WRAPPERS[name]['dir']}/{WRAPPERS[name]['header']}"
        (cu_dir / f"{ident(name)}.cuh").write_text(emit_cuda(m, rel))
        (c_dir / f"{ident(name)}.h").write_text(emit_c(m, rel))
        if name in ADJOINT_MODELS:
            (cu_dir / f"{ident(name)}_adjoint.cuh").write_text(emit_adjoint_header(m, rel))
        print(f"{name}: {len(m.states)} states, {len(m.algebraic)} algebraic, "
              f"{len(m.constants)} constants, {counts[name]['flops']:.0f} flops + "
              f"{counts[name]['transcendental']:.0f} transcendentals per RHS")
    (cu_dir / "opcounts.json").write_text(json.dumps(counts, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
