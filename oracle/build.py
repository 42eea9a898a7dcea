"""Build recipe for the oracle (test infrastructure only).

``build()`` compiles oracle.c (and the generated models) into
``oracle/_build/liboracle.so`` with ``-ffp-contract=off`` so that x86-64 and
aarch64 hosts round identically.  ``build_ref()`` runs ``ref/build_ref.sh`` when
a cardiacFoam checkout is available, producing ``oracle/_ref/libref_models.so``
from the reference's own generated ionic-model headers.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_models.so"


def reference_dir() -> Path | None:
    """The cardiacFoam checkout this recipe reads: $CARDIACFOAM_REFERENCE, else
    the build container's read-only mount.  None where neither exists (the
    GPU host, a user's machine): then nothing that needs the reference runs."""
    env = os.environ.get("CARDIACFOAM_REFERENCE")
    for cand in ([Path(env)] if env else []) + [Path("/root/reference")]:
        if (cand / "src" / "ionicModels").is_dir():
            return cand
    return None


def _sources():
    return [HERE / "oracle.c", HERE / "oracle.h", HERE / "oracle_common.h",
            *sorted((HERE / "models").glob("*.h"))]


def build(force: bool = False) -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if not force and LIB.exists():
        mt = LIB.stat().st_mtime
        if all(s.stat().st_mtime <= mt for s in _sources()):
            return LIB
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-ffp-contract=off", "-fPIC", "-shared",
           "-fopenmp", "-o", str(LIB) + ".tmp", str(HERE / "oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


def build_ref(reference: Path | None = None) -> Path | None:
    """Compile the reference's generated model headers, if the reference exists."""
    reference = reference or reference_dir()
    if reference is None or not (reference / "src" / "ionicModels").is_dir():
        return None
    subprocess.run(["sh", str(HERE / "ref" / "build_ref.sh"), str(reference)], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_LIB
