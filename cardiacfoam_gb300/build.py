"""Build libcardiac_gpu.so in-tree for sm_103a (GB300).

Each ionic model is compiled twice from ``csrc/ionic_instance.cu``: the plain
form with ``--fmad=false`` (FP64 rounding in the host's evaluation order) and
the mixed form with FMA contraction.  Translation units are compiled in
parallel; only changed ones are rebuilt.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcardiac_gpu.so"
INCLUDE = PKG.parent / "include"

MODELS = ["tnnp", "ord", "torord_dyncl", "alievpanfilov", "buenoorovio",
          "monodomainfdamanufactured", "bidomainfdamanufactured"]
# per-model unroll factor of the per-state loops around the right-hand side
# (measured on GB300: ORd fastest at 4, the others at 1)
STATE_UNROLL = {"ord": 4}
# resident blocks of 64 per SM the mixed kernel is built for, where the
# model's registers (right-hand side plus the state held in registers) and
# not its shared-memory slice set the limit: TNNP at 8 (128 registers)
MIXED_MIN_BLOCKS = {"tnnp": 8}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC), "-I", str(INCLUDE)]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return cand


def _units():
    units = []
    # register budget of the ionic kernels: resident 128-thread blocks per SM
    mb = os.environ.get("CFG_IONIC_MIN_BLOCKS")
    ionic_extra = [f"-DCFG_IONIC_MIN_BLOCKS={int(mb)}"] if mb else []
    unroll = os.environ.get("CFG_IONIC_STATE_UNROLL")
    if unroll:
        ionic_extra.append(f"-DCFG_IONIC_STATE_UNROLL={int(unroll)}")
    for m in MODELS:
        for prec, flags in (("fp64", ["--fmad=false", "-DCFG_FP64=1"]),
                            ("mixed", ["--use_fast_math", "-DCFG_FP64=0"])):
            extra = list(ionic_extra)
            if not unroll and m in STATE_UNROLL:
                extra.append(f"-DCFG_IONIC_STATE_UNROLL={STATE_UNROLL[m]}")
            if prec == "mixed" and m in MIXED_MIN_BLOCKS:
                extra.append(f"-DCFG_MIXED_MIN_BLOCKS={MIXED_MIN_BLOCKS[m]}")
            units.append((f"ionic_{m}_{prec}", CSRC / "ionic_instance.cu",
                          flags + [f"-DCFG_MODEL={m}"] + extra))
    units.append(("ionic_registry", CSRC / "ionic_registry.cu", []))
    units.append(("ionic", CSRC / "ionic.cu", []))
    units.append(("batch", CSRC / "batch.cu", []))
    units.append(("diffusion", CSRC / "diffusion.cu", []))
    units.append(("monodomain", CSRC / "monodomain.cu", []))
    units.append(("diffusion_coop", CSRC / "diffusion_coop.cu", []))
    units.append(("step_graph", CSRC / "step_graph.cu", []))
    units.append(("noalloc", CSRC / "noalloc.cu", []))
    units.append(("dictionary", CSRC / "dictionary.cpp", []))
    units.append(("geometry", CSRC / "geometry.cpp", []))
    # staged pseudo-ECG launch shape: cells per tile, blocks per SM
    ecg_extra = [f"-D{k}={int(os.environ[k])}" for k in ("CFG_ECG_TILE", "CFG_ECG_STAGED_PER_SM")
                 if os.environ.get(k)]
    units.append(("ecg", CSRC / "ecg.cu", ecg_extra))
    units.append(("bidomain", CSRC / "bidomain.cu", []))
    units.append(("purkinje", CSRC / "purkinje.cu", []))
    units.append(("adjoint", CSRC / "adjoint.cu", ["--use_fast_math"]))
    return units


def _deps_hash(src: Path, flags) -> str:
    h = hashlib.sha256()
    h.update(" ".join(ARCH + COMMON + list(flags)).encode())
    for p in sorted(list(CSRC.rglob("*.cu")) + list(CSRC.rglob("*.cuh")) +
                    list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cpp")) +
                    list(INCLUDE.glob("*.h"))):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    units = _units()

    def compile_unit(u):
        name, src, flags = u
        obj = BUILD / f"{name}.o"
        stamp = BUILD / f"{name}.hash"
        digest = _deps_hash(src, flags)
        if not force and obj.exists() and stamp.exists() and stamp.read_text() == digest:
            return name, False
        cmd = [cc, *ARCH, *COMMON, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr[-6000:]}")
        stamp.write_text(digest)
        return name, True

    jobs = jobs or max(1, min(len(units), os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(compile_unit, units))
    rebuilt = any(r for _, r in results)
    if rebuilt or force or not LIB.exists():
        objs = [str(BUILD / f"{n}.o") for n, _, _ in units]
        tmp = str(LIB) + ".tmp"
        cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
