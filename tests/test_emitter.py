"""cellML2foam-to-CUDA emitter: parser units and reproducibility."""
from pathlib import Path

import pytest

from cardiacfoam_gb300.cellml2cuda import cexpr
from cardiacfoam_gb300.cellml2cuda.emit import emit_c, emit_cuda
from cardiacfoam_gb300.cellml2cuda.model import WRAPPERS, load_model, use_before_def
from oracle.build import reference_dir

ROOT = Path(__file__).resolve().parents[1]
_REF = reference_dir()
REF = (_REF / "src" / "ionicModels") if _REF is not None else None


def test_parser_precedence():
    e = cexpr.parse_expr("- 56.86 - STATES[V] / 2.0 * x")
    assert isinstance(e, cexpr.Bin) and e.op == "-"
    assert isinstance(e.l, cexpr.Unary)
    c = cexpr.parse_expr("a < - 40.0 ? 1.0 : b == 2 ? 3 : 4")
    assert isinstance(c, cexpr.Cond) and isinstance(c.b, cexpr.Cond)
    p = cexpr.parse_expr("pow(STATES[Ca_i] / 0.000325, 8.00000)")
    assert isinstance(p, cexpr.Call) and p.fn == "pow"
    with pytest.raises(cexpr.ParseError):
        cexpr.parse_expr("a ^ b")


def test_generated_files_present():
    for name in WRAPPERS:
        key = name.lower()
        assert (ROOT / "cardiacfoam_gb300" / "csrc" / "models" / f"{key}.cuh").exists()
        assert (ROOT / "oracle" / "models" / f"{key}.h").exists()


@pytest.mark.skipif(REF is None, reason="no cardiacFoam checkout: set CARDIACFOAM_REFERENCE")
@pytest.mark.parametrize("name", list(WRAPPERS))
def test_regeneration_is_identical(name):
    m = load_model(REF, name)
    rel = f"src/ionicModels/{WRAPPERS[name]['dir']}/{WRAPPERS[name]['header']}"
    key = name.lower()
    assert emit_cuda(m, rel) == (ROOT / "cardiacfoam_gb300/csrc/models" / f"{key}.cuh").read_text()
    assert emit_c(m, rel) == (ROOT / "oracle/models" / f"{key}.h").read_text()


@pytest.mark.skipif(REF is None, reason="no cardiacFoam checkout: set CARDIACFOAM_REFERENCE")
def test_use_before_def_is_only_istim():
    for name in WRAPPERS:
        m = load_model(REF, name)
        assert set(use_before_def(m.rates)) <= {"Istim"}


@pytest.mark.skipif(REF is None, reason="no cardiacFoam checkout: set CARDIACFOAM_REFERENCE")
def test_supplement_covers_exactly_the_unassigned_constants():
    from cardiacfoam_gb300.cellml2cuda.emit import SUPPLEMENT, supplement_for, unassigned_constants
    for name in WRAPPERS:
        m = load_model(REF, name)
        sup = supplement_for(m)          # raises on any mismatch
        assert [c for c, _ in sup] == [c for c, _ in SUPPLEMENT.get(name, [])]
        assert (len(unassigned_constants(m)) > 0) == (name == "ORd")


def test_reciprocal_slots_are_read_only_as_divisors():
    """The tissue form stores cfg_hrcp(v) in the per-step slots that the
    stage body reads only as divisors, and reads exactly those through
    cfg_hdiv: every slot that holds a reciprocal is read nowhere else, so
    the FP64 form (where cfg_hrcp is the identity and cfg_hdiv a division)
    is unchanged and the mixed form multiplies by the reciprocal."""
    import re
    n_recip = 0
    for name in WRAPPERS:
        text = (ROOT / "cardiacfoam_gb300" / "csrc" / "models" / f"{name.lower()}.cuh").read_text()
        if "rhs_tissue" not in text or "constexpr int NH = 0;" in text:
            continue
        hoist = text[text.index("void hoist("):text.index("R rhs_tissue(")]
        body = text[text.index("R rhs_tissue("):]
        body = body[:body.index("\n}\n")]
        stored = set(re.findall(r"H\[([^\]]+)\] = cfg_hrcp\(", hoist))
        divisors = set(re.findall(r"cfg_hdiv\([^;]*?, H\(([^)]+)\)\)", body))
        assert stored == divisors, name
        reads = re.findall(r"H\(([^)]+)\)", body)
        div_reads = len(re.findall(r"cfg_hdiv\(", body))
        other = [r for r in reads if r in stored]
        assert len(other) == div_reads, name     # every read of such a slot is a divisor
        n_recip += len(stored)
    assert n_recip > 0
