"""The left-ventricle configuration on the GPU: tetrahedral shell, per-cell
conductivity tensor from the rule-based fibres and TNNP cell types by
transmural depth, with the Gauss-linear-corrected Laplacian (explicit
non-orthogonal and tangential-conductivity corrections every PIMPLE
corrector), through the C ABI against the oracle."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib, lv

LV_DIMS = (4, 8, 12)         # 6*4*(64 + 4*8*12) = 10752 tetrahedra
DT = 5e-5


@pytest.fixture(scope="module")
def small_lv():
    """A coarse LV (cells of about 2 mm): at ten times the configuration's
    conductivities the wave still propagates on it."""
    return lv.left_ventricle(*LV_DIMS, sigma_l=10 * lv.SIGMA_L, sigma_t=10 * lv.SIGMA_T)


def _boxes(L):
    lo, hi = L.apex_box(8e-3)
    return [(lo, hi, 0.0, 2e-3, 5e4)]


def _gpu(L, precision=lib.PRECISION_FP64, implicit=True, grad=lib.GRAD_LEAST_SQUARES,
         uncorrected=False, persistent=True, graph=True, dt=DT):
    g = api.Monodomain(L.mesh, "TNNP", "epicardialCells", dt=dt, precision=precision,
                       implicit=implicit, boxes=_boxes(L), tissue_per_cell=L.tissue,
                       conductivity_per_cell=L.conductivity, grad_scheme=grad,
                       laplacian_uncorrected=uncorrected, stencil=False)
    g.set_persistent(persistent)
    g.set_graph(graph)
    return g


def _oracle(oracle, L, implicit=True, grad=lib.GRAD_LEAST_SQUARES, uncorrected=False):
    d = oracle.tissue_desc("TNNP", 1, implicit=implicit, precond_dic=False, boxes=_boxes(L),
                           grad_gauss=grad == lib.GRAD_GAUSS_LINEAR, uncorrected=uncorrected)
    o = oracle.Tissue(d, oracle.Mesh.general(L.mesh))
    o.set_conductivity(L.conductivity)
    o.set_cell_tissue(L.tissue)
    return o


def _compare(g, o, nsteps, implicit=True, dt=DT):
    solves = []
    for _ in range(nsteps):
        g.step(dt)
        o.step(dt, 8)
        if implicit:
            solves.append((g.stats()[2], o.solves()[2]))
    vg, vo = g.vm(), o.vm()
    assert np.max(np.abs(vg - vo) / np.abs(vo)) < 1e-9
    ag, ao = g.activation(), o.activation()
    assert np.array_equal(ag > 0, ao > 0)
    assert (ag > 0).sum() > 0
    assert np.max(np.abs(ag - ao)) < 1e-9
    for gi, oi in solves:
        assert len(gi) == len(oi)
        assert np.max(np.abs(gi.astype(int) - oi.astype(int))) <= 1
    return vg


@pytest.mark.gpu
@pytest.mark.parametrize("persistent,graph", [(True, True), (False, True), (False, False)],
                         ids=["persistent", "graph", "host"])
def test_lv_fp64_matches_oracle(gpu_lib, oracle, small_lv, persistent, graph):
    g = _gpu(small_lv, persistent=persistent, graph=graph)
    o = _oracle(oracle, small_lv)
    _compare(g, o, 160)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("grad,uncorrected", [(lib.GRAD_GAUSS_LINEAR, False),
                                              (lib.GRAD_LEAST_SQUARES, True)],
                         ids=["gauss-linear", "uncorrected"])
def test_lv_fp64_schemes_match_oracle(gpu_lib, oracle, small_lv, grad, uncorrected):
    g = _gpu(small_lv, grad=grad, uncorrected=uncorrected)
    o = _oracle(oracle, small_lv, grad=grad, uncorrected=uncorrected)
    _compare(g, o, 100)
    g.close()


@pytest.mark.gpu
def test_lv_explicit_fp64_matches_oracle(gpu_lib, oracle, small_lv):
    g = _gpu(small_lv, implicit=False)
    o = _oracle(oracle, small_lv, implicit=False)
    _compare(g, o, 160, implicit=False)
    g.close()


@pytest.mark.gpu
def test_lv_correction_changes_the_solution(gpu_lib, small_lv):
    """On tetrahedra with rotated fibres the explicit correction is not a
    round-off term: dropping its non-orthogonal part moves Vm."""
    a, b = _gpu(small_lv), _gpu(small_lv, uncorrected=True)
    for _ in range(100):
        a.step(DT)
        b.step(DT)
    va, vb = a.vm(), b.vm()
    assert np.max(np.abs(va - vb)) > 1e-4
    a.close()
    b.close()


@pytest.mark.gpu
def test_lv_mixed_activation_error(gpu_lib, small_lv):
    """Mixed form against the FP64 form on the LV: activation times within
    0.05 ms."""
    runs = []
    for precision in (lib.PRECISION_FP64, lib.PRECISION_MIXED):
        g = _gpu(small_lv, precision=precision)
        for _ in range(400):
            g.step(DT)
        runs.append((g.activation(), g.vm()))
        g.close()
    (a0, v0), (a1, v1) = runs
    assert np.array_equal(a0 > 0, a1 > 0) and (a0 > 0).sum() > 100
    assert np.max(np.abs(a0 - a1)) <= 5e-5
