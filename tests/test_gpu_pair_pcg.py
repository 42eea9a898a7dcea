"""The persistent implicit solve with its PCG in float pairs (the default of
the mixed form: operator, vectors and sums as (hi, lo) float pairs on the
FP32 pipe) through the C ABI: against the oracle with the FP64 ionic form,
and against the FP64 PCG of the same mixed context on a propagating slab and
on the tetrahedral LV."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib, lv
from cardiacfoam_gb300.mesh import box_mesh

SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
BOX = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, 1.5e-3), 0.0, 2e-3, 5e4)]


def _slab(dims, h, dt, precision, stencil=True, arithmetic=None):
    mesh = box_mesh(*dims, dims[0] * h, dims[1] * h, dims[2] * h)
    g = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, precision=precision,
                       boxes=BOX, stencil=stencil)
    if arithmetic is not None:
        g.set_pcg_arithmetic(arithmetic)
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("stencil", [True, False], ids=["stencil", "ell"])
def test_float_pair_pcg_matches_oracle(gpu_lib, oracle, stencil):
    """FP64 ionic update, float-pair PCG: the oracle's step (same diagonal
    preconditioner) within the FP64 tests' bounds, PCG iterations within
    one of the oracle's."""
    dims, h, dt, nsteps = (20, 7, 3), 1e-3, 1e-5, 300
    g = _slab(dims, h, dt, lib.PRECISION_FP64, stencil, lib.PCG_FLOAT_PAIRS)
    om = oracle.Mesh(*dims, dims[0] * h, dims[1] * h, dims[2] * h)
    o = oracle.Tissue(oracle.tissue_desc("TNNP", api.TISSUE_FLAGS["epicardialCells"], SIGMA,
                                         implicit=True, precond_dic=False, boxes=BOX), om)
    for _ in range(nsteps):
        g.step(dt)
        o.step(dt, 4)
        gi, oi = g.stats()[2], o.solves()[2]
        assert len(gi) == len(oi)
        assert np.max(np.abs(gi.astype(int) - oi.astype(int))) <= 1
    vg, vo = g.vm(), o.vm()
    assert np.max(np.abs(vg - vo) / np.abs(vo)) < 1e-9
    ag, ao = g.activation(), o.activation()
    assert np.array_equal(ag > 0, ao > 0)
    assert (ag > 0).sum() > 0
    assert np.max(np.abs(ag - ao)) < 1e-9
    g.close()


@pytest.mark.gpu
def test_float_pairs_against_fp64_pcg_on_a_propagating_slab(gpu_lib):
    """Mixed form, TNNP slab at h = 0.5 mm over 10 ms (the wave leaves the
    stimulus box): float-pair PCG against FP64 PCG in the same context type;
    also switching the arithmetic between steps."""
    dims, h, dt, nsteps = (40, 14, 6), 5e-4, 1e-5, 1000
    a = _slab(dims, h, dt, lib.PRECISION_MIXED, arithmetic=lib.PCG_FP64)
    b = _slab(dims, h, dt, lib.PRECISION_MIXED)          # float pairs by default
    with pytest.raises(RuntimeError):
        b.set_pcg_arithmetic(7)
    ia = ib = 0
    for s in range(nsteps):
        a.step(dt)
        b.step(dt)
        ia += int(np.sum(a.stats()[2]))
        ib += int(np.sum(b.stats()[2]))
    va, vb = a.vm(), b.vm()
    assert np.max(np.abs(va - vb)) <= 1e-9 * np.max(np.abs(va))
    aa, ab = a.activation(), b.activation()
    assert np.array_equal(aa > 0, ab > 0)
    assert (aa > 0).sum() > 60            # the stimulus box holds 27 cells
    assert np.max(np.abs(aa - ab)) <= 1e-8
    assert abs(ia - ib) <= max(2, ia // 100)
    # back to FP64 and to pairs again: the context keeps stepping
    b.set_pcg_arithmetic(lib.PCG_FP64)
    a.step(dt)
    b.step(dt)
    b.set_pcg_arithmetic(lib.PCG_FLOAT_PAIRS)
    a.step(dt)
    b.step(dt)
    assert np.max(np.abs(a.vm() - b.vm())) <= 1e-9 * np.max(np.abs(a.vm()))
    a.close()
    b.close()


@pytest.mark.gpu
def test_float_pairs_against_fp64_pcg_on_the_lv(gpu_lib):
    """Tetrahedral LV with per-cell tensors (the explicit corrections in the
    source every corrector): float-pair PCG against FP64 PCG, mixed form."""
    L = lv.left_ventricle(4, 8, 12, sigma_l=10 * lv.SIGMA_L, sigma_t=10 * lv.SIGMA_T)
    lo, hi = L.apex_box(8e-3)
    dt, nsteps = 5e-5, 160
    runs = []
    for arithmetic in (lib.PCG_FP64, lib.PCG_FLOAT_PAIRS):
        g = api.Monodomain(L.mesh, "TNNP", "epicardialCells", dt=dt,
                           precision=lib.PRECISION_MIXED, boxes=[(lo, hi, 0.0, 2e-3, 5e4)],
                           tissue_per_cell=L.tissue, conductivity_per_cell=L.conductivity,
                           stencil=False)
        g.set_pcg_arithmetic(arithmetic)
        iters = []
        for _ in range(nsteps):
            g.step(dt)
            iters.append(g.stats()[2])
        runs.append((g.vm(), g.activation(), iters))
        g.close()
    (va, aa, ia), (vb, ab, ib) = runs
    assert np.max(np.abs(va - vb)) <= 1e-9 * np.max(np.abs(va))
    assert np.array_equal(aa > 0, ab > 0)
    assert (aa > 0).sum() > 0
    assert np.max(np.abs(aa - ab)) <= 1e-8
    for x, y in zip(ia, ib):
        assert len(x) == len(y)
        assert np.max(np.abs(x.astype(int) - y.astype(int))) <= 1
