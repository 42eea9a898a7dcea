"""The autotuner of the ionic step kernel (cfg_ionic_autotune,
cfg_monodomain_autotune): every launch shape gives bitwise the same cells,
and a tuned context steps exactly like an untuned one."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from cardiacfoam_gb300.mesh import box_mesh

SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
BOX = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, 1.5e-3), 0.0, 2e-3, 5e4)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [lib.PRECISION_FP64, lib.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_launch_shapes_give_identical_cells(gpu_lib, precision):
    n, dt = 5000, 1e-5
    vm = -0.084 + 0.12 * np.random.default_rng(4).random(n)
    out = []
    for block, cpt in ((0, 1), (32, 1), (32, 4), (64, 2)):
        m = api.IonicModel("ORd", "myocyte", n, dt, precision=precision)
        m.set_launch(block, cpt)
        im = np.zeros(n)
        for k in range(4):
            m.solveODE(k * dt, dt, vm, im)
        out.append((im.copy(), m.states(), m.steps()))
        m.close()
    for o in out[1:]:
        for x, y in zip(o, out[0]):
            assert np.array_equal(x, y)


@pytest.mark.gpu
def test_tuned_monodomain_steps_like_an_untuned_one(gpu_lib):
    mesh = box_mesh(30, 12, 4, 0.003, 0.0012, 0.0004)
    dt = 1e-5
    a = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX,
                       precision=lib.PRECISION_MIXED)
    b = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX,
                       precision=lib.PRECISION_MIXED)
    for m in (a, b):
        m.run(dt, 20)
    block, cpt, ms = b.autotune()
    assert block % 32 == 0 and block > 0 and cpt in (1, 2, 4) and ms > 0
    for m in (a, b):
        m.run(dt, 100)
    assert np.array_equal(a.vm(), b.vm())
    assert np.array_equal(a.activation(), b.activation())
    a.close()
    b.close()
