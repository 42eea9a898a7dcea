"""Failure statuses of the GPU path, made to happen without faulting the GPU.

The reference stops with FatalError where the ODE solver exceeds maxSteps
(OpenFOAM's ODESolver, called from ionicModel::solveODE, e.g.
src/ionicModels/TNNP/TNNP.C:143) and where a domain cannot proceed
(myocardiumDomain.C:385-392); the library returns a status instead, with the
message in cfg_last_error.  Each case here is brought about by its inputs or
by a wait limit set to zero through the public setters:

* maxSteps 1 -> CFG_ERR_ODE_STEPS naming the first failing cell;
* a NaN ionic state -> CFG_ERR_NONFINITE;
* a zero spin limit on the persistent diffusion kernel's grid barriers ->
  the step gives up with CFG_ERR_PCG ("a grid barrier timed out");
* a zero cycle limit on the pseudo-ECG's tile-copy waits -> CFG_ERR_CUDA,
  the flag cleared, and the next evaluation with the default limit equal to
  the oracle's.

Every wait involved is bounded, so each case ends by itself; afterwards the
device is used again normally.
"""
import re

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from cardiacfoam_gb300.mesh import box_mesh, with_box_geometry

SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
BOX = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, 1.5e-3), 0.0, 2e-3, 5e4)]


def _error(excinfo):
    return excinfo.value.code, str(excinfo.value)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [lib.PRECISION_FP64, lib.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_max_steps_exceeded_names_the_failing_cell(gpu_lib, precision):
    n, dt = 256, 1e-5
    ion = api.IonicModel("TNNP", "epicardialCells", n, dt, precision=precision,
                         ode=api.ode_desc(max_steps=1))
    vm, im = np.full(n, -0.084), np.zeros(n)
    with pytest.raises(lib.CfgError) as e:
        ion.solveODE(0.0, dt, vm, im)
    code, msg = _error(e)
    assert code == lib.CFG_ERR_ODE_STEPS
    m = re.search(r"cell (\d+)", msg)
    assert m and 0 <= int(m.group(1)) < n
    assert "maximum 1" in msg
    ion.close()
    # the same solve with the default maxSteps goes through
    ok = api.IonicModel("TNNP", "epicardialCells", n, dt, precision=precision)
    ok.solveODE(0.0, dt, vm, im)
    assert np.all(np.isfinite(im))
    ok.close()


@pytest.mark.gpu
def test_max_steps_exceeded_in_a_tissue_step(gpu_lib):
    mesh = box_mesh(20, 7, 3, 0.02, 0.007, 0.003)
    m = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=1e-5, boxes=BOX, max_steps=1)
    with pytest.raises(lib.CfgError) as e:
        m.step(1e-5)
    assert _error(e)[0] == lib.CFG_ERR_ODE_STEPS
    m.close()


@pytest.mark.gpu
def test_nan_state_gives_nonfinite_current(gpu_lib):
    n, dt = 64, 1e-5
    ion = api.IonicModel("TNNP", "epicardialCells", n, dt)
    y = ion.states()
    y[7, 17] = np.nan              # the INa activation gate m of one cell
    ion.set_states(y)
    vm, im = np.full(n, -0.084), np.zeros(n)
    with pytest.raises(lib.CfgError) as e:
        ion.solveODE(0.0, dt, vm, im)
    assert _error(e)[0] == lib.CFG_ERR_NONFINITE
    assert np.isnan(im[17])
    assert np.all(np.isfinite(np.delete(im, 17)))
    ion.close()


@pytest.mark.gpu
def test_grid_barrier_wait_limit_aborts_the_step(gpu_lib):
    """A zero spin limit: the first block to reach a grid barrier of the
    persistent diffusion kernel (7 blocks on this slab) gives up at once, every
    block leaves, and the step reports it."""
    dt = 1e-5
    mesh = box_mesh(40, 14, 6, 0.02, 0.007, 0.003)
    m = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX)
    m.step(dt)
    m.set_wait_limit(0)
    with pytest.raises(lib.CfgError) as e:
        m.step(dt)
    code, msg = _error(e)
    assert code == lib.CFG_ERR_PCG
    assert "grid barrier timed out" in msg
    m.close()
    # fresh contexts with the default limit: the same steps, the same fields
    runs = []
    for _ in range(2):
        f = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX)
        f.run(dt, 20)
        runs.append(f.vm())
        f.close()
    assert np.all(np.isfinite(runs[0])) and np.array_equal(runs[0], runs[1])


@pytest.mark.gpu
def test_pseudo_ecg_copy_wait_limit(gpu_lib, oracle):
    """A zero cycle limit on the staged kernel's tile-copy waits: the
    evaluation reports CFG_ERR_CUDA (its copies in flight drained under the
    default limit before the blocks leave), the flag is cleared, and with the
    default limit restored the next evaluation equals the oracle's."""
    h, dt = 2.5e-4, 1e-5
    nx, ny, nz = 64, 32, 8
    mesh = with_box_geometry(box_mesh(nx, ny, nz, nx * h, ny * h, nz * h),
                             nx * h, ny * h, nz * h)
    md = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX, stencil=False)
    md.run(dt, 50)
    el = np.array([[-2e-3, 4e-3, 1e-3], [2e-2, 4e-3, 1e-3], [8e-3, -3e-3, 1e-3]])
    pe = api.PseudoECG(mesh, el, sigma=SIGMA)
    pe.set_wait_limit(0)
    with pytest.raises(lib.CfgError) as e:
        pe.compute(md)
    code, msg = _error(e)
    assert code == lib.CFG_ERR_CUDA
    assert "wait limit" in msg
    pe.set_wait_limit(-1)
    got = pe.compute(md)
    o = oracle.Tissue(oracle.tissue_desc("TNNP", 1, SIGMA), oracle.Mesh.general(mesh))
    want = o.pseudo_ecg(md.vm(), el)
    assert np.all(np.abs(got - want) <= 1e-10 * np.max(np.abs(want)))
    # the monodomain context is unaffected
    md.step(dt)
    pe.close()
    md.close()
