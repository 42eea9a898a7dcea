"""The plain FP64 step on the benchmark slabs at their own sizes, against the
oracle (through the C ABI).

* The 20 x 7 x 3 mm slab at h = 0.5 mm (40 x 14 x 6 = 3,360 cells), TNNP
  epicardialCells from Vm0 = -84 mV, dt = 0.01 ms, the full 50 ms: the
  wavefront propagates from the 27-cell stimulus corner through about 1,200
  cells.  Against the oracle with the same (diagonal) preconditioner: Vm
  within 1e-9 of the field's largest value after every 500 steps (measured
  on a GB300: 1e-10; pointwise relative errors grow only where Vm crosses
  0 mV), PCG iteration counts within one per solve (identical in practice),
  the same cells activated, within 1e-9 s.  Against the reference's own DIC
  preconditioner: activation within one dt, and a cell activated in one run
  only lies on the front at the last step.
* The same slab at h = 0.1 mm (200 x 70 x 30 = 420,000 cells), ORd myocyte,
  dt = 5 us: 100 steps, Vm within 1e-9 of its largest value and PCG
  iteration counts within one per solve.

The ionic update is adaptive (RKF45) and the device's exp/log differ from
the host C library's in the last bit now and then; through the adaptive
step control such a difference stays at the level of the ODE tolerance's
effect on one step, far below the bars above.

Settings of both: backward ddt, PIMPLE residualControl 1e-6, PCG tolerance
1e-8 (relTol 0), corner box stimulus 5e4 A/m^3 over [0, 1.5 mm]^3 for 2 ms,
sigma = diag(0.1334, 0.0176, 0.0176) S/m, chi = 1.4e5 1/m, Cm = 0.01 F/m^2.
"""
import os

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from cardiacfoam_gb300.mesh import box_mesh

SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
BOX = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, 1.5e-3), 0.0, 2e-3, 5e4)]
THREADS = os.cpu_count() or 1


def slab(oracle, dims, h, model, tissue, dt, precond_dic):
    nx, ny, nz = dims
    mesh = box_mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    g = api.Monodomain(mesh, model, tissue, SIGMA, dt=dt, precision=lib.PRECISION_FP64,
                       boxes=BOX, pcg_tol=1e-8)
    d = oracle.tissue_desc(model, api.TISSUE_FLAGS[tissue], SIGMA, implicit=True,
                           precond_dic=precond_dic, boxes=BOX, pcg_tol=1e-8,
                           ode=oracle.ode_settings(max_steps=10 ** 6))
    o = oracle.Tissue(d, oracle.Mesh(nx, ny, nz, nx * h, ny * h, nz * h))
    return g, o


@pytest.mark.gpu
def test_tnnp_slab_h05_full_50ms_against_oracle(gpu_lib, oracle):
    dt, steps = 1e-5, 5000
    g, o = slab(oracle, (40, 14, 6), 5e-4, "TNNP", "epicardialCells", dt, False)
    worst, same = 0.0, 0
    for s in range(steps):
        g.step(dt)
        o.step(dt, THREADS)
        gi, oi = g.stats()[2], o.solves()[2]
        assert len(gi) == len(oi) and np.max(np.abs(gi - oi)) <= 1, (s, gi, oi)
        same += int(np.array_equal(gi, oi))
        if (s + 1) % 500 == 0:
            vg, vo = g.vm(), o.vm()
            worst = max(worst, float(np.max(np.abs(vg - vo)) / np.max(np.abs(vo))))
            assert worst < 1e-9, (s, worst)
    assert same >= 0.99 * steps
    ag, ao = g.activation(), o.activation()
    # activated by propagation, far beyond the 27 stimulated cells
    assert np.array_equal(ag > 0, ao > 0)
    assert int(np.sum(ag > 0)) > 1000
    assert np.max(np.abs(ag - ao)) < 1e-9
    assert abs(g.time() - o.time()) == 0.0
    t_end = g.time()
    g.close()

    # the reference's DIC preconditioner: activation within one dt
    _, od = slab(oracle, (40, 14, 6), 5e-4, "TNNP", "epicardialCells", dt, True)
    for _ in range(steps):
        od.step(dt, THREADS)
    ad = od.activation()
    both = (ag > 0) & (ad > 0)
    assert np.max(np.abs(ag[both] - ad[both])) <= dt
    only = (ag > 0) != (ad > 0)
    assert np.all(np.maximum(ag[only], ad[only]) >= t_end - 2 * dt)


@pytest.mark.gpu
def test_ord_slab_h01_420k_cells_against_oracle(gpu_lib, oracle):
    dt, steps = 5e-6, 100
    g, o = slab(oracle, (200, 70, 30), 1e-4, "ORd", "myocyte", dt, False)
    for s in range(steps):
        g.step(dt)
        o.step(dt, THREADS)
        gi, oi = g.stats()[2], o.solves()[2]
        assert len(gi) == len(oi) and np.max(np.abs(gi - oi)) <= 1, (s, gi, oi)
    vg, vo = g.vm(), o.vm()
    assert np.max(np.abs(vg - vo)) < 1e-9 * np.max(np.abs(vo))
    ag, ao = g.activation(), o.activation()
    assert np.array_equal(ag > 0, ao > 0)
    if np.any(ao > 0):
        assert np.max(np.abs(ag - ao)) < 1e-9
    g.close()
