"""Bidomain on the CPU: the oracle's restatement of BidomainSolver
(oracle_bidomain_*) on the bidomain tutorial's manufactured solution
(bidomainFDAManufactured, manufacturedFDABidomainReference.H): second-order
convergence of Vm, and of phiE up to the constant that setReference fixes at
the reference cell's centre rather than at phiERefPoint."""
import numpy as np
import pytest

from cardiacfoam_gb300 import verification as V


def _oracle_run(oracle, dim, n, steps=None, dic=True, tol=1e-12):
    m = V.geometry_mesh_for(dim, n)
    dt = V.SWEEP[n]
    d = oracle.tissue_desc("bidomainFDAManufactured", 10 + dim, V.BIDOMAIN_SIGMA_I, chi=V.CHI,
                           cm=V.CM, implicit=True, precond_dic=dic, pcg_tol=tol, pcg_rel_tol=0.0,
                           pcg_max_iter=2000, n_outer=2, outer_tol=0.0, grad_gauss=True)
    B = oracle.Bidomain(d, V.BIDOMAIN_SIGMA_E, oracle.Mesh.general(m), V.BIDOMAIN_REF_POINT, 0.0,
                        tol, 0.0, 4000)
    vm, pe, _, u1, u2, u3 = V.bidomain_fields(m.centres, 0.0, dim)
    B.tissue.set_vm(vm)
    B.tissue.set_states(np.stack([vm, u1, u2, u3]), dt)
    B.set_phie(pe)
    steps = int(round(V.END_TIME / dt)) if steps is None else steps
    for _ in range(steps):
        B.step(dt)
    return m, B


def test_manufactured_convergence_1d(oracle):
    err_v, err_e = [], []
    for n in (10, 20, 40):
        m, B = _oracle_run(oracle, 1, n)
        ve, pe, pie, *_ = V.bidomain_fields(m.centres, B.tissue.time(), 1)
        err_v.append(np.max(np.abs(B.tissue.vm() - ve)))
        e = B.phie() - pe
        err_e.append(np.max(np.abs(e - e.mean())))
        # phiI = Vm + phiE
        assert np.array_equal(B.phii(), B.tissue.vm() + B.phie())
    assert V.rate(err_v[0], err_v[1], 10, 20) > 1.9 and V.rate(err_v[1], err_v[2], 20, 40) > 1.9
    assert V.rate(err_e[0], err_e[1], 10, 20) > 1.9 and V.rate(err_e[1], err_e[2], 20, 40) > 1.9


def test_reference_cell_and_compatibility(oracle):
    """setReference pins phiE at the reference cell (the source of the
    Neumann problem sums to zero on the box, so the pinned row's residual
    vanishes); the reference cell is the nearest centre, the first on ties
    (phiERefPoint x = 0.125 lies on a face of the 40-cell mesh)."""
    m, B = _oracle_run(oracle, 1, 40, steps=3)
    assert B.ref_cell() == 4
    assert abs(B.phie()[B.ref_cell()]) < 1e-12 * np.max(np.abs(B.phie()))
    m, B = _oracle_run(oracle, 2, 10, steps=2)
    c = m.centres[B.ref_cell()]
    assert np.allclose(c[:2], [0.15, 0.05])


def test_2d_phie_shape_converges(oracle):
    errs = []
    for n in (10, 20):
        m, B = _oracle_run(oracle, 2, n)
        _, pe, *_ = V.bidomain_fields(m.centres, B.tissue.time(), 2)
        e = B.phie() - pe
        errs.append(np.max(np.abs(e - e.mean())))
    assert V.rate(errs[0], errs[1], 10, 20) > 1.7
