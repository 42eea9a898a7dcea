"""The bidomain step on the GPU (cfg_bidomain_*) against the oracle's
restatement of BidomainSolver: the manufactured case (FP64, both
preconditioners of the oracle), a propagating TNNP slab, second-order
convergence of the manufactured run, a tetrahedral left ventricle with the
Laplacians' explicit corrections, and the explicit algorithm; the PCG of
both systems in FP64 and in float pairs."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib, lv, verification as V
from cardiacfoam_gb300.mesh import box_mesh, with_box_geometry


def _gpu_mms(dim, n, dt):
    mesh = V.geometry_mesh_for(dim, n)
    bd = api.Bidomain(mesh, model="bidomainFDAManufactured", tissue=f"{dim}D",
                      sigma_i=V.BIDOMAIN_SIGMA_I, sigma_e=V.BIDOMAIN_SIGMA_E, chi=V.CHI, cm=V.CM,
                      dt=dt, pcg_tol=1e-12, phie_tol=1e-12, phie_max_iter=4000, n_outer=2,
                      ref_point=V.BIDOMAIN_REF_POINT, grad_scheme=lib.GRAD_GAUSS_LINEAR)
    vm, pe, _, u1, u2, u3 = V.bidomain_fields(mesh.centres, 0.0, dim)
    bd.set_field(lib.FIELD_VM, vm)
    bd.set_field(lib.FIELD_PHIE, pe)
    bd.set_states(np.stack([vm, u1, u2, u3]))
    return mesh, bd


def _oracle_mms(oracle, mesh, dim, dt, dic):
    d = oracle.tissue_desc("bidomainFDAManufactured", 10 + dim, V.BIDOMAIN_SIGMA_I, chi=V.CHI,
                           cm=V.CM, implicit=True, precond_dic=dic, pcg_tol=1e-12,
                           pcg_rel_tol=0.0, pcg_max_iter=2000, n_outer=2, outer_tol=0.0,
                           grad_gauss=True)
    B = oracle.Bidomain(d, V.BIDOMAIN_SIGMA_E, oracle.Mesh.general(mesh), V.BIDOMAIN_REF_POINT,
                        0.0, 1e-12, 0.0, 4000)
    vm, pe, _, u1, u2, u3 = V.bidomain_fields(mesh.centres, 0.0, dim)
    B.tissue.set_vm(vm)
    B.tissue.set_states(np.stack([vm, u1, u2, u3]), dt)
    B.set_phie(pe)
    return B


def _close(a, b, tol):
    return np.max(np.abs(a - b)) <= tol * np.max(np.abs(b))


@pytest.mark.gpu
@pytest.mark.parametrize("dic,arithmetic", [(False, lib.PCG_FP64), (False, lib.PCG_FLOAT_PAIRS),
                                            (True, lib.PCG_FP64)],
                         ids=["diagonal", "diagonal-float-pairs", "dic"])
def test_manufactured_matches_oracle(gpu_lib, oracle, dic, arithmetic):
    """8^3 cube, 20 steps: with the same (diagonal) preconditioner Vm, phiE and
    phiI within 1e-9 and PCG iteration counts within one, with the GPU's PCG
    in FP64 or in float pairs; against the reference's DIC preconditioner
    within the solver tolerance's reach."""
    dt = 2e-3
    mesh, bd = _gpu_mms(3, 8, dt)
    bd.set_pcg_arithmetic(arithmetic)
    B = _oracle_mms(oracle, mesh, 3, dt, dic)
    assert bd.reference_cell() == B.ref_cell()
    tol = 1e-9 if not dic else 1e-7
    for _ in range(20):
        bd.step(dt)
        B.step(dt)
        if not dic:
            (_, _, it_v), (_, _, it_e) = bd.stats()
            assert np.max(np.abs(it_v - B.tissue.solves()[2])) <= 1
            assert np.max(np.abs(it_e - B.phie_solves()[2])) <= 1
    assert _close(bd.vm(), B.tissue.vm(), tol)
    assert _close(bd.phie(), B.phie(), tol)
    assert _close(bd.phii(), B.phii(), tol)
    bd.close()


@pytest.mark.gpu
def test_tnnp_slab_matches_oracle(gpu_lib, oracle):
    """A propagating TNNP slab (24 x 8 x 2 cells of 0.25 mm, corner stimulus):
    Vm, phiE and activation times against the oracle."""
    h, dt = 2.5e-4, 2e-5
    mesh = with_box_geometry(box_mesh(24, 8, 2, 24 * h, 8 * h, 2 * h), 24 * h, 8 * h, 2 * h)
    box = [((0.0, 0.0, 0.0), (1.0e-3, 2 * h * 8, 2 * h), 0.0, 1e-3, 1e5)]
    gi, ge = (0.17, 0.0, 0.0, 0.019, 0.0, 0.019), (0.62, 0.0, 0.0, 0.24, 0.0, 0.24)
    bd = api.Bidomain(mesh, "TNNP", "epicardialCells", sigma_i=gi, sigma_e=ge, dt=dt,
                      pcg_tol=1e-10, phie_tol=1e-10, n_outer=2, ref_point=(0.0, 0.0, 0.0),
                      boxes=box)
    d = oracle.tissue_desc("TNNP", 1, gi, implicit=True, precond_dic=False, pcg_tol=1e-10,
                           pcg_rel_tol=0.0, n_outer=2, outer_tol=0.0, boxes=box)
    B = oracle.Bidomain(d, ge, oracle.Mesh.general(mesh), (0.0, 0.0, 0.0), 0.0, 1e-10, 0.0, 1000)
    for _ in range(200):
        bd.step(dt)
        B.step(dt)
    vg, vo = bd.vm(), B.tissue.vm()
    assert np.max(np.abs(vg - vo) / np.abs(vo)) < 1e-9
    assert _close(bd.phie(), B.phie(), 1e-9)
    ag, ao = bd.activation(), B.tissue.activation()
    assert np.array_equal(ag > 0, ao > 0) and (ag > 0).sum() > 20
    assert np.max(np.abs(ag - ao)) < 1e-9
    bd.close()


@pytest.mark.gpu
def test_manufactured_convergence(gpu_lib):
    """The tutorial's 3D case at 10 and 20 cells to t = 0.2 s: Vm and phiE
    (up to its reference constant) converge towards second order (the
    oracle's rates on the same meshes: L1/L2/Linf of Vm 1.69/1.74/1.65, phiE
    1.76, still pre-asymptotic at 10 cells; 1D reaches 1.99)."""
    r = [V.run_bidomain(3, n) for n in (10, 20)]
    assert V.rate(r[0]["V"][1], r[1]["V"][1], 10, 20) > 1.6
    assert V.rate(r[0]["V"][2], r[1]["V"][2], 10, 20) > 1.6
    errs = []
    for n in (10, 20):
        mesh, bd = _gpu_mms(3, n, V.SWEEP[n])
        bd.run(V.SWEEP[n], int(round(V.END_TIME / V.SWEEP[n])))
        _, pe, *_ = V.bidomain_fields(mesh.centres, bd.time(), 3)
        e = bd.phie() - pe
        errs.append(np.max(np.abs(e - e.mean())))
        bd.close()
    assert V.rate(errs[0], errs[1], 10, 20) > 1.6


@pytest.mark.gpu
@pytest.mark.parametrize("arithmetic", [lib.PCG_FP64, lib.PCG_FLOAT_PAIRS],
                         ids=["fp64", "float-pairs"])
def test_tetrahedral_lv_matches_oracle(gpu_lib, oracle, arithmetic):
    """A tetrahedral left ventricle (4,104 tets): non-orthogonal faces, so
    both Laplacians carry their explicit corrections (Gauss linear corrected,
    leastSquares gradient) in the phiE and the Vm solve.  Vm, phiE and the
    activation times against the oracle, PCG iteration counts within one."""
    L = lv.left_ventricle(3, 6, 8)
    lo, hi = L.apex_box(8e-3)
    box = [(lo, hi, 0.0, 1e-3, 1e5)]
    gi, ge = (0.17, 0.0, 0.0, 0.019, 0.0, 0.019), (0.62, 0.0, 0.0, 0.24, 0.0, 0.24)
    dt = 2e-5
    bd = api.Bidomain(L.mesh, "TNNP", "epicardialCells", sigma_i=gi, sigma_e=ge, dt=dt,
                      pcg_tol=1e-10, phie_tol=1e-10, n_outer=2, ref_point=(0.0, 0.0, 0.0),
                      boxes=box)
    bd.set_pcg_arithmetic(arithmetic)
    d = oracle.tissue_desc("TNNP", 1, gi, implicit=True, precond_dic=False, pcg_tol=1e-10,
                           pcg_rel_tol=0.0, n_outer=2, outer_tol=0.0, boxes=box)
    B = oracle.Bidomain(d, ge, oracle.Mesh.general(L.mesh), (0.0, 0.0, 0.0), 0.0, 1e-10, 0.0,
                        1000)
    for _ in range(150):
        bd.step(dt)
        B.step(dt)
        (_, _, it_v), (_, _, it_e) = bd.stats()
        assert np.max(np.abs(it_v - B.tissue.solves()[2])) <= 1
        assert np.max(np.abs(it_e - B.phie_solves()[2])) <= 1
    assert _close(bd.vm(), B.tissue.vm(), 1e-9)
    assert _close(bd.phie(), B.phie(), 1e-9)
    ag, ao = bd.activation(), B.tissue.activation()
    assert np.array_equal(ag > 0, ao > 0) and (ag > 0).sum() >= 10
    assert np.max(np.abs(ag - ao)) < 1e-9
    bd.close()
    with pytest.raises(ValueError):
        api.Bidomain(box_mesh(4, 4, 4, 1e-3, 1e-3, 1e-3), "TNNP", "epicardialCells")


ELECTRO_PROPERTIES = """
myocardiumSolver  bidomainSolver;
bidomainSolverCoeffs
{
    conductivityIntracellular [-1 -3 3 0 0 2 0] (0.17 0 0 0.019 0 0.019);
    conductivityExtracellular [-1 -3 3 0 0 2 0] (0.62 0 0 0.24 0 0.24);
    chi  [0 -1 0 0 0 0 0] 140000;
    cm   [-1 -4 4 0 0 2 0] 0.01;
    ionicModel TNNP;
    tissue epicardialCells;
    solutionAlgorithm implicit;
    maxSteps 1000000;
    phiERefPoint (0 0 0);
    externalStimulus
    {
        stimulusLocationMin (0 0 0);
        stimulusLocationMax (1e-3 4e-3 5e-4);
        stimulusDuration [0 0 1 0 0 0 0] 1e-3;
        stimulusIntensity [0 -3 0 0 0 1 0] 1e5;
    }
}
"""


@pytest.mark.gpu
def test_from_dict_equals_the_description(gpu_lib):
    """cfg_bidomain_create_from_dict builds the same context as the
    description with the dictionary's values and the documented defaults
    (PCG 1e-12, maxIter 1000, two correctors, Gauss linear gradients)."""
    h, dt = 2.5e-4, 2e-5
    mesh = with_box_geometry(box_mesh(24, 8, 2, 24 * h, 8 * h, 2 * h), 24 * h, 8 * h, 2 * h)
    a = api.Bidomain.from_dict(ELECTRO_PROPERTIES, mesh, dt)
    b = api.Bidomain(mesh, "TNNP", "epicardialCells", sigma_i=(0.17, 0, 0, 0.019, 0, 0.019),
                     sigma_e=(0.62, 0, 0, 0.24, 0, 0.24), chi=140000.0, cm=0.01, dt=dt,
                     pcg_tol=1e-12, phie_tol=1e-12, n_outer=2, ref_point=(0.0, 0.0, 0.0),
                     boxes=[((0.0, 0.0, 0.0), (1e-3, 4e-3, 5e-4), 0.0, 1e-3, 1e5)],
                     grad_scheme=lib.GRAD_GAUSS_LINEAR, max_steps=10 ** 6)
    for _ in range(30):
        a.step(dt)
        b.step(dt)
    assert np.array_equal(a.vm(), b.vm())
    assert np.array_equal(a.phie(), b.phie())
    assert np.max(a.vm()) > -0.084
    a.close()
    b.close()


@pytest.mark.gpu
def test_explicit_algorithm_matches_oracle(gpu_lib, oracle):
    """solutionAlgorithm explicit (bidomainSolver.C:183-213): the phiE solve,
    then Vm from the diagonal ddt matrix with div(Gi grad(Vm + phiE)), on the
    propagating TNNP slab against the oracle's restatement; and from the
    dictionary front end."""
    h, dt = 2.5e-4, 5e-6
    mesh = with_box_geometry(box_mesh(24, 8, 2, 24 * h, 8 * h, 2 * h), 24 * h, 8 * h, 2 * h)
    box = [((0.0, 0.0, 0.0), (1.0e-3, 2 * h * 8, 2 * h), 0.0, 1e-3, 1e5)]
    gi, ge = (0.17, 0.0, 0.0, 0.019, 0.0, 0.019), (0.62, 0.0, 0.0, 0.24, 0.0, 0.24)
    bd = api.Bidomain(mesh, "TNNP", "epicardialCells", sigma_i=gi, sigma_e=ge, dt=dt,
                      phie_tol=1e-10, ref_point=(0.0, 0.0, 0.0), boxes=box, implicit=False)
    d = oracle.tissue_desc("TNNP", 1, gi, implicit=False, precond_dic=False, pcg_tol=1e-10,
                           pcg_rel_tol=0.0, n_outer=1, outer_tol=0.0, boxes=box)
    B = oracle.Bidomain(d, ge, oracle.Mesh.general(mesh), (0.0, 0.0, 0.0), 0.0, 1e-10, 0.0, 1000)
    for _ in range(400):
        bd.step(dt)
        B.step(dt)
        (_, _, it_v), (_, _, it_e) = bd.stats()
        assert it_v.size == 0 or np.all(it_v == 0)
        assert np.max(np.abs(it_e - B.phie_solves()[2])) <= 1
    vg, vo = bd.vm(), B.tissue.vm()
    assert np.max(np.abs(vg - vo)) <= 1e-9 * np.max(np.abs(vo))
    assert _close(bd.phie(), B.phie(), 1e-9)
    assert _close(bd.phii(), B.phii(), 1e-9)
    ag, ao = bd.activation(), B.tissue.activation()
    assert np.array_equal(ag > 0, ao > 0) and (ag > 0).sum() > 20
    assert np.max(np.abs(ag - ao)) < 1e-9
    bd.close()


@pytest.mark.gpu
def test_mixed_form_float_pairs_against_fp64_pcg(gpu_lib):
    """Mixed ionic form on the propagating TNNP slab: the default float-pair
    PCG against the FP64 PCG of the same context type (Vm and phiE within
    1e-9 of their scale, the same activated cells within 1e-8 s)."""
    h, dt = 2.5e-4, 2e-5
    mesh = with_box_geometry(box_mesh(24, 8, 2, 24 * h, 8 * h, 2 * h), 24 * h, 8 * h, 2 * h)
    box = [((0.0, 0.0, 0.0), (1.0e-3, 2 * h * 8, 2 * h), 0.0, 1e-3, 1e5)]
    gi, ge = (0.17, 0.0, 0.0, 0.019, 0.0, 0.019), (0.62, 0.0, 0.0, 0.24, 0.0, 0.24)
    runs = []
    for arithmetic in (lib.PCG_FP64, lib.PCG_FLOAT_PAIRS):
        bd = api.Bidomain(mesh, "TNNP", "epicardialCells", sigma_i=gi, sigma_e=ge, dt=dt,
                          pcg_tol=1e-10, phie_tol=1e-10, n_outer=2, ref_point=(0.0, 0.0, 0.0),
                          boxes=box, precision=lib.PRECISION_MIXED)
        bd.set_pcg_arithmetic(arithmetic)
        for _ in range(200):
            bd.step(dt)
        runs.append((bd.vm(), bd.phie(), bd.activation()))
        bd.close()
    (va, pa, aa), (vb, pb, ab) = runs
    assert _close(vb, va, 1e-9)
    assert _close(pb, pa, 1e-9)
    assert np.array_equal(aa > 0, ab > 0) and (aa > 0).sum() > 20
    assert np.max(np.abs(aa - ab)) < 1e-8
