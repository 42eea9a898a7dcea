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


BIDOMAIN_DICT = """
myocardiumSolver  %s;
bidomainSolverCoeffs
{
    conductivityIntracellular [-1 -3 3 0 0 2 0] (0.17 0 0 0.019 0 0.019);
    conductivityExtracellular [-1 -3 3 0 0 2 0] %s;
    chi  [0 -1 0 0 0 0 0] 140000;
    cm   [-1 -4 4 0 0 2 0] 0.01;
    ionicModel TNNP;
    tissue epicardialCells;
    solutionAlgorithm %s;
    maxSteps 1000000;
    %s
    externalStimulus
    {
        stimulusLocationMin (0 0 0);
        stimulusLocationMax (1e-3 4e-3 5e-4);
        stimulusDuration [0 0 1 0 0 0 0] 1e-3;
        stimulusIntensity [0 -3 0 0 0 1 0] 1e5;
    }
}
"""
GOOD = ("bidomainSolver", "(0.62 0 0 0.24 0 0.24)", "implicit", "phiERefPoint (0 0 0);")


def _from_dict(gpu_lib, text, mesh):
    import ctypes as C
    from cardiacfoam_gb300 import api
    md, keep = api.mesh_desc(mesh, structured=False)
    h = C.c_void_p()
    return gpu_lib.cfg_bidomain_create_from_dict(text.encode(), C.byref(md), 2e-5, 0, C.byref(h))


def test_bidomain_dictionary_errors(gpu_lib):
    """Errors of cfg_bidomain_create_from_dict found while reading the
    dictionary or the mesh, before any device work."""
    from cardiacfoam_gb300 import lib
    from cardiacfoam_gb300.mesh import box_mesh, with_box_geometry
    geo = with_box_geometry(box_mesh(4, 2, 1, 1e-3, 5e-4, 2.5e-4), 1e-3, 5e-4, 2.5e-4)
    bad = [(("monodomainSolver",) + GOOD[1:], lib.CFG_ERR_UNSUPPORTED),
           ((GOOD[0], GOOD[1], "sideways", GOOD[3]), lib.CFG_ERR_INVALID),
           ((GOOD[0], "(0.62 0 0 0.24)", GOOD[2], GOOD[3]), lib.CFG_ERR_INVALID),
           (GOOD[:3] + ("",), lib.CFG_ERR_INVALID)]
    for args, code in bad:
        assert _from_dict(gpu_lib, BIDOMAIN_DICT % args, geo) == code, args
    # a mesh without its geometry is refused before the device is touched
    assert _from_dict(gpu_lib, BIDOMAIN_DICT % GOOD, box_mesh(4, 2, 1, 1e-3, 5e-4, 2.5e-4)) == \
        lib.CFG_ERR_INVALID
    assert "geometry" in lib.load().cfg_last_error().decode()


def test_bidomain_model_constants(oracle):
    """bidomainFDAManufactured's initConsts (bidomainFDAManufactured_2014.H)
    as emitted: Cm 2, Chi 3, Beta = betaBase(dimension) (1 - k) with the
    tutorial's k, everything else as the monodomain manufactured model; the
    right-hand sides agree with the monodomain model's once Beta is equal."""
    k = V.BIDOMAIN_K
    rng = np.random.default_rng(5)
    for dim, base in ((1, -1.1), (2, -5.9), (3, -8.6)):
        c, _ = oracle.model_init("bidomainFDAManufactured", 10 + dim)
        assert c[0] == 2.0 and c[2] == 3.0
        assert c[1] == base * (1.0 - k)
        cm, _ = oracle.model_init("monodomainFDAManufactured", 10 + dim)
        y = rng.uniform(0.5, 1.5, 4)
        out = []
        for cc, model in ((c, "bidomainFDAManufactured"), (cm, "monodomainFDAManufactured")):
            dydt, alg = np.zeros(4), np.zeros(1)
            oracle.lib().oracle_model_variables(oracle.MODELS[model], 0.0, oracle.ptr(cc),
                                                oracle.ptr(dydt), oracle.ptr(y), oracle.ptr(alg),
                                                10 + dim, 0, None)
            out.append((dydt.copy(), alg.copy()))
        assert np.array_equal(out[0][0], out[1][0])   # the rates do not involve Beta


def test_create_rejects_bad_arguments(gpu_lib):
    """cfg_bidomain_create's argument checks, made before any device work."""
    import ctypes as C
    from cardiacfoam_gb300 import api, lib
    from cardiacfoam_gb300.mesh import box_mesh
    geo = V.geometry_mesh_for(3, 4)

    def create(mesh, n_cells=None, n_outer=2, boxes=0, zero_sigma=False):
        keep = []
        d = lib.BidomainDesc()
        d.ionic = api.ionic_desc("TNNP", "epicardialCells",
                                 mesh.n_cells if n_cells is None else n_cells, 1e-5, False,
                                 lib.PRECISION_FP64, api.ode_desc(), None, None, None, keep)
        d.n_outer, d.n_boxes = n_outer, boxes
        for i in range(6):
            if not zero_sigma:
                d.conductivity_i[i] = (0.17, 0, 0, 0.019, 0, 0.019)[i]
                d.conductivity_e[i] = (0.62, 0, 0, 0.24, 0, 0.24)[i]
        md, k2 = api.mesh_desc(mesh, structured=False)
        h = C.c_void_p()
        return gpu_lib.cfg_bidomain_create(C.byref(d), C.byref(md), C.byref(h))

    assert create(box_mesh(4, 4, 4, 1.0, 1.0, 1.0)) == lib.CFG_ERR_INVALID    # no geometry
    assert create(geo, n_cells=7) == lib.CFG_ERR_INVALID
    assert create(geo, n_outer=0) == lib.CFG_ERR_INVALID
    assert create(geo, boxes=9) == lib.CFG_ERR_INVALID
    assert create(geo, zero_sigma=True) == lib.CFG_ERR_INVALID
