"""The pseudo-ECG on the GPU (cfg_pseudo_ecg_*) against the oracle's
restatement of PseudoECGSolver::compute: on the left ventricle after a
propagating run (per-cell conductivity tensors, both gradient schemes), on
the manufactured field (second-order convergence to the quadrature
reference), through a full manufactured monodomain run with the ECG recorded
every step, and its edge cases."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib, lv, verification as V

LV_DIMS = (4, 8, 12)
DT = 5e-5
ELECTRODES = [p for _, p in V.ECG_ELECTRODES]


def _lv_electrodes(L):
    return L.ecg_electrodes()


@pytest.fixture(scope="module")
def small_lv():
    return lv.left_ventricle(*LV_DIMS, sigma_l=10 * lv.SIGMA_L, sigma_t=10 * lv.SIGMA_T)


def _tol(ref):
    return 1e-10 * np.max(np.abs(ref))


ARITHMETIC = pytest.mark.parametrize("arith", [lib.ECG_FLOAT_PAIRS, lib.ECG_FP64],
                                     ids=["float-pairs", "fp64"])


@pytest.mark.gpu
@ARITHMETIC
@pytest.mark.parametrize("grad", [lib.GRAD_LEAST_SQUARES, lib.GRAD_GAUSS_LINEAR],
                         ids=["least-squares", "gauss-linear"])
def test_lv_matches_oracle(gpu_lib, oracle, small_lv, grad, arith):
    L = small_lv
    lo, hi = L.apex_box(8e-3)
    md = api.Monodomain(L.mesh, "TNNP", "epicardialCells", dt=DT, boxes=[(lo, hi, 0.0, 2e-3, 5e4)],
                        tissue_per_cell=L.tissue, conductivity_per_cell=L.conductivity,
                        grad_scheme=grad, stencil=False)
    el = _lv_electrodes(L)
    pe = api.PseudoECG(L.mesh, el, conductivity_per_cell=L.conductivity, grad_scheme=grad,
                       arithmetic=arith)
    d = oracle.tissue_desc("TNNP", 1, grad_gauss=grad == lib.GRAD_GAUSS_LINEAR)
    o = oracle.Tissue(d, oracle.Mesh.general(L.mesh))
    o.set_conductivity(L.conductivity)
    seen = 0.0
    for k in range(4):
        md.run(DT, 40)
        got = pe.compute(md)
        want = o.pseudo_ecg(md.vm(), el)
        assert np.all(np.abs(got - want) <= _tol(want)), (k, got, want)
        seen = max(seen, np.max(np.abs(want)))
    assert seen > 0
    pe.close()
    md.close()


@pytest.mark.gpu
def test_record_matches_compute(gpu_lib, small_lv):
    """record() after every step keeps what compute() returns, with the
    step's time; the series is bitwise reproducible and bounded."""
    L = small_lv
    lo, hi = L.apex_box(8e-3)
    md = api.Monodomain(L.mesh, "TNNP", "epicardialCells", dt=DT, boxes=[(lo, hi, 0.0, 2e-3, 5e4)],
                        tissue_per_cell=L.tissue, conductivity_per_cell=L.conductivity,
                        stencil=False)
    pe = api.PseudoECG(L.mesh, _lv_electrodes(L), conductivity_per_cell=L.conductivity,
                       max_rows=30)
    times, rows = [], []
    for _ in range(30):
        md.step(DT)
        pe.record(md)
        times.append(md.time())
        rows.append(pe.compute(md))
    t, v = pe.series()
    assert np.array_equal(t, times)
    assert np.array_equal(v, np.array(rows))
    assert np.max(np.abs(v[-1])) > 0
    with pytest.raises(lib.CfgError):
        pe.record(md)
    pe.reset()
    pe.record(md)
    t2, v2 = pe.series()
    assert t2.shape == (1,) and np.array_equal(v2[0], v[-1])
    pe.close()
    md.close()


@pytest.mark.gpu
@pytest.mark.parametrize("grad", [lib.GRAD_LEAST_SQUARES, lib.GRAD_GAUSS_LINEAR],
                         ids=["least-squares", "gauss-linear"])
def test_manufactured_field(gpu_lib, oracle, grad):
    """The exact field on 8/16/32-cell cubes from a torch tensor: equal to the
    oracle, second order towards the quadrature reference."""
    torch = pytest.importorskip("torch")
    ref = V.pseudo_ecg_spatial_reference(ELECTRODES, 3, 96)
    err = []
    for n in (8, 16, 32):
        m = V.geometry_mesh_for(3, n)
        vm = V.manufactured_fields(m.centres, 0.0, 3)[0]
        pe = api.PseudoECG(m, ELECTRODES, sigma=V.SIGMA, grad_scheme=grad)
        got = pe.compute(torch.tensor(vm, device="cuda"))
        pe.close()
        d = oracle.tissue_desc("TNNP", 1, grad_gauss=grad == lib.GRAD_GAUSS_LINEAR)
        o = oracle.Tissue(d, oracle.Mesh.general(m))
        o.set_conductivity(np.tile(np.asarray(V.SIGMA), (m.n_cells, 1)))
        want = o.pseudo_ecg(vm, ELECTRODES)
        assert np.all(np.abs(got - want) <= _tol(want)), (n, got, want)
        err.append(np.max(np.abs(got - ref)))
    assert V.rate(err[0], err[1], 8, 16) > 1.8 and V.rate(err[1], err[2], 16, 32) > 1.9


@pytest.mark.gpu
def test_manufactured_run_records_the_ecg(gpu_lib):
    """The tutorial's manufactured monodomain run (3D, 10 and 20 cells at the
    sweep's time steps) with the pseudo-ECG recorded every step: the error
    against sqrt(1 + t) times the quadrature reference falls at second order."""
    runs = [V.run(3, n, ecg=True) for n in (10, 20)]
    for r in runs:
        assert r["ecg"]["values"].shape == (r["steps"], 5)
    e = [np.max(r["ecg"]["Linf"]) for r in runs]
    assert V.rate(e[0], e[1], 10, 20) > 1.7, e


@pytest.mark.gpu
@ARITHMETIC
def test_many_electrodes_and_a_centre_electrode(gpu_lib, oracle, arith):
    """19 electrodes (three launches of up to 8), one of them exactly on a
    cell centre (that cell is skipped), an odd cell count (the tail of the
    paired loads) and a misaligned Vm."""
    torch = pytest.importorskip("torch")
    m = V.geometry_mesh_for(3, 11)
    assert m.n_cells % 2 == 1
    rng = np.random.default_rng(8)
    el = np.vstack([m.centres[[5, 300]], rng.uniform(-1.0, 2.0, (17, 3))])
    vm = rng.standard_normal(m.n_cells) * 0.02 - 0.08
    pe = api.PseudoECG(m, el, sigma=V.SIGMA, grad_scheme=lib.GRAD_GAUSS_LINEAR, arithmetic=arith)
    x = torch.tensor(vm, device="cuda")
    got = pe.compute(x)
    assert np.array_equal(got, pe.compute(x))
    d = oracle.tissue_desc("TNNP", 1, grad_gauss=True)
    o = oracle.Tissue(d, oracle.Mesh.general(m))
    o.set_conductivity(np.tile(np.asarray(V.SIGMA), (m.n_cells, 1)))
    want = o.pseudo_ecg(vm, el)
    assert np.all(np.abs(got - want) <= 1e-10 * np.abs(want).max())
    # Vm at an address that is not 16-byte aligned: the one-cell-per-load path
    xs = torch.tensor(np.r_[0.0, vm], device="cuda")[1:]
    assert xs.data_ptr() % 16 == 8
    got1 = pe.compute(xs)
    assert np.all(np.abs(got1 - want) <= 1e-10 * np.abs(want).max())
    pe.close()


@pytest.mark.gpu
def test_invalid_arguments(gpu_lib, small_lv):
    torch = pytest.importorskip("torch")
    m = V.geometry_mesh_for(3, 4)
    with pytest.raises(ValueError):
        api.PseudoECG(V.mesh_for(3, 4), ELECTRODES)          # no geometry
    with pytest.raises(lib.CfgError):
        api.PseudoECG(m, np.zeros((0, 3)))
    pe = api.PseudoECG(m, ELECTRODES)
    with pytest.raises(ValueError):
        pe.compute(torch.zeros(m.n_cells + 1, dtype=torch.float64, device="cuda"))
    md = api.Monodomain(small_lv.mesh, "TNNP", "epicardialCells", dt=DT, stencil=False)
    with pytest.raises(lib.CfgError):
        pe.compute(md)                                        # other cell count
    md.close()
    pe.close()


@pytest.mark.gpu
def test_float_pairs_against_fp64(gpu_lib, small_lv):
    """The two arithmetic forms on the same Vm: within 1e-12 of the largest
    electrode value, including a Vm with exact zeros and a uniform Vm (whose
    pseudo-ECG vanishes up to the rows' round-off)."""
    torch = pytest.importorskip("torch")
    L = small_lv
    el = _lv_electrodes(L)
    a = api.PseudoECG(L.mesh, el, conductivity_per_cell=L.conductivity,
                      arithmetic=lib.ECG_FLOAT_PAIRS)
    b = api.PseudoECG(L.mesh, el, conductivity_per_cell=L.conductivity, arithmetic=lib.ECG_FP64)
    rng = np.random.default_rng(3)
    vm = -0.084 + 0.12 * (L.mesh.centres[:, 2] > -0.03) + 1e-3 * rng.standard_normal(L.mesh.n_cells)
    vm[::7] = 0.0
    x = torch.tensor(vm, device="cuda")
    pa, pb = a.compute(x), b.compute(x)
    assert np.max(np.abs(pa - pb)) <= 1e-12 * np.max(np.abs(pb))
    flat = torch.full((L.mesh.n_cells,), -0.084, dtype=torch.float64, device="cuda")
    scale = np.max(np.abs(pb))
    assert np.max(np.abs(a.compute(flat))) <= 1e-12 * scale
    assert np.max(np.abs(b.compute(flat))) <= 1e-12 * scale
    a.close()
    b.close()


@pytest.mark.gpu
def test_bidomain_source(gpu_lib, oracle):
    """ECGDomain over a bidomain state (conductivity Gi, the context's Vm): the
    pseudo-ECG read from the Bidomain context equals the one of the same Vm
    as a tensor, and the oracle's on its own bidomain run."""
    torch = pytest.importorskip("torch")
    from cardiacfoam_gb300.mesh import box_mesh, with_box_geometry
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
    el = np.array([[-2e-3, 1e-3, 2.5e-4], [8e-3, 1e-3, 2.5e-4], [3e-3, -4e-3, 1e-3]])
    pe = api.PseudoECG(mesh, el, sigma=gi, max_rows=4)
    for _ in range(100):
        bd.step(dt)
        B.step(dt)
    got = pe.compute(bd)
    same = pe.compute(torch.tensor(bd.vm(), device="cuda"))
    assert np.array_equal(got, same)
    want = B.tissue.pseudo_ecg(B.tissue.vm(), el)
    assert np.all(np.abs(got - want) <= 1e-7 * np.max(np.abs(want)))
    pe.record(bd)
    t, v = pe.series()
    assert t[0] == bd.time() and np.array_equal(v[0], got)
    pe.close()
    # lead rows folded with another conductivity than the context's Gi
    wrong = api.PseudoECG(mesh, el, sigma=ge)
    with pytest.raises(ValueError):
        wrong.compute(bd)
    wrong.close()
    bd.close()
