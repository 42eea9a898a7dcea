"""Pseudo-ECG on the CPU: the oracle's restatement of PseudoECGSolver::compute
against the manufactured-solution reference of the reference's own verifier
(Gauss-Legendre quadrature of the exact dipole integral), the electrode
reader of the C library, and the ecgModelIO time-series format."""

import numpy as np
import pytest

from cardiacfoam_gb300 import io, verification as V

ELECTRODES = [p for _, p in V.ECG_ELECTRODES]


def _oracle_tissue(oracle, mesh, gauss=True, sigma=V.SIGMA):
    d = oracle.tissue_desc("TNNP", 1, grad_gauss=gauss)
    t = oracle.Tissue(d, oracle.Mesh.general(mesh))
    t.set_conductivity(np.tile(np.asarray(sigma, dtype=np.float64), (mesh.n_cells, 1)))
    return t


def test_quadrature_rule():
    """The rule is exact for polynomials up to degree 2n-1, and the
    reference order (96) agrees with order 48 on the dipole integral to
    round-off (the verifier's deltaQuadrature columns)."""
    x, w = V.gauss_legendre(7)
    for k in range(14):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs((w * x ** k).sum() - exact) < 1e-14
    r96 = V.pseudo_ecg_spatial_reference(ELECTRODES, 3, 96)
    r48 = V.pseudo_ecg_spatial_reference(ELECTRODES, 3, 48)
    assert np.max(np.abs(r96 - r48)) < 1e-14
    # E1 and E2 sit on the symmetry plane of cos(2 pi y) cos(3 pi z): zero
    assert np.all(np.abs(r96[:2]) < 1e-15) and np.all(np.abs(r96[2:]) > 1e-4)
    with pytest.raises(ValueError):
        V.gauss_legendre(0)


@pytest.mark.parametrize("gauss", [True, False], ids=["gauss-linear", "least-squares"])
def test_oracle_converges_to_quadrature_reference(oracle, gauss):
    """The cell sum of the exact field's finite-volume dipoles approaches the
    dipole integral at second order (8 -> 16 cells per direction)."""
    ref = V.pseudo_ecg_spatial_reference(ELECTRODES, 3, 96)
    err = []
    for n in (8, 16):
        m = V.geometry_mesh_for(3, n)
        vm = V.manufactured_fields(m.centres, 0.0, 3)[0]
        err.append(np.max(np.abs(_oracle_tissue(oracle, m, gauss).pseudo_ecg(vm, ELECTRODES) - ref)))
    assert err[1] < 0.05 * np.max(np.abs(ref))
    assert V.rate(err[0], err[1], 8, 16) > 1.8


def test_oracle_matches_its_gradient(oracle):
    """The oracle's sum restated from its own cell gradient, with an electrode
    placed exactly on a cell centre (that cell is skipped: |r| <= VSMALL)."""
    m = V.geometry_mesh_for(3, 6)
    rng = np.random.default_rng(4)
    vm = rng.standard_normal(m.n_cells)
    el = np.array([m.centres[17], [1.4, 0.3, 0.2], [-0.3, -0.2, 1.1]])
    t = _oracle_tissue(oracle, m, gauss=True)
    got = t.pseudo_ecg(vm, el)
    g = t.gradient(vm)
    S = np.array([[V.SIGMA[0], V.SIGMA[1], V.SIGMA[2]], [V.SIGMA[1], V.SIGMA[3], V.SIGMA[4]],
                  [V.SIGMA[2], V.SIGMA[4], V.SIGMA[5]]])
    dip = (g @ S.T) * m.volumes[:, None]
    want = []
    for p in el:
        r = m.centres - p
        mag = np.sqrt((r * r).sum(axis=1))
        ok = mag > 1e-300
        want.append(((dip[ok] * r[ok]).sum(axis=1) / mag[ok] ** 3).sum())
    assert np.allclose(got, want, rtol=1e-12, atol=0)


ELECTRO_PROPERTIES = """
myocardiumSolver  monodomainSolver;
monodomainSolverCoeffs
{
    conductivity [-1 -3 3 0 0 2 0] (0.1 0 0 0.1 0 0.1);
    ecgDomains
    {
        torso
        {
            ecgSolver    pseudoECG;
            electrodePositions
            {
                V2    (0.01 -0.02 0.03);
                LA    (1.5 0.5 0.5);   // comment
                V1    (-1e-2 2 3e-1);
            }
        }
        bath
        {
            ecgSolver    bidomainBathECG;
        }
    }
}
"""


def test_electrodes_from_dict(gpu_lib):
    from cardiacfoam_gb300 import api, lib
    names, pos = api.ecg_electrodes(ELECTRO_PROPERTIES)
    assert names == ["V2", "LA", "V1"]     # the dictionary's order
    assert np.array_equal(pos, [[0.01, -0.02, 0.03], [1.5, 0.5, 0.5], [-1e-2, 2, 3e-1]])
    assert api.ecg_electrodes(ELECTRO_PROPERTIES, "torso")[0] == names
    with pytest.raises(lib.CfgError) as e:
        api.ecg_electrodes(ELECTRO_PROPERTIES, "bath")
    assert e.value.code == lib.CFG_ERR_UNSUPPORTED
    with pytest.raises(lib.CfgError):
        api.ecg_electrodes(ELECTRO_PROPERTIES, "missing")
    with pytest.raises(lib.CfgError):
        api.ecg_electrodes("myocardiumSolver monodomainSolver; monodomainSolverCoeffs { }")
    bad = ELECTRO_PROPERTIES.replace("(1.5 0.5 0.5)", "(1.5 0.5)")
    with pytest.raises(lib.CfgError):
        api.ecg_electrodes(bad)


def test_ecg_time_series_format(tmp_path):
    path = io.write_pseudo_ecg(tmp_path, ["E1", "E2"], [0.0, 0.1],
                               [[1.5e-3, -2.25], [0.0, 123456.789]])
    assert path == tmp_path / "postProcessing" / "pseudoECG.dat"
    assert path.read_text() == ("# time  E1  E2\n"
                                "0.00000000e+00  1.50000000e-03  -2.25000000e+00\n"
                                "1.00000000e-01  0.00000000e+00  1.23456789e+05\n")


def test_create_rejects_bad_arguments(gpu_lib):
    """cfg_pseudo_ecg_create's argument checks, made before any device work."""
    import ctypes as C
    from cardiacfoam_gb300 import api, lib
    from cardiacfoam_gb300.mesh import box_mesh
    geo = V.geometry_mesh_for(3, 4)
    el = np.ascontiguousarray(ELECTRODES, dtype=np.float64)

    def create(mesh, n_el=5, grad=lib.GRAD_GAUSS_LINEAR, arith=lib.ECG_FLOAT_PAIRS, rows=0):
        d = lib.PseudoEcgDesc()
        for i, v in enumerate(V.SIGMA):
            d.conductivity[i] = v
        d.grad_scheme, d.n_electrodes, d.max_rows, d.arithmetic = grad, n_el, rows, arith
        d.electrodes = lib.dptr(el)
        md, keep = api.mesh_desc(mesh, structured=False)
        h = C.c_void_p()
        return gpu_lib.cfg_pseudo_ecg_create(C.byref(d), C.byref(md), C.byref(h))

    assert create(box_mesh(4, 4, 4, 1.0, 1.0, 1.0)) == lib.CFG_ERR_INVALID    # no geometry
    assert create(geo, n_el=0) == lib.CFG_ERR_INVALID
    assert create(geo, grad=7) == lib.CFG_ERR_INVALID
    assert create(geo, arith=9) == lib.CFG_ERR_INVALID
    assert create(geo, rows=-1) == lib.CFG_ERR_INVALID
