"""General meshes and the corrected Laplacian on the CPU: the tetrahedral
left-ventricle generator (closure, orientation, volumes, fibres, cell types)
and the oracle's Gauss-linear-corrected Laplacian with a per-cell
conductivity tensor (linear-field exactness, box-as-general equality, the
whole tissue step on both forms of a box)."""
import numpy as np
import pytest

from cardiacfoam_gb300 import lv
from cardiacfoam_gb300.mesh import box_mesh, tet_mesh, tet_volumes6, with_box_geometry

SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
SIGMA_FULL = (0.12, 0.02, -0.01, 0.05, 0.015, 0.03)


@pytest.fixture(scope="module")
def small_lv():
    return lv.left_ventricle(4, 10, 12)


def _closure(m):
    S = np.zeros((m.n_cells, 3))
    np.add.at(S, m.owner, m.face_sf)
    np.add.at(S, m.neighbour, -m.face_sf)
    np.add.at(S, m.boundary_cell, m.boundary_sf)
    return np.abs(S).max() / np.abs(m.face_sf).max()


def test_single_tet_geometry():
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    m = tet_mesh(p, np.array([[0, 2, 1, 3]]))       # negative orientation is fixed
    assert m.n_faces == 0 and m.n_boundary_faces == 4
    assert abs(m.volumes[0] - 1.0 / 6.0) < 1e-15
    assert np.allclose(m.centres[0], 0.25)
    out = np.einsum("ij,ij->i", m.boundary_sf, m.boundary_centres - m.centres[0])
    assert np.all(out > 0)                                      # outward


def test_lv_mesh_is_closed_and_oriented(small_lv):
    m = small_lv.mesh
    nt, mm, nr = small_lv.dims
    assert m.n_cells == 6 * nt * (mm * mm + 4 * mm * nr)
    assert np.all(tet_volumes6(small_lv.points, small_lv.tets) > 0)
    assert _closure(m) < 1e-13
    key = m.owner.astype(np.int64) * m.n_cells + m.neighbour
    assert np.all(np.diff(key) > 0) and np.all(m.owner < m.neighbour)
    d = m.centres[m.neighbour] - m.centres[m.owner]
    assert np.all(np.einsum("ij,ij->i", d, m.face_sf) > 0)     # owner -> neighbour
    # every cell: 4 faces in all
    faces = np.bincount(m.owner, minlength=m.n_cells) + np.bincount(m.neighbour, minlength=m.n_cells)
    faces += np.bincount(m.boundary_cell, minlength=m.n_cells)
    assert np.all(faces == 4)


def test_lv_shape_and_quality():
    L = lv.left_ventricle(6, 20, 24)
    m = L.mesh
    exact = 0.5 * 4.0 / 3.0 * np.pi * ((35e-3) ** 2 * 70e-3 - (25e-3) ** 2 * 60e-3)
    assert abs(m.volumes.sum() / exact - 1.0) < 5e-3
    assert np.all(m.centres[:, 2] < 0.0)
    d = m.centres[m.neighbour] - m.centres[m.owner]
    cos = np.einsum("ij,ij->i", d, m.face_sf) / (np.linalg.norm(d, axis=1) *
                                                  np.linalg.norm(m.face_sf, axis=1))
    assert np.degrees(np.arccos(np.clip(cos.min(), -1, 1))) < 60.0
    v6 = tet_volumes6(L.points, L.tets)
    assert v6.min() > 0.2 * v6.mean()


def test_lv_fibres_and_conductivity(small_lv):
    L = small_lv
    f = L.fibre
    assert np.allclose(np.linalg.norm(f, axis=1), 1.0)
    # sigma f = sigma_l f, and sigma t = sigma_t t for t normal to f
    s = L.conductivity
    S = np.stack([s[:, [0, 1, 2]], s[:, [1, 3, 4]], s[:, [2, 4, 5]]], axis=1)
    assert np.allclose(np.einsum("nij,nj->ni", S, f), lv.SIGMA_L * f)
    t = np.cross(f, np.array([0.3, -0.5, 0.8]))
    t /= np.linalg.norm(t, axis=1)[:, None]
    assert np.allclose(np.einsum("nij,nj->ni", S, t), lv.SIGMA_T * t)
    # the fibre angle follows the transmural fraction: +60 deg at the
    # endocardium to -60 deg at the epicardium, measured from e_l towards e_n
    x = L.mesh.centres
    a = lv.ENDO_A + L.transmural * lv.WALL
    c = lv.ENDO_C + L.transmural * lv.WALL
    et = np.stack([x[:, 0] / a ** 2, x[:, 1] / a ** 2, x[:, 2] / c ** 2], axis=1)
    et /= np.linalg.norm(et, axis=1)[:, None]
    assert np.abs(np.einsum("ij,ij->i", f, et)).max() < 1e-12
    far = np.hypot(x[:, 0], x[:, 1]) > 5e-3                      # away from the apex axis
    en = np.array([0, 0, 1.0]) - et[:, 2:3] * et
    en /= np.linalg.norm(en, axis=1)[:, None]
    el = np.cross(en, et)
    alpha = np.arctan2(np.einsum("ij,ij->i", f, en), np.einsum("ij,ij->i", f, el))
    expect = np.deg2rad(60.0) * (1 - L.transmural) + np.deg2rad(-60.0) * L.transmural
    assert np.abs(alpha - expect)[far].max() < 1e-9
    # cell types by transmural fraction
    s_ = L.transmural
    assert np.all(L.tissue[s_ < 0.3] == 3) and np.all(L.tissue[(s_ >= 0.3) & (s_ < 0.6)] == 2)
    assert np.all(L.tissue[s_ >= 0.6] == 1)


def test_config_size_is_four_million_tets():
    nt, m, nr = lv.config_sizes()
    n = 6 * nt * (m * m + 4 * m * nr)
    assert abs(n - 4.0e6) < 0.05e6


def test_apex_box_holds_cells(small_lv):
    lo, hi = small_lv.apex_box(8e-3)          # cells of the small mesh are ~3 mm
    x = small_lv.mesh.centres
    inside = np.all((x >= lo) & (x <= hi), axis=1)
    assert inside.sum() > 0


# ------------------------------------------------------------- oracle

def test_box_through_the_general_path_matches(oracle):
    nx, ny, nz, lx, ly, lz = 8, 6, 5, 0.004, 0.003, 0.0025
    bm = box_mesh(nx, ny, nz, lx, ly, lz)
    gm = with_box_geometry(bm, lx, ly, lz)
    assert _closure(gm) == 0.0
    Tb = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA), oracle.Mesh(nx, ny, nz, lx, ly, lz))
    Tg = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA), oracle.Mesh.general(gm))
    phi = np.random.default_rng(0).standard_normal(bm.n_cells)
    a, b = Tb.laplacian(phi), Tg.laplacian(phi)
    assert np.abs(a - b).max() <= 1e-14 * np.abs(a).max()


def test_box_step_through_the_general_path_matches(oracle):
    """Whole tissue steps (ionic, corrected implicit diffusion, PIMPLE) on
    the box as a structured and as a general mesh: the corrections vanish
    to round-off on an orthogonal mesh with a diagonal tensor."""
    nx, ny, nz = 10, 4, 3
    h = 2.5e-4
    lx, ly, lz = nx * h, ny * h, nz * h
    boxes = [((0, 0, 0), (3 * h, 2 * h, 2 * h), 0.0, 2e-3, 5e4)]
    runs = []
    for mesh in (oracle.Mesh(nx, ny, nz, lx, ly, lz),
                 oracle.Mesh.general(with_box_geometry(box_mesh(nx, ny, nz, lx, ly, lz),
                                                       lx, ly, lz))):
        T = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA, boxes=boxes), mesh)
        for _ in range(40):
            T.step(2e-5)
        runs.append((T.vm(), T.solves()[2]))
    (va, ia), (vb, ib) = runs
    assert np.abs(va - vb).max() <= 1e-11 * np.abs(va).max()
    assert np.abs(ia.astype(int) - ib.astype(int)).max() <= 1


def test_linear_field_is_exact_in_the_interior(oracle, small_lv):
    m = small_lv.mesh
    gvec = np.array([3.0, -2.0, 1.5])
    phi = m.centres @ gvec
    bnd = np.zeros(m.n_cells, bool)
    bnd[m.boundary_cell] = True
    near = bnd.copy()
    near[m.owner[bnd[m.neighbour]]] = True
    near[m.neighbour[bnd[m.owner]]] = True
    scale = np.abs(gvec).max() * 0.12 / np.cbrt(m.volumes).mean()
    T = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA_FULL), oracle.Mesh.general(m))
    assert np.abs(T.gradient(phi)[~bnd] - gvec).max() < 1e-12
    assert np.abs(T.laplacian(phi)[~near]).max() < 1e-11 * scale
    # without the non-orthogonal correction the tets see O(1) errors
    Tu = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA_FULL, uncorrected=True),
                       oracle.Mesh.general(m))
    assert np.abs(Tu.laplacian(phi)[~near]).max() > 0.1 * scale


def test_per_cell_conductivity_equal_to_uniform(oracle, small_lv):
    m = small_lv.mesh
    T0 = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA_FULL), oracle.Mesh.general(m))
    T1 = oracle.Tissue(oracle.tissue_desc(sigma=SIGMA), oracle.Mesh.general(m))
    T1.set_conductivity(np.tile(SIGMA_FULL, (m.n_cells, 1)))
    phi = np.random.default_rng(2).standard_normal(m.n_cells)
    a, b = T0.laplacian(phi), T1.laplacian(phi)
    assert np.array_equal(a, b)


def test_lv_tissue_steps_with_cell_types(oracle, small_lv):
    """A few steps of the LV tissue with per-cell sigma and TNNP cell types:
    the stimulated apex depolarises, PCG converges, and a cell's ionic
    constants follow its type (M cells' g_Ks differs from endo/epi)."""
    L = small_lv
    m = L.mesh
    lo, hi = L.apex_box(8e-3)
    T = oracle.Tissue(oracle.tissue_desc(model="TNNP", boxes=[(lo, hi, 0.0, 2e-3, 5e4)]),
                      oracle.Mesh.general(m))
    T.set_conductivity(L.conductivity)
    T.set_cell_tissue(L.tissue)
    for _ in range(30):
        T.step(5e-5)
    vm = T.vm()
    x = m.centres
    inside = np.all((x >= lo) & (x <= hi), axis=1)
    assert inside.any() and vm[inside].max() > vm[~inside].max() - 1e-12
    assert vm[inside].max() > -0.06
    ir, fr, it = T.solves()
    assert np.all(fr < 1e-8)
