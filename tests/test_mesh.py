import numpy as np

from cardiacfoam_gb300.mesh import box_mesh, slab


def test_box_mesh_matches_oracle(oracle):
    m = box_mesh(7, 5, 3, 0.007, 0.005, 0.003)
    om = oracle.Mesh(7, 5, 3, 0.007, 0.005, 0.003)
    o, nb = om.addressing()
    assert np.array_equal(o, m.owner) and np.array_equal(nb, m.neighbour)
    assert np.array_equal(om.centres(), m.centres)


def test_upper_triangular_order():
    m = box_mesh(6, 4, 3, 1.0, 1.0, 1.0)
    key = m.owner.astype(np.int64) * m.n_cells + m.neighbour
    assert np.all(np.diff(key) > 0)
    assert np.all(m.owner < m.neighbour)


def test_slab_sizes():
    m = slab(0.5)
    assert (m.n_cells, m.structured) == (3360, (40, 14, 6))
    assert m.n_faces == 39 * 14 * 6 + 40 * 13 * 6 + 40 * 14 * 5
