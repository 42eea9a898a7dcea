"""Purkinje network on the CPU: the graph file reader, the oracle's
restatement of Monodomain1DSolver (Hines elimination over the tree) and of
the reaction-diffusion PVJ coupling."""
import numpy as np
import pytest

from cardiacfoam_gb300 import io

GRAPH = """
FoamFile { version 2.0; format ascii; class dictionary; object purkinjeGraph; }
// a trunk of three edges and two branches of two
rootNode 0;
pvjNodes 2(5 7);
pvjLocations 2((0.004 0.001 0.0005) (0.004 -0.001 0.0005));
conductionEdges
7
(
4(0 1 0.001 1)
4(1 2 0.001 1)
4(2 3 0.001 1)
4(3 4 0.001 0.5)
4(4 5 0.001 0.5)
4(3 6 0.001 0.5)
(6 7 1e-3 5e-1)
);
"""


def test_graph_reader():
    g = io.read_purkinje_graph(GRAPH)
    assert g["root"] == 0
    assert g["edges"].shape == (7, 4)
    assert np.array_equal(g["edges"][6], [6, 7, 1e-3, 0.5])
    assert list(g["pvj_nodes"]) == [5, 7]
    assert np.allclose(g["pvj_locations"][1], [0.004, -0.001, 0.0005])
    with pytest.raises(ValueError):
        io.read_purkinje_graph(GRAPH.replace("4(0 1 0.001 1)", "3(0 1 0.001)"))


def test_tutorial_graph_fixture():
    """The reference Purkinje tutorial's graph (fixture made from its
    purkinjeGraph by tests/golden/make_purkinje_fixture.py): 192 edges of a
    193-node tree rooted at node 0, eight PVJs inside the Niederer slab; the
    reader gives the same arrays from the file itself where the reference
    is at hand."""
    from pathlib import Path
    from oracle.build import reference_dir
    g = np.load(Path(__file__).parent / "golden" / "niederer_purkinje_graph.npz")
    e = g["edges"]
    assert e.shape == (192, 4) and int(g["root"]) == 0
    nodes = np.unique(e[:, :2].astype(int))
    assert nodes.size == 193 and nodes[0] == 0 and nodes[-1] == 192
    assert list(g["pvj_nodes"]) == list(range(8, 16))
    assert np.all((g["pvj_locations"] > 0) & (g["pvj_locations"] < [0.02, 0.003, 0.007]))
    ref = reference_dir()
    if ref is not None:
        f = Path(ref) / "tutorials/Niederer/NiedererEtAl2011MonodomainPurkinje/constant/purkinjeGraph"
        r = io.read_purkinje_graph(f.read_text())
        assert np.array_equal(r["edges"], e)
        assert np.array_equal(r["pvj_locations"], g["pvj_locations"])


def test_synthetic_tree_is_a_tree():
    e, pos, leaves = io.synthetic_purkinje_tree(3, 4, 2.5e-4)
    n = len(pos)
    assert len(e) == n - 1
    assert leaves.size == 8
    assert np.allclose(np.linalg.norm(pos[e[:, 1].astype(int)] - pos[e[:, 0].astype(int)],
                                      axis=1), 2.5e-4)


def test_oracle_network_propagates_from_the_root(oracle):
    """A root stimulus excites the whole tree; along each path from the root
    the nodes depolarise in order of their distance (the cable step over
    the tree, solved by elimination)."""
    e, pos, leaves = io.synthetic_purkinje_tree(3, 6, 2.5e-4)
    P = oracle.Purkinje(e, "BuenoOrovio", 1, 1e-5, root_stimulus=(0.0, 2e-3, 5e5))
    n = P.n
    first = np.full(n, np.inf)
    for s in range(2500):
        P.advance(1e-5)
        v = P.vm()
        newly = (v > 0.0) & ~np.isfinite(first)
        first[newly] = P.t
    assert np.all(np.isfinite(first))
    # path from a leaf to the root: activation times decrease towards the root
    parent = {int(b): int(a) for a, b, _, _ in e}
    for leaf in leaves:
        path, v = [], int(leaf)
        while v != 0:
            path.append(v)
            v = parent[v]
        t = first[path]
        assert np.all(np.diff(t) <= 1e-12)


def test_oracle_coupling_deposits_into_the_tissue(oracle):
    """A bidirectional coupling between a network ending in a slab and the
    slab: the terminal currents are (Vnet - Vtissue)/R and the tissue under
    a terminal depolarises when the network does."""
    h = 2.5e-4
    nx, ny, nz = 24, 12, 2
    mesh = oracle.Mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    # one corrector: the slab starts uniform, where residualControl's
    # normalised residual is not meaningful
    d = oracle.tissue_desc("BuenoOrovio", 1, (0.1334177215, 0, 0, 0.01760617761, 0,
                                              0.01760617761), implicit=True, precond_dic=False,
                           n_outer=1, outer_tol=0.0)
    T = oracle.Tissue(d, mesh)
    e, pos, leaves = io.synthetic_purkinje_tree(1, 8, h, origin=(0.5e-3, 1.5e-3, 2.5e-4))
    P = oracle.Purkinje(e, "BuenoOrovio", 1, 1e-5, root_stimulus=(0.0, 2e-3, 5e5),
                        pvj_nodes=leaves, pvj_locations=pos[leaves])
    P.couple(mesh, 1e4, 4e-4, bidirectional=True)
    for _ in range(800):
        P.coupled_step(T, 1e-5)
    act = T.activation()
    assert np.sum(act > 0) > 10          # the tissue was activated through the junctions
    I = P.terminal_current()
    assert I.shape == (leaves.size,) and np.all(np.isfinite(I))
