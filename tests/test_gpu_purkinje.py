"""The Purkinje network on the GPU (cfg_purkinje_*) against the oracle's
restatement of Monodomain1DSolver and of the reaction-diffusion PVJ
coupling, through the C ABI."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, io, lib
from cardiacfoam_gb300.mesh import box_mesh

SIGMA = (0.1334177215, 0.0, 0.0, 0.01760617761, 0.0, 0.01760617761)


@pytest.mark.gpu
def test_network_alone_matches_oracle(gpu_lib, oracle):
    """A branching tree (5 generations, 254 edges), BuenoOrovio nodes, root
    stimulus: Vm and Iion of every node within 1e-9 of the field scale after
    the wave has run through the tree (level-parallel elimination on the
    device, node-by-node elimination in the oracle)."""
    dt = 1e-5
    e, pos, leaves = io.synthetic_purkinje_tree(5, 4, 2.5e-4)
    g = api.Purkinje(e, "BuenoOrovio", "epicardialCells", dt=dt,
                     root_stimulus=(0, 0.0, 2e-3, 5e5))
    o = oracle.Purkinje(e, "BuenoOrovio", 1, dt, root_stimulus=(0.0, 2e-3, 5e5))
    assert np.array_equal(g.vm(), o.vm())          # the model's resting Vm
    for s in range(1500):
        g.step(dt)
        o.advance(dt)
        if (s + 1) % 300 == 0:
            vg, vo = g.vm(), o.vm()
            assert np.max(np.abs(vg - vo)) <= 1e-9 * np.max(np.abs(vo)), s
    assert np.max(o.vm()) > 0.0                     # the tree depolarised
    ig, io_ = g.iion(), o.iion()
    assert np.max(np.abs(ig - io_)) <= 1e-9 * np.max(np.abs(io_))
    assert abs(g.time() - o.t) < 1e-15
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bidirectional", [False, True], ids=["unidirectional", "bidirectional"])
def test_coupled_slab_matches_oracle(gpu_lib, oracle, bidirectional):
    """A network whose two terminals end inside a BuenoOrovio slab, coupled
    through reactionDiffusionPvjCoupler (rPvj 1e4, pvjRadius 0.4 mm): the
    tissue's Vm and activation times, the network's Vm and the terminal
    currents against the oracle's staggered coupled step."""
    h, dt = 2.5e-4, 1e-5
    nx, ny, nz = 24, 12, 2
    mesh = box_mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    md = api.Monodomain(mesh, "BuenoOrovio", "epicardialCells", SIGMA, dt=dt, n_outer=1,
                        outer_tol=0.0, stencil=False)
    e, pos, leaves = io.synthetic_purkinje_tree(1, 8, h, origin=(0.5e-3, 1.5e-3, 2.5e-4))
    pk = api.Purkinje(e, "BuenoOrovio", "epicardialCells", dt=dt,
                      root_stimulus=(0, 0.0, 2e-3, 5e5), pvj_nodes=leaves,
                      pvj_locations=pos[leaves])
    pk.couple(md, 1e4, 4e-4, bidirectional=bidirectional)
    om = oracle.Mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    d = oracle.tissue_desc("BuenoOrovio", 1, SIGMA, implicit=True, precond_dic=False,
                           n_outer=1, outer_tol=0.0)
    T = oracle.Tissue(d, om)
    P = oracle.Purkinje(e, "BuenoOrovio", 1, dt, root_stimulus=(0.0, 2e-3, 5e5),
                        pvj_nodes=leaves, pvj_locations=pos[leaves])
    P.couple(om, 1e4, 4e-4, bidirectional=bidirectional)
    for s in range(1200):
        md.step(dt)
        P.coupled_step(T, dt)
    vg, vo = md.vm(), T.vm()
    assert np.max(np.abs(vg - vo)) <= 1e-9 * np.max(np.abs(vo))
    ag, ao = md.activation(), T.activation()
    assert np.array_equal(ag > 0, ao > 0) and np.sum(ao > 0) > 10
    assert np.max(np.abs(ag - ao)) < 1e-9
    pv, po = pk.vm(), P.vm()
    assert np.max(np.abs(pv - po)) <= 1e-9 * np.max(np.abs(po))
    ig, io_ = pk.terminal_current(), P.terminal_current()
    assert np.max(np.abs(ig - io_)) <= 1e-9 * max(np.max(np.abs(io_)), 1e-300)
    with pytest.raises(lib.CfgError):
        pk.step(dt)                      # a coupled network steps with its context
    pk.close()
    md.step(dt)                          # the context goes on without the network
    md.close()


@pytest.mark.gpu
def test_network_argument_checks(gpu_lib):
    e, pos, leaves = io.synthetic_purkinje_tree(1, 3, 2.5e-4)
    with pytest.raises(lib.CfgError):          # a cycle: N edges for N nodes
        api.Purkinje(np.vstack([e, [[1, 3, 2.5e-4, 1.0]]]), "BuenoOrovio", "epicardialCells")
    mesh = box_mesh(8, 8, 2, 4e-3, 4e-3, 1e-3)
    md = api.Monodomain(mesh, "BuenoOrovio", "epicardialCells", SIGMA, stencil=False)
    pk = api.Purkinje(e, "BuenoOrovio", "epicardialCells", pvj_nodes=leaves,
                      pvj_locations=pos[leaves])
    with pytest.raises(lib.CfgError) as err:   # pvjRadius below the cell size (0.5 mm)
        pk.couple(md, 1e4, 1e-4)
    assert "pvjRadius" in str(err.value)
    pk.close()
    md.close()


@pytest.mark.gpu
def test_niederer_purkinje_tutorial_matches_oracle(gpu_lib, oracle):
    """The reference's Purkinje tutorial (tutorials/Niederer/
    NiedererEtAl2011MonodomainPurkinje): its 193-node graph (fixture from
    its purkinjeGraph), BuenoOrovio epicardial nodes, root stimulus 5e5 at
    10-12 ms, unidirectional reactionDiffusionPvjCoupler (rPvj 1e4,
    pvjRadius 0.3 mm) into the Niederer slab (100 x 15 x 35 cells of 0.2 mm,
    explicit algorithm at the maxCo 0.1 time step, no box stimulus).  Over
    24 ms the network fires, its eight terminals excite the tissue, and the
    tissue's Vm and activation times, the network's Vm and the terminal
    currents equal the oracle's coupled step."""
    import os
    from pathlib import Path
    g = np.load(Path(__file__).parent / "golden" / "niederer_purkinje_graph.npz")
    nx, ny, nz, lx, ly, lz = 100, 15, 35, 0.02, 0.003, 0.007
    chicm = 140000 * 0.01
    dt = 0.1 * (lx / nx) ** 2 / (SIGMA[0] / chicm)
    mesh = box_mesh(nx, ny, nz, lx, ly, lz)
    md = api.Monodomain(mesh, "BuenoOrovio", "epicardialCells", SIGMA, dt=dt, implicit=False)
    root = (int(g["root"]), 0.01, 2e-3, 5e5)
    pk = api.Purkinje(g["edges"], "BuenoOrovio", "epicardialCells", dt=dt, chi=140000.0,
                      cm=0.01, root_stimulus=root, pvj_nodes=g["pvj_nodes"],
                      pvj_locations=g["pvj_locations"])
    pk.couple(md, 1e4, 3e-4)
    om = oracle.Mesh(nx, ny, nz, lx, ly, lz)
    T = oracle.Tissue(oracle.tissue_desc("BuenoOrovio", 1, SIGMA, implicit=False), om)
    P = oracle.Purkinje(g["edges"], "BuenoOrovio", 1, dt, root_stimulus=root[1:],
                        pvj_nodes=g["pvj_nodes"], pvj_locations=g["pvj_locations"])
    P.couple(om, 1e4, 3e-4)
    threads = os.cpu_count() or 1
    for _ in range(int(0.024 / dt)):
        md.step(dt)
        P.coupled_step(T, dt, threads)
    assert np.all(P.vm()[g["pvj_nodes"]] > -0.084)       # the terminals fired
    vg, vo = md.vm(), T.vm()
    assert np.max(np.abs(vg - vo)) <= 1e-9 * np.max(np.abs(vo))
    ag, ao = md.activation(), T.activation()
    assert np.array_equal(ag > 0, ao > 0) and np.sum(ao > 0) > 50
    assert np.max(np.abs(ag - ao)) < 1e-9
    pv, po = pk.vm(), P.vm()
    assert np.max(np.abs(pv - po)) <= 1e-9 * np.max(np.abs(po))
    ig, io_ = pk.terminal_current(), P.terminal_current()
    assert np.max(np.abs(ig - io_)) <= 1e-9 * max(np.max(np.abs(io_)), 1e-300)
    pk.close()
    md.close()
