"""GPU monodomain step (cfg_monodomain_* through the C ABI) against the oracle."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from cardiacfoam_gb300.mesh import box_mesh

SIGMA = (0.1334, 0.0, 0.0, 0.0176, 0.0, 0.0176)
BOX = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, 1.5e-3), 0.0, 2e-3, 5e4)]


def run_pair(oracle, model, tissue, nsteps, dt=1e-5, implicit=True, precond_dic=False,
             precision=lib.PRECISION_FP64, dims=(20, 7, 3), h=1e-3, stencil=True,
             pcg_tol=1e-8):
    nx, ny, nz = dims
    mesh = box_mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    g = api.Monodomain(mesh, model, tissue, SIGMA, dt=dt, precision=precision,
                       implicit=implicit, boxes=BOX, stencil=stencil, pcg_tol=pcg_tol)
    om = oracle.Mesh(nx, ny, nz, nx * h, ny * h, nz * h)
    d = oracle.tissue_desc(model, api.TISSUE_FLAGS[tissue], SIGMA, implicit=implicit,
                           precond_dic=precond_dic, boxes=BOX, pcg_tol=pcg_tol)
    o = oracle.Tissue(d, om)
    stats = []
    for s in range(nsteps):
        g.step(dt)
        o.step(dt, 4)
        if implicit:
            stats.append((g.stats(), o.solves()))
    return g, o, stats


@pytest.mark.gpu
@pytest.mark.parametrize("model,tissue", [("TNNP", "epicardialCells"), ("ORd", "myocyte")])
def test_implicit_fp64_matches_oracle_same_preconditioner(gpu_lib, oracle, model, tissue):
    g, o, stats = run_pair(oracle, model, tissue, 300)
    vg, vo = g.vm(), o.vm()
    assert np.max(np.abs(vg - vo) / np.abs(vo)) < 1e-9
    ag, ao = g.activation(), o.activation()
    assert np.array_equal(ag > 0, ao > 0)
    assert np.max(np.abs(ag - ao)) < 1e-9
    for (gi, gf, git), (oi, of, oit) in stats:
        assert len(git) == len(oit)
        assert np.array_equal(git, oit)
        # residuals agree to 1e-6 where they are resolved; below the PCG
        # tolerance they are round-off of the converged field
        big = np.maximum(np.abs(gi), np.abs(oi)) > 1e-9
        assert np.allclose(gi[big], oi[big], rtol=1e-6)
        assert np.all(gi[~big] < 1e-8) and np.all(oi[~big] < 1e-8)
    assert abs(g.time() - o.time()) == 0.0


@pytest.mark.gpu
def test_implicit_fp64_against_dic_reference_solver(gpu_lib, oracle):
    """The reference's own preconditioner (DIC) converges to the same field
    within the PCG tolerance."""
    g, o, _ = run_pair(oracle, "TNNP", "epicardialCells", 300, precond_dic=True)
    vg, vo = g.vm(), o.vm()
    assert np.max(np.abs(vg - vo) / np.abs(vo)) < 1e-6
    ag, ao = g.activation(), o.activation()
    assert np.array_equal(ag > 0, ao > 0)
    assert np.max(np.abs(ag - ao)) <= 1e-5       # within one dt


@pytest.mark.gpu
def test_general_ell_operator_matches_stencil(gpu_lib, oracle):
    g1, o, _ = run_pair(oracle, "TNNP", "epicardialCells", 100, stencil=False)
    assert np.max(np.abs(g1.vm() - o.vm()) / np.abs(o.vm())) < 1e-9


@pytest.mark.gpu
def test_explicit_fp64_matches_oracle(gpu_lib, oracle):
    g, o, _ = run_pair(oracle, "TNNP", "epicardialCells", 300, implicit=False)
    vg, vo = g.vm(), o.vm()
    assert np.max(np.abs(vg - vo) / np.abs(vo)) < 1e-9
    assert np.max(np.abs(g.activation() - o.activation())) < 1e-9


@pytest.mark.gpu
def test_mixed_precision_activation_error(gpu_lib, oracle):
    dims, h, dt, n = (20, 7, 3), 1e-3, 1e-5, 1500
    mesh = box_mesh(*dims, dims[0] * h, dims[1] * h, dims[2] * h)
    a = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX)
    b = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX,
                       precision=lib.PRECISION_MIXED)
    for s in range(n):
        a.step(dt)
        b.step(dt)
    aa, ab = a.activation(), b.activation()
    assert np.array_equal(aa > 0, ab > 0)
    assert np.max(np.abs(aa - ab)) <= 5e-5          # <= 0.05 ms


@pytest.mark.gpu
def test_dictionary_front_end_equals_direct(gpu_lib):
    text = """
myocardiumSolver  monodomainSolver;
monodomainSolverCoeffs
{
    conductivity [-1 -3 3 0 0 2 0] (0.1334 0 0 0.0176 0 0.0176);
    chi   [0 -1 0 0 0 0 0] 140000;
    cm    [-1 -4 4 0 0 2 0] 0.01;
    ionicModel    TNNP;
    tissue    epicardialCells;
    solutionAlgorithm implicit;
    solver RKF45;
    maxSteps 1000000000;
    externalStimulus
    {
        stimulusLocationMin (0 0 0);
        stimulusLocationMax (1.5e-3 1.5e-3 1.5e-3);
        stimulusDuration [0 0 1 0 0 0 0] 2e-3;
        stimulusIntensity [0 -3 0 0 0 1 0] 50000;
        stimulusStartTime 0.0;
    }
}
"""
    dt = 1e-5
    mesh = box_mesh(20, 7, 3, 0.02, 0.007, 0.003)
    a = api.Monodomain.from_dict(text, mesh, dt)
    b = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX)
    for _ in range(50):
        a.step(dt)
        b.step(dt)
    assert np.array_equal(a.vm(), b.vm())
    assert np.array_equal(a.source(), b.source())


@pytest.mark.gpu
@pytest.mark.parametrize("implicit", [True, False])
def test_step_graph_equals_host_control(gpu_lib, implicit):
    """The step graph (device-driven PIMPLE/PCG loops) gives the same fields
    and solver statistics as host-driven control, and run(n) equals n steps."""
    dt, nsteps = 1e-5, 120
    mesh = box_mesh(20, 7, 3, 0.02, 0.007, 0.003)
    runs = []
    for mode in ("graph", "host", "run"):
        m = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX,
                           implicit=implicit)
        if mode == "host":
            m.set_graph(False)
        if mode == "run":
            m.run(dt, nsteps)
        else:
            for _ in range(nsteps):
                m.step(dt)
        runs.append((m.vm(), m.activation(), m.stats(), m.time()))
    (v0, a0, s0, t0), (v1, a1, s1, t1), (v2, a2, s2, t2) = runs
    assert np.array_equal(v0, v1) and np.array_equal(v0, v2)
    assert np.array_equal(a0, a1) and np.array_equal(a0, a2)
    if implicit:
        assert np.array_equal(s0[2], s1[2]) and np.array_equal(s0[2], s2[2])
    assert t0 == t1 == t2


@pytest.mark.gpu
@pytest.mark.parametrize("stencil", [True, False], ids=["stencil", "ell"])
def test_persistent_diffusion_equals_kernel_sequence(gpu_lib, stencil):
    """One persistent cooperative kernel per step (all correctors and PCG
    iterations in one launch) against the kernel sequence per iteration:
    the same solve up to the order of the reduction sums."""
    dt, nsteps = 1e-5, 150
    mesh = box_mesh(20, 7, 3, 0.02, 0.007, 0.003)
    runs = []
    for persistent in (True, False):
        m = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX,
                           stencil=stencil)
        m.set_persistent(persistent)
        iters = 0
        for _ in range(nsteps):
            m.step(dt)
            iters += int(np.sum(m.stats()[2]))
        runs.append((m.vm(), m.activation(), iters))
    (v0, a0, i0), (v1, a1, i1) = runs
    assert np.max(np.abs(v0 - v1)) <= 1e-7 * np.max(np.abs(v1))
    assert np.array_equal(a0 > 0, a1 > 0)
    assert np.max(np.abs(a0 - a1)) <= 1e-8
    assert abs(i0 - i1) <= max(2, nsteps // 50)


@pytest.mark.gpu
def test_fields_written_as_openfoam_volscalarfields(gpu_lib, tmp_path):
    """Vm and activationTime of a context written at its current time and
    read back from the ASCII files."""
    mesh = box_mesh(20, 7, 3, 0.02, 0.007, 0.003)
    m = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=1e-5, boxes=BOX)
    m.run(1e-5, 50)
    d = m.write(tmp_path, patches=[("walls", "zeroGradient")])
    assert d.name == "0.0005"
    for name, ref in (("Vm", m.vm()), ("activationTime", m.activation())):
        text = (d / name).read_text()
        assert f"object      {name};" in text
        if "nonuniform" in text:
            body = text.split("nonuniform List<scalar>")[1].split("(", 1)[1].split(")", 1)[0]
            vals = np.array([float(x) for x in body.split()])
        else:
            vals = np.full(ref.size, float(text.split("uniform")[1].split(";")[0]))
        assert vals.size == ref.size
        assert np.allclose(vals, ref, rtol=1e-5, atol=1e-12)
    m.close()


NIEDERER_DICT = """
myocardiumSolver  monodomainSolver;
monodomainSolverCoeffs
{
    conductivity [-1 -3 3 0 0 2 0] (0.1334177215 0 0 0.01760617761 0 0.01760617761);
    chi   [0 -1 0 0 0 0 0] 140000;
    cm    [-1 -4 4 0 0 2 0] 0.01;
    ionicModel    BuenoOrovio;
    tissue    epicardialCells;
    solutionAlgorithm    explicit;
    solver RKF45;
    maxSteps 1000000000;
    externalStimulus
    {
        stimulusLocationMin (0 0 5.5e-3);
        stimulusLocationMax (1.5e-3 1.5e-3 7e-3);
        stimulusDuration [0 0 1 0 0 0 0] 2e-3;
        stimulusIntensity [0 -3 0 0 0 1 0] 50000;
        stimulusStartTime 0.0;
    }
}
"""


@pytest.mark.gpu
def test_explicit_delta_t_rule_on_the_niederer_slab(gpu_lib):
    """electroModel::setDeltaT for the explicit algorithm: deltaT becomes
    maxCo * min(dx^2/Df) (myocardiumDomain.C:532-550), computed here as the
    regression test's restatement does, and steps taken with dt = 0 use it."""
    nx, ny, nz, lx, ly, lz = 100, 15, 35, 0.02, 0.003, 0.007
    mesh = box_mesh(nx, ny, nz, lx, ly, lz)
    sig = (0.1334177215, 0.01760617761, 0.01760617761)
    chicm = 140000 * 0.01
    dxs = (lx / nx, ly / ny, lz / nz)
    expect = 0.1 * min(dxs[d] ** 2 / (sig[d] / chicm) for d in range(3))
    m = api.Monodomain.from_dict(NIEDERER_DICT, mesh, 5e-5)
    # the library measures dx between cell centres: equal up to rounding
    assert abs(m.delta_t() - expect) <= 1e-12 * expect
    assert abs(m.suggest_explicit_delta_t(0.2) - 2 * expect) <= 1e-12 * expect
    m.step(0.0)
    m.run(0.0, 4)
    assert abs(m.time() - 5 * m.delta_t()) <= 1e-15
    # the controlDict's maxCo through the gpu sub-dictionary
    text = NIEDERER_DICT.replace("solver RKF45;", "solver RKF45;\n    gpu { maxCo 0.05; }")
    m2 = api.Monodomain.from_dict(text, mesh, 5e-5)
    assert abs(m2.delta_t() - 0.5 * expect) <= 1e-12 * expect
    # an implicit dictionary keeps the caller's deltaT
    m3 = api.Monodomain.from_dict(NIEDERER_DICT.replace("explicit;", "implicit;"), mesh, 5e-5)
    assert m3.delta_t() == 5e-5
    for x in (m, m2, m3):
        x.close()


@pytest.mark.gpu
def test_niederer_regression_probes_on_openfoam_centres(gpu_lib, oracle):
    """The reference's NiedererEtAl2012 regression case through the
    dictionary front end, on the cell centres OpenFOAM computes for its
    blockMesh (which decide the stimulated set: the box's inner faces pass
    through cell centres): the six probes within the reference's own
    tolerances (NiedererEtAl2012.reference:8-13), and every activation time
    within 1e-9 s of the oracle on the same mesh and time step."""
    import niederer_case as nc
    mesh = nc.openfoam_mesh(oracle, 0)
    m = api.Monodomain.from_dict(NIEDERER_DICT, mesh, 5e-5)
    dt = m.delta_t()
    assert abs(dt - nc.explicit_dt()) <= 1e-12 * dt
    d = oracle.tissue_desc("BuenoOrovio", 1, nc.SIGMA, implicit=False, ddt_backward=True,
                           boxes=[(*nc.BOX, *nc.STIMULUS)])
    o = oracle.Tissue(d, oracle.Mesh.general(mesh))
    while m.time() < nc.END_TIME - 1e-12:
        m.step(0.0)
        o.step(dt, 8)
    ag, ao = m.activation(), o.activation()
    assert np.array_equal(ag > 0, ao > 0)
    assert np.max(np.abs(ag - ao)) < 1e-9
    for probe, expect, tol in nc.pins():
        got = ag[nc.probe_cell(nc.PROBES[probe])]
        assert abs(got - expect) <= tol, (probe, got, expect)
    m.close()


@pytest.mark.gpu
def test_tissue_apd_tracking_equals_trace_postprocessing(gpu_lib):
    """Per-cell beat detection on the tissue's Vm (cfg_monodomain_track_apd)
    over a full beat of a TNNP slab, sampled every 0.1 ms: the device's
    beats, last-beat APD90 and upstroke times equal the restated
    post-processing (oracle/apd.py) run on the same samples read back."""
    from oracle import apd as oapd
    dt, every, n_samples = 1e-5, 10, 4000
    mesh = box_mesh(20, 7, 3, 0.02, 0.007, 0.003)
    m = api.Monodomain(mesh, "TNNP", "epicardialCells", SIGMA, dt=dt, boxes=BOX,
                       precision=lib.PRECISION_MIXED)
    m.track_apd(every)
    t = [m.time()]
    trace = [m.vm() * 1000.0]
    for _ in range(n_samples):
        m.run(dt, every)
        t.append(m.time())
        trace.append(m.vm() * 1000.0)
    t, trace = np.array(t), np.array(trace)
    nb, apd, tup = m.apd_results()
    for c in range(mesh.n_cells):
        b, a, u, _ = oapd.last_beat(t, trace[:, c])
        assert nb[c] == b, (c, nb[c], b)
        if np.isnan(a):
            assert np.isnan(apd[c])
            continue
        assert abs(a - apd[c]) <= 1e-9 * abs(a), (c, a, apd[c])
        assert abs(u - tup[c]) <= 1e-12, (c, u, tup[c])
    done = (nb >= 1) & ~np.isnan(apd)
    assert done.sum() >= 8                          # at least the stimulated corner
    assert 100.0 < np.min(apd[done]) and np.max(apd[done]) < 400.0
    m.close()
