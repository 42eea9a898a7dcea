"""Adjoint of the differentiable monodomain step (cfg_adjoint_*): gradients of
a probe-voltage misfit with respect to per-cell log-scales of g_Na and g_K1
and the two conductivities, checked against central finite differences of
the forward run, checkpoint-invariant, and through torch.autograd."""
import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from cardiacfoam_gb300.fields import gaussian_random_field
from cardiacfoam_gb300.mesh import box_mesh

H = 2.5e-4
NX = NY = 24
DT = 1e-5


def _problem(n_steps=400, checkpoint_every=50, sample_every=20, seed=3,
             precision=lib.PRECISION_FP64):
    mesh = box_mesh(NX, NY, 1, NX * H, NY * H, H)
    rng = np.random.default_rng(seed)
    probes = rng.choice(mesh.n_cells, 8, replace=False)
    boxes = [((0.0, 0.0, 0.0), (1.5e-3, 1.5e-3, H), 0.0, 2e-3, 5e4)]
    return api.AdjointProblem(mesh, n_steps, DT, probes, sample_every,
                              checkpoint_every=checkpoint_every, substeps=5, boxes=boxes,
                              precision=precision)


def _fields(seed):
    a = gaussian_random_field((NY, NX), H, 1.25e-3, 0.2, seed).ravel()
    b = gaussian_random_field((NY, NX), H, 1.25e-3, 0.2, seed + 100).ravel()
    return a, b


@pytest.fixture(scope="module")
def setup(gpu_lib):
    p = _problem()
    ta, tb = _fields(11)
    _, target = p.forward(ta, tb, 0.15, 0.03)
    p.set_target(target)
    a, b = _fields(5)
    return p, a, b, (0.1334, 0.0176)


@pytest.mark.gpu
def test_gradient_matches_central_differences(setup):
    p, a, b, (sl, st) = setup
    J, _ = p.forward(a, b, sl, st)
    ga, gb, gs = p.backward()
    assert J > 0 and np.all(np.isfinite(ga)) and np.all(np.isfinite(gb))
    assert np.abs(ga).max() > 0 and np.abs(gb).max() > 0 and np.all(gs != 0)
    rng = np.random.default_rng(7)
    eps = 1e-6
    for _ in range(4):
        va, vb = rng.standard_normal(a.size), rng.standard_normal(b.size)
        vs = rng.standard_normal(2) * np.array([sl, st])
        ad = ga @ va + gb @ vb + gs @ vs
        jp, _ = p.forward(a + eps * va, b + eps * vb, sl + eps * vs[0], st + eps * vs[1])
        jm, _ = p.forward(a - eps * va, b - eps * vb, sl - eps * vs[0], st - eps * vs[1])
        fd = (jp - jm) / (2 * eps)
        assert abs(fd - ad) <= 1e-5 * abs(fd) + 1e-14, (fd, ad)


@pytest.mark.gpu
def test_single_parameter_directions(setup):
    """The conductivity derivatives and one cell's g_Na alone."""
    p, a, b, (sl, st) = setup
    p.forward(a, b, sl, st)
    ga, gb, gs = p.backward()
    eps = 1e-6
    for k in range(2):
        s = [sl, st]
        sp, sm = list(s), list(s)
        sp[k] += eps * s[k]
        sm[k] -= eps * s[k]
        fd = (p.forward(a, b, *sp)[0] - p.forward(a, b, *sm)[0]) / (2 * eps * s[k])
        assert abs(fd - gs[k]) <= 1e-5 * abs(fd), (k, fd, gs[k])
    c = int(np.argmax(np.abs(ga)))
    e = np.zeros_like(a)
    e[c] = 1.0
    fd = (p.forward(a + eps * e, b, sl, st)[0] - p.forward(a - eps * e, b, sl, st)[0]) / (2 * eps)
    assert abs(fd - ga[c]) <= 1e-5 * abs(fd), (fd, ga[c])


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient(gpu_lib, setup):
    p0, a, b, (sl, st) = setup
    _, target = p0.forward(*_fields(11), 0.15, 0.03)
    out = []
    for every in (50, 400, 37):
        p = _problem(checkpoint_every=every)
        p.set_target(target)
        J, _ = p.forward(a, b, sl, st)
        out.append((J, *p.backward()))
        p.close()
    for o in out[1:]:
        assert o[0] == out[0][0]
        for x, y in zip(o[1:], out[0][1:]):
            assert np.array_equal(x, y)


@pytest.mark.gpu
def test_torch_autograd_function(setup):
    torch = pytest.importorskip("torch")
    from cardiacfoam_gb300.autograd import probe_misfit
    p, a, b, (sl, st) = setup
    ta = torch.tensor(a, requires_grad=True)
    tb = torch.tensor(b, requires_grad=True)
    ts = torch.tensor([sl, st], dtype=torch.float64, requires_grad=True)
    J = probe_misfit(p, ta, tb, ts)
    (3.0 * J).backward()
    ga, gb, gs = p.backward()
    assert np.allclose(ta.grad.numpy(), 3.0 * ga, rtol=0, atol=0)
    assert np.allclose(tb.grad.numpy(), 3.0 * gb, rtol=0, atol=0)
    assert np.allclose(ts.grad.numpy(), 3.0 * gs, rtol=0, atol=0)


@pytest.mark.gpu
def test_mixed_gradient_against_fp64_reference(gpu_lib, setup):
    """The mixed form (FP32 right-hand side and derivative, FP64 states,
    adjoint accumulation and solves) against the FP64 reference gradient."""
    p64, a, b, (sl, st) = setup
    _, target = p64.forward(*_fields(11), 0.15, 0.03)
    p64.set_target(target)
    J64, _ = p64.forward(a, b, sl, st)
    g64 = p64.backward()
    pm = _problem(precision=lib.PRECISION_MIXED)
    pm.set_target(target)
    Jm, _ = pm.forward(a, b, sl, st)
    gm = pm.backward()
    pm.close()
    assert abs(Jm - J64) <= 1e-3 * J64
    for x, y in zip(gm[:2], g64[:2]):
        assert np.linalg.norm(x - y) <= 1e-2 * np.linalg.norm(y)
    assert np.all(np.abs(gm[2] - g64[2]) <= 1e-2 * np.abs(g64[2]))
    rng = np.random.default_rng(9)
    for _ in range(4):
        va, vb, vs = rng.standard_normal(a.size), rng.standard_normal(b.size), rng.standard_normal(2)
        d64 = g64[0] @ va + g64[1] @ vb + g64[2] @ vs
        dm = gm[0] @ va + gm[1] @ vb + gm[2] @ vs
        assert abs(dm - d64) <= 1e-2 * abs(d64), (dm, d64)
