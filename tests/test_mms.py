"""Manufactured-solution verification on the CPU oracle: the restated
OpenFOAM numerics reproduce the second-order convergence of the
monodomainFDAManufactured case (the order no reference test asserts)."""
import pytest

from cardiacfoam_gb300 import verification as vf
from mms_util import oracle_run


@pytest.mark.parametrize("dim,sizes", [(1, (10, 20, 40)), (2, (10, 20, 40)), (3, (10, 20))])
def test_oracle_manufactured_convergence_order(oracle, dim, sizes):
    res = {n: oracle_run(oracle, dim, n) for n in sizes}
    for a, b in zip(sizes, sizes[1:]):
        r_inf = vf.rate(res[a]["V"][2], res[b]["V"][2], a, b)
        r_l2 = vf.rate(res[a]["V"][1], res[b]["V"][1], a, b)
        assert 1.75 < r_inf < 2.2, (dim, a, b, r_inf)
        assert 1.8 < r_l2 < 2.2, (dim, a, b, r_l2)
        assert vf.rate(res[a]["u1"][2], res[b]["u1"][2], a, b) > 0.8


def test_manufactured_fields_solve_the_model_ode():
    """d(u1)/dt and d(u2)/dt of the exact fields equal the model's rates at
    the exact state (a check of the restated formulas, by central
    differences in time)."""
    import numpy as np
    c = np.random.default_rng(0).uniform(0, 1, (50, 3))
    t, h = 0.1, 1e-6
    V, u1, u2, u3 = vf.manufactured_fields(c, t, 3)
    _, u1p, u2p, _ = vf.manufactured_fields(c, t + h, 3)
    _, u1m, u2m, _ = vf.manufactured_fields(c, t - h, 3)
    w = u1 + u3 - V
    du1 = w ** 2 * u2 ** 2 + 0.5 * w * u2 ** 2 * (V - u3)
    du2 = -w * u2 ** 3
    assert np.allclose((u1p - u1m) / (2 * h), du1, rtol=1e-6, atol=1e-8)
    assert np.allclose((u2p - u2m) / (2 * h), du2, rtol=1e-6, atol=1e-8)
