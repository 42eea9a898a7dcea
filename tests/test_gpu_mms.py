"""Manufactured-solution verification on the GPU: the FP64 monodomain step
with the monodomainFDAManufactured model against the oracle (same
diagonal-preconditioned PCG), and its convergence order over the tutorial's
sweep (10/20/40 cells per direction, dt shrinking with h^2)."""
import numpy as np
import pytest

from cardiacfoam_gb300 import verification as vf
from mms_util import oracle_run


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_gpu_manufactured_matches_oracle(gpu_lib, oracle, dim):
    n = 10
    g = vf.run(dim, n)
    o = oracle_run(oracle, dim, n)
    assert g["t"] == o["t"]
    for field in ("V", "u1", "u2"):
        for eg, eo in zip(g[field], o[field]):
            assert abs(eg - eo) <= 1e-7 * eo + 1e-15, (field, eg, eo)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_gpu_manufactured_convergence_order(gpu_lib, dim):
    sizes = (10, 20, 40)
    res = {n: vf.run(dim, n) for n in sizes}
    for a, b in zip(sizes, sizes[1:]):
        r_inf = vf.rate(res[a]["V"][2], res[b]["V"][2], a, b)
        r_l2 = vf.rate(res[a]["V"][1], res[b]["V"][1], a, b)
        assert 1.75 < r_inf < 2.2, (dim, a, b, r_inf)
        assert 1.8 < r_l2 < 2.2, (dim, a, b, r_l2)
