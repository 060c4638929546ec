"""GPU: grids whose shapes stress the indexing of the pressure solve.

Odd and very unequal sides, one-row slices and a single sigma layer exercise
what the common cases do not:

* the colour-split copy of the level-0 operator (padding of odd rows);
* ragged last aggregates and the switch to 4 x 4 aggregation;
* bilinear prolongation clamped at the walls, and rows of one aggregate;
* line solves of one level;
* the single-block coarse cycle taking the whole hierarchy.

Each case steps FP64 against the oracle (eta and P within 1e-10, the mask bit
for bit) and FP32+IR eta within 1e-6.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [(37, 23, 3), (5, 131, 4), (130, 3, 7), (33, 17, 1), (31, 1, 5)]


def _case(M, N, K, precision, tol):
    from nhwave_gb300 import default_params
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.5, dy=0.5, dt_ini=0.01, tol=tol, itmax=20000)
    p.precision = precision
    x = (np.arange(M) + 0.5) * 0.5
    y = (np.arange(N) + 0.5) * 0.5
    X, Y = np.meshgrid(x, y)
    depth = 1.0 + 0.3 * np.sin(X / 3.0) * np.cos(Y / 4.0)
    eta = 0.05 * np.exp(-((X - x.mean()) ** 2 + (Y - y.mean()) ** 2) / 4.0)
    return p, depth, eta


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_shapes_step_like_the_oracle(shape, precision, oracle_mod, gpu_lib):
    from nhwave_gb300 import fields as F, lib
    p, depth, eta = _case(*shape, precision, 1e-13 if precision == 0 else 1e-10)
    g = lib.Scenario(p, depth, eta)
    po, _, _ = _case(*shape, 0, 1e-13)
    o = oracle_mod.Oracle(po, depth.ravel(), eta.ravel())
    for n in range(4):
        assert g.step() == 0 and o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    r = rel_l2(g.get(F.ETA)[sl(F.ETA)], o.get(F.ETA)[sl(F.ETA)])
    assert r < (1e-10 if precision == 0 else 1e-6), f"{shape} eta rel L2 {r:.3e}"
    if precision == 0:
        r = rel_l2(g.get(F.P)[sl(F.P)], o.get(F.P)[sl(F.P)])
        assert r < 1e-10, f"{shape} P rel L2 {r:.3e}"
        assert g.scalars().last_rel_residual <= 1e-13
    g.close()
