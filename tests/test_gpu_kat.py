"""Known answers of the reference's evaluation tests on the GPU: prescribed
velocity fields (pm_set_fields) through the device reductions give the
permeabilities of tests/test_evaluation.py of the reference, equal to the
oracle's."""
import numpy as np
import pytest

import poremaps_gb300 as pm
from oracle.oracle import OracleProblem

pytestmark = pytest.mark.gpu
RE = 0.01


def both(u=None, v=None, w=None, dx=1e-6, porosity=-1.0, order="redblack"):
    g = np.zeros((6, 6, 6), np.uint8)
    z = np.zeros(g.shape)
    f = [z if a is None else a for a in (u, v, w)]
    with pm.Problem(g, None, boundary_method=0, solving_algorithm=2, voxel_size=dx,
                    porosity=porosity, order=order) as p:
        p.set_fields(*f, z)
        r = p.permeability()
    orc = OracleProblem(g, 0, 2, dx, porosity=porosity)
    orc.set_fields(*f, z)
    return r, orc.permeability()


@pytest.mark.parametrize("order", ["redblack", "reference"])
def test_uniform_fields(order):
    one = np.ones((6, 6, 6))
    r, o = both(w=one, order=order)
    assert r.wk33 == pytest.approx(1e-12 / RE) and r.wk13 == 0.0 and r.wk23 == 0.0
    assert r.wk33 == pytest.approx(o.wk33, rel=1e-15)
    r, _ = both(u=one, order=order)
    assert r.wk13 == pytest.approx(1e-12 / RE) and r.wk33 == 0.0


def test_scalings_mean_and_max():
    one = np.ones((6, 6, 6))
    assert both(w=one, porosity=0.5)[0].wk33 == pytest.approx(0.5 * both(w=one, porosity=1.0)[0].wk33)
    assert both(w=one, dx=2.0)[0].wk33 == pytest.approx(4.0 * both(w=one, dx=1.0)[0].wk33)
    w = np.ones((6, 6, 6))
    w[3:] = 2.0
    r, o = both(w=w, dx=1.0)
    assert r.wmax_velz == pytest.approx(2.0) and r.wmean_velz == pytest.approx(1.5)
    assert (r.wmax_velz, r.wmean_velz) == (o.wmax_velz, o.wmean_velz)
