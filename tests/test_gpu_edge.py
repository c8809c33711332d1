"""Edge cases of the domain: no fluid at all, and a single isolated fluid
voxel, in every order and precision, against the oracle (which reproduces
the reference program).  With no fluid the reference's convergence value is
0/0 = NaN at its first check (iteration 1100), which ends its loop; the C ABI
returns PM_ERR_NONFINITE there with the result filled."""
import math

import numpy as np
import pytest

import poremaps_gb300 as pm
from oracle.oracle import OracleProblem

pytestmark = pytest.mark.gpu

FORMS = [dict(order="reference", arith=pm.ARITH_EXACT), dict(order="redblack"),
         dict(order="jacobi"), dict(precision="mixed")]


@pytest.mark.parametrize("kw", FORMS)
def test_all_solid_stops_like_the_reference(kw):
    g = np.ones((10, 9, 8), np.uint8)
    with pm.Problem(g, None, boundary_method=0, solving_algorithm=2, **kw) as p:
        r = pm.Result()
        st = pm.load_library().pm_solve(p.h, pm.C.byref(r))
    o = OracleProblem(g, 0, 2).calc_flow(100000, 100, 100, 1e-6, "reference")
    assert st == 5  # PM_ERR_NONFINITE
    assert r.iterations == o.iterations == 1100
    assert math.isnan(r.wk33) and math.isnan(o.wk33)


@pytest.mark.parametrize("bc", [0, 2, 4])
def test_single_fluid_voxel_reference_order_bitwise(bc):
    g = np.ones((9, 8, 7), np.uint8)
    g[4, 3, 2] = 0
    with pm.Problem(g, None, boundary_method=bc, solving_algorithm=2, order="reference",
                    arith=pm.ARITH_EXACT) as p:
        p.iterate(60)
        f = p.fields()
    o = OracleProblem(g, bc, 2)
    o.iterate(60, "reference")
    of = o.fields()
    for a, b in zip(f, (of.u, of.v, of.w, of.p)):
        assert np.array_equal(a, b)
    assert OracleProblem(g, bc, 2).nhood()[4, 3, 2] == 111


@pytest.mark.parametrize("kw", FORMS[1:])
def test_single_fluid_voxel_other_forms(kw):
    g = np.ones((9, 8, 7), np.uint8)
    g[4, 3, 2] = 0
    with pm.Problem(g, None, boundary_method=0, solving_algorithm=2, **kw) as p:
        p.iterate(60)
        f = p.fields()
    order = "jacobi" if kw.get("precision") == "mixed" else kw["order"]
    o = OracleProblem(g, 0, 2)
    o.iterate(60, order)
    of = o.fields()
    for a, b in zip(f, (of.u, of.v, of.w, of.p)):
        assert np.allclose(a, b, rtol=1e-6, atol=1e-12)


def test_server_all_solid_request_finishes_nonfinite():
    solid = np.ones((12, 12, 12), np.uint8)
    fluid = np.zeros((12, 12, 12), np.uint8)
    fluid[:, :, :2] = 1  # a slab of solid: flow along z stays possible
    kw = dict(boundary_method=0, solving_algorithm=2, eps=1e-6, it_eval=100, it_write=100,
              max_iter=20000)
    s = pm.Server(precision="mixed", use_graphs=1, autotune=0)
    t_solid = s.submit(solid, **kw)
    t_fluid = s.submit(fluid, **kw)
    res = {}
    for _ in range(1000):
        active = s.step()
        for c in s.poll():
            res[c.ticket] = c
        if active == 0 and len(res) == 2:
            break
    s.close()
    assert res[t_solid].status == 5 and math.isnan(res[t_solid].result.wk33)
    assert res[t_solid].result.iterations == 1100
    assert res[t_fluid].status == 0 and res[t_fluid].result.converged
