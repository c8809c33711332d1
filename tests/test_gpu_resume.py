"""Checkpoint/resume through the field dumps (pm_set_fields,
pm_resume_outputs).  Where the dumps hold the whole state (no periodic axis:
boundary_method 3 and 4), a resumed reference-order run is bit for bit the
uninterrupted run.  With periodic axes the dumps lack the pre-reapply pressure
of the last interior plane's halo copies, so the resumed run converges to the
same permeability (1e-6) instead."""
import numpy as np
import pytest

import poremaps_gb300 as pm
from poremaps_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", ["reference", "redblack", "jacobi"])
def test_set_get_round_trip(order):
    g = synth.random_solid((14, 12, 10), 0.25, 21)
    kw = dict(boundary_method=0, solving_algorithm=2, order=order)
    with pm.Problem(g, None, **kw) as a:
        a.iterate(40)
        f = a.fields()
    with pm.Problem(g, None, **kw) as b:
        b.set_fields(*f, iteration=40)
        assert b.iteration == 40
        for x, y in zip(f, b.fields()):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("bc,solver", [(3, 2), (4, 3), (4, 1)])
def test_resume_bitwise_without_periodic_axes(bc, solver):
    g = synth.random_solid((16, 12, 14), 0.2, 22)
    kw = dict(boundary_method=bc, solving_algorithm=solver, order="reference",
              arith=pm.ARITH_EXACT)
    with pm.Problem(g, None, **kw) as a:
        a.iterate(300)
        mid = a.fields()
        a.iterate(300)
        straight = a.fields()
        ka = a.permeability()
    with pm.Problem(g, None, **kw) as b:
        b.set_fields(*mid, iteration=300)
        b.iterate(300)
        assert b.iteration == 600
        for x, y in zip(straight, b.fields()):
            assert np.array_equal(x, y)
        assert b.permeability().wk33 == ka.wk33


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_resume_from_dumps_converges_to_same_k(tmp_path, monkeypatch, precision):
    monkeypatch.chdir(tmp_path)
    g = synth.sphere_pack((24, 24, 24), rmin=2.0, rmax=4.0, solid_fraction=0.6, seed=23)
    kw = dict(boundary_method=0, solving_algorithm=3, eps=1e-9, precision=precision,
              geometry_file_name="sample.raw", write_output=(1, 1, 0, 0), max_iter=200000)
    with pm.Problem(g, None, **kw) as a:
        full = a.solve()
    with pm.Problem(g, None, **kw) as b:
        b.iterate(700)
        b.write_outputs()
    with pm.Problem(g, None, **kw) as c:
        c.resume_outputs(700)
        r = c.solve()
    assert r.iterations > 700
    for k in ("wk13", "wk23", "wk33"):
        assert abs(getattr(r, k) - getattr(full, k)) <= 1e-6 * abs(full.wk33), k
