"""The oracle's worker pool gives the single-thread values bit for bit.

The large-domain parity tests run the oracle on many host threads: Jacobi and
red-black passes split each slab's z planes among the workers, the reference
order sweeps whole slabs (ranks) per worker.  Each phase ends at a barrier, so
the fields must not depend on the thread count.
"""
import numpy as np
import pytest

from oracle.oracle import OracleProblem
from poremaps_gb300 import synth


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_built):
    return oracle_built


@pytest.mark.parametrize("order", ["reference", "jacobi", "redblack"])
@pytest.mark.parametrize("bc,nslabs", [(0, 1), (2, 1), (4, 1), (0, 3), (3, 2)])
def test_threads_bitwise(order, bc, nslabs):
    g = synth.random_solid((19, 11, 13), 0.25, seed=17 + bc)
    out = []
    for threads in (1, 5):
        orc = OracleProblem(g, bc, 2, 1e-5, nslabs=nslabs, threads=threads)
        orc.iterate(7, order)
        f = orc.fields()
        out.append((f, orc.convergence(0.0)[0]))
    (a, ca), (b, cb) = out
    for x, y in ((a.u, b.u), (a.v, b.v), (a.w, b.w), (a.p, b.p)):
        assert np.array_equal(x, y)
    assert ca == cb


def test_calc_flow_threads_same_stop():
    """calc_flow runs blocks between evaluations on the pool: same stop
    iteration and permeability as one thread."""
    g = synth.random_solid((16, 10, 12), 0.2, seed=41)
    r = []
    for threads in (1, 4):
        orc = OracleProblem(g, 0, 2, 2e-5, threads=threads)
        r.append(orc.calc_flow(3000, 100, 100, 1e-9, "jacobi"))
    assert (r[0].iterations, r[0].sweeps) == (r[1].iterations, r[1].sweeps)
    assert r[0].wk33 == r[1].wk33 and r[0].conv == r[1].conv
