"""Concurrent blocks of several problems (pm_block_group_timed, the bench's
step over the three rotated problems of the tensor) give exactly the results
of running each problem's blocks alone: the problems share nothing but the
device."""
import numpy as np
import pytest

import poremaps_gb300 as pm
from poremaps_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,solver", [("mixed", 3), ("fp64", 2)])
def test_group_blocks_equal_separate_blocks(precision, solver):
    g = synth.random_solid((24, 20, 28), 0.3, 31)
    rots = [g, np.ascontiguousarray(np.transpose(g, (2, 0, 1))),
            np.ascontiguousarray(np.transpose(g, (1, 2, 0)))]
    kw = dict(solving_algorithm=solver, order="jacobi", precision=precision, it_eval=50)
    together = [pm.Problem(r, None, **kw) for r in rots]
    alone = [pm.Problem(r, None, **kw) for r in rots]
    perm = [0.0] * 3
    for _ in range(4):
        ms, conv, perm = pm.block_group_timed(together, 50, True, perm)
        assert ms > 0
    for i, p in enumerate(alone):
        k = 0.0
        for _ in range(4):
            _, c, k = p.block_timed(50, True, k)
        assert k == perm[i] and c == conv[i]
        for x, y in zip(together[i].fields(), p.fields()):
            assert np.array_equal(x, y)
    for p in together + alone:
        p.close()
