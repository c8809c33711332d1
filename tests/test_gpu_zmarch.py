"""The TMA-fed FP32 correction sweeps (z-march, bricks) against the
fluid-list kernel.

All run the same per-voxel arithmetic (update_fast<float> + residual), the
TMA kernels reading the stencil from shared-memory planes or bricks, the
fluid-list kernels from global memory, so the mixed form must give bitwise
identical fields with every kernel -- on sizes that are not multiples of the
tiles or bricks, short z extents, every boundary family and every solver the
mixed form supports.
"""
import numpy as np
import pytest

import poremaps_gb300 as pm
from poremaps_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = [((20, 20, 20), 0, 2), ((13, 37, 45), 1, 2), ((5, 17, 33), 2, 3), ((40, 19, 70), 3, 3),
         ((9, 48, 64), 4, 2), ((64, 64, 64), 0, 3)]


@pytest.mark.parametrize("shape,bc,solver", CASES)
def test_tma_kernels_equal_fluid_list(shape, bc, solver):
    g = synth.random_solid(shape, 0.3, sum(shape) + bc)
    out = []
    for kernel, brick in ((1, (0, 0, 0)), (0, (0, 0, 0)), (3, (0, 0, 0)), (2, (32, 8, 8)),
                          (4, (32, 8, 8)), (4, (32, 8, 4)), (4, (32, 4, 4)), (5, (0, 0, 0)),
                          (6, (32, 8, 8)), (7, (0, 0, 0))):
        with pm.Problem(g, None, boundary_method=bc, solving_algorithm=solver, order="jacobi",
                        precision="mixed", kernel=kernel, brick=brick, mixed_inner=40) as p:
            assert p.kernel() == kernel and p.brick() == brick
            p.iterate(117)
            out.append(p.fields())
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b), float(np.abs(a - b).max())


def test_autotuned_kernel_is_a_candidate():
    g = synth.random_solid((32, 32, 32), 0.3, 1)
    with pm.Problem(g, None, solving_algorithm=2, order="jacobi", precision="mixed") as p:
        assert p.kernel() in tuple(range(8))


@pytest.mark.parametrize("shape,bc", [((40, 36, 70), 0), ((33, 21, 50), 2)])
def test_autotuned_kernel_and_list_order_bitwise(shape, bc):
    """Whatever kernel and fluid-list brick order the autotuner picks, the
    fields equal the lexicographic fluid-list sweep bit for bit."""
    g = synth.random_solid(shape, 0.3, 5)
    out = []
    for kernel in (-1, 1):
        with pm.Problem(g, None, boundary_method=bc, solving_algorithm=2, order="jacobi",
                        precision="mixed", kernel=kernel) as p:
            p.iterate(150)
            out.append(p.fields())
    for a, b in zip(*out):
        assert np.array_equal(a, b)
