"""The FP32 correction sweeps of the mixed form against one another.

All run the same per-voxel arithmetic (update_fast<float> + residual): the
TMA kernels read the stencil from shared-memory planes or bricks, the
fluid-list kernels from the padded store in global memory, the compact-store
kernel (8) from a store of fluid voxels only, located through the fluid mask,
with periodic images instead of halo copies.  The mixed form must give
bitwise identical fields with every kernel -- on sizes that are not multiples
of the tiles, bricks or mask words, short and length-1 axes, every boundary
family and every solver the mixed form supports -- and identical sums when a
reduction reads the correction in the middle of a block.
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
                          (6, (32, 8, 8)), (7, (0, 0, 0)), (8, (0, 0, 0)), (9, (0, 0, 0)),
                          (10, (0, 0, 0)), (11, (0, 0, 0)), (12, (0, 0, 0)), (13, (0, 0, 0))):
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
        assert p.kernel() in tuple(range(14))


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


@pytest.mark.parametrize("shape", [(1, 6, 9), (2, 3, 5), (7, 1, 33), (3, 5, 2), (4, 4, 1),
                                   (6, 9, 65)])
@pytest.mark.parametrize("bc", [0, 2, 4])
def test_compact_store_small_axes(shape, bc):
    """Axes of length 1 and 2 (where a periodic halo cell has no image one
    period away and the padded store holds 0 there) and rows longer than one
    mask word: the compact store equals the padded fluid-list sweep."""
    g = synth.random_solid(shape, 0.25, 3 * sum(shape) + bc)
    out = []
    for kernel in (1, 8, 9, 10, 11, 12, 13):
        with pm.Problem(g, None, boundary_method=bc, solving_algorithm=2, order="jacobi",
                        precision="mixed", kernel=kernel, mixed_inner=25) as p:
            p.iterate(61)
            out.append(p.fields())
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b), float(np.abs(a - b).max())


@pytest.mark.parametrize("bc,di", [(0, (0, 0, 0, 0, 0, 0)), (1, (2, 20, 1, 15, 3, 30))])
def test_compact_store_reductions_mid_block(bc, di):
    """Permeability and convergence read x + e while a correction block is
    open: the compact store's sums equal the padded store's bit for bit."""
    g = synth.random_solid((36, 22, 41), 0.3, 17)
    res = []
    for kernel in (6, 8, 9, 10, 11, 13):
        with pm.Problem(g, None, boundary_method=bc, solving_algorithm=3, order="jacobi",
                        precision="mixed", kernel=kernel, dom_interest=di) as p:
            p.iterate(157)  # 57 sweeps into a 100-sweep block
            k = p.permeability()
            conv, perm = p.convergence()
            res.append((k.wk13, k.wk23, k.wk33, k.k33, k.wmax_velz, conv, perm))
    assert all(r == res[0] for r in res[1:])


@pytest.mark.parametrize("kernel", [0, 3, 11, 12])
def test_pipeline_wait_timeout_path(kernel):
    """The failure path of the sweeps fed by asynchronous copies (TMA
    z-march 0 / 3, bulk-staged compact store 11 / 12): with the test hook
    every CTA treats its first pipeline wait as timed out, sets the error flag
    and waits for its copies in flight before it returns.  The sweep reports PM_ERR_CUDA;
    afterwards the same problem, reset, sweeps normally and gives the
    fluid-list kernel's fields bit for bit."""
    g = synth.random_solid((24, 20, 30), 0.3, 41)
    kw = dict(boundary_method=0, solving_algorithm=2, order="jacobi", precision="mixed",
              mixed_inner=40)
    with pm.Problem(g, None, kernel=kernel, **kw) as p:
        p.iterate(3)
        pm.debug_tma_fail(True)
        try:
            with pytest.raises(pm.PMError) as ei:
                p.iterate(1)
                p.fields()  # synchronises; the flag is read there at the latest
        finally:
            pm.debug_tma_fail(False)
        assert ei.value.status == 3 and "timed out" in str(ei.value)
        p.reset()
        p.iterate(57)
        got = p.fields()
    with pm.Problem(g, None, kernel=1, **kw) as p:
        p.iterate(57)
        want = p.fields()
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("shape,bc", [((30, 40, 50), 0), ((70, 90, 8), 0), ((40, 300, 300), 1),
                                      ((12, 16, 20), 3)])
def test_packed_records_escapes_bitwise(shape, bc):
    """Kernel 13 stores each position's six neighbours as 16-bit offsets and
    falls back to the full slots where an offset does not fit: periodic
    z faces of many fluid voxels (first and last planes), planes of more than
    32767 fluid voxels (every position escapes), and no periodic axes.  Every
    case equals kernel 10 bit for bit."""
    g = synth.random_solid(shape, 0.3, sum(shape) + 7 * bc)
    out = []
    for kernel in (10, 13):
        with pm.Problem(g, None, boundary_method=bc, solving_algorithm=3, order="jacobi",
                        precision="mixed", kernel=kernel, mixed_inner=30) as p:
            p.iterate(71)
            out.append(p.fields())
    for a, b in zip(*out):
        assert np.array_equal(a, b), float(np.abs(a - b).max())
