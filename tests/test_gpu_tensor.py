"""Full permeability tensor of every solver against the reference program.

The golden vectors hold the reference program's own converged runs of one
16^3 sphere pack in the three axis rotations of README.md:221-225, for
solving_algorithm 1, 2 and 3 (tests/golden/make_golden.py).  The GPU tensor
driver (pm_solve_tensor: three rotated problems, default red-black order, and
the mixed form where it applies) must give every component within 1e-6 of
the tensor's scale, and the diagonal within 1e-6 relative.  Full-precision
reference values come from the oracle, which reproduces those runs bit for
bit (tests/test_oracle_golden.py); the 7 printed digits of the reference logs
are checked too.  Iteration counts of both sides are printed.
"""
import json
import os
import sys

import numpy as np
import pytest

import poremaps_gb300 as pm
from oracle.oracle import OracleProblem

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = np.load(os.path.join(HERE, "golden", "golden.npz"), allow_pickle=False)
META = json.loads(str(GOLDEN["__meta__"]))
# K[i, j]: response along axis i to the pressure drop along axis j
SLOTS = {"x": ((1, 0), (2, 0), (0, 0)), "y": ((2, 1), (0, 1), (1, 1)),
         "z": ((0, 2), (1, 2), (2, 2))}


def reference_tensor(solver):
    K_log, K_full, its = np.zeros((3, 3)), np.zeros((3, 3)), {}
    for rot in "xyz":
        name = f"tensor_s{solver}_{rot}"
        c = META[name]
        last = [v.strip() for v in str(GOLDEN[f"{name}/log"]).strip().splitlines()[-1].split(",")]
        orc = OracleProblem(make_golden.geometry(c["geom"]), 0, solver, 1e-5)
        r = orc.calc_flow(c["max_iter"], 100, 100, c["eps"], "reference")
        assert r.iterations == int(last[0])
        its[rot] = r.iterations
        for (i, j), lv, fv in zip(SLOTS[rot], last[-3:], (r.wk13, r.wk23, r.wk33)):
            K_log[i, j] = float(lv)
            K_full[i, j] = fv
    return K_log, K_full, its


@pytest.mark.parametrize("solver,precision", [(1, "fp64"), (2, "fp64"), (3, "fp64"),
                                              (2, "mixed"), (3, "mixed")])
def test_tensor_matches_reference_program(solver, precision):
    K_log, K_full, its = reference_tensor(solver)
    eps = META[f"tensor_s{solver}_z"]["eps"]
    g = make_golden.geometry(dict(make_golden.TENSOR_GEOM))
    K, res = pm.solve_tensor(g, None, boundary_method=0, solving_algorithm=solver,
                             voxel_size=1e-5, eps=eps, max_iter=400000, precision=precision)
    scale = np.abs(np.diag(K_full)).max()
    assert np.abs(K - K_full).max() <= 1e-6 * scale
    assert np.all(np.abs(np.diag(K) - np.diag(K_full)) <= 1e-6 * np.abs(np.diag(K_full)))
    assert np.abs(K - K_log).max() <= 1e-6 * scale  # the reference log's 7 digits
    print(f"solver {solver} {precision}: reference iterations {its}, "
          f"GPU iterations {[r.iterations for r in res]}")


@pytest.mark.parametrize("precision,bc", [("fp64", 0), ("mixed", 1), ("fp64", 3)])
def test_tensor_rotations_on_a_non_cubic_medium(precision, bc):
    """pm_solve_tensor rotates the geometry of the x and y solves on the
    device.  On a medium with three different axis lengths (where a mix-up of
    the rotated sizes shows), every component equals three problems created
    from geometry rotated on the host, bit for bit: flow along x sees sizes
    (ny, nz, nx) with (x', y', z') = (y, z, x), flow along y (nz, nx, ny) with
    (x', y', z') = (z, x, y) (README.md:221-225 of the reference)."""
    from poremaps_gb300 import synth
    g = synth.random_solid((14, 11, 9), 0.3, 23)  # (nz, ny, nx)
    kw = dict(boundary_method=bc, solving_algorithm=2, voxel_size=1e-5, eps=1e-30,
              max_iter=1300, precision=precision)
    K, res = pm.solve_tensor(g, None, **kw)
    rot = {"x": np.transpose(g, (2, 0, 1)), "y": np.transpose(g, (1, 2, 0)), "z": g}
    want = np.zeros((3, 3))
    for axis in "xyz":
        with pm.Problem(np.ascontiguousarray(rot[axis]), None, **kw) as p:
            r = p.solve()
        for (i, j), v in zip(SLOTS[axis], (r.wk13, r.wk23, r.wk33)):
            want[i, j] = v
    assert np.array_equal(K, want), np.abs(K - want).max()
