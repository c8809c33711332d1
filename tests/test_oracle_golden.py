"""The CPU oracle against golden vectors written by the reference program.

tests/golden/golden.npz holds the output of the reference's own sources
(built unmodified against the MPI shim; tests/golden/make_golden.py): log rows
and field files of small seeded runs covering every solver, every boundary
method, a dom_interest box, a given porosity, z-slab decompositions (2 and 3
ranks), a run to convergence and the 24x14x50 channel benchmark.  The oracle
must reproduce them bit for bit.
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402
from oracle.oracle import OracleProblem  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "golden.npz"), allow_pickle=False)
META = json.loads(str(GOLDEN["__meta__"]))
SLOW = {"c1_cylinder"}
CASES = [n for n in META if n not in SLOW or os.environ.get("PM_SLOW")]


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_built):
    return oracle_built


def run_oracle(c, tmp_path):
    g = make_golden.geometry(c["geom"])
    nslabs = c.get("ranks", 1)
    if nslabs > 1:
        assert c["dims"] == [1, 1, nslabs]
    orc = OracleProblem(g, c["bc"], c["solver"], c.get("dx", 1e-5), c.get("porosity", -1.0),
                        tuple(c.get("dom_interest", [0] * 6)), nslabs=nslabs)
    log = str(tmp_path / "o.log")
    orc.calc_flow(c["max_iter"], c.get("it_eval", 100), c.get("it_write", 100), c["eps"],
                  "reference", log)
    return g, orc, make_golden.blank_tps(open(log).read())


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name, tmp_path):
    c = META[name]
    g, orc, log = run_oracle(c, tmp_path)
    assert log == str(GOLDEN[f"{name}/log"])
    f = orc.fields()
    dx = c.get("dx", 1e-5)
    outs = {"velx_": f.u * dx, "vely_": f.v * dx, "velz_": f.w * dx, "press_": f.p,
            "voxel_neighborhood_": orc.nhood()}
    for pre, arr in outs.items():
        raw = np.ascontiguousarray(arr).tobytes()
        assert hashlib.sha256(raw).hexdigest() == str(GOLDEN[f"{name}/sha_{pre}"]), pre
        if c["fields"]:
            assert np.array_equal(arr, GOLDEN[f"{name}/{pre}"]), pre


def test_golden_channel_permeability():
    """Known answer: the channel benchmark converges to wk33 = 1.405994e-08 m^2
    after 11,200 iterations (7 printed digits of the reference log)."""
    last = str(GOLDEN["channel_24_14_50/log"]).strip().splitlines()[-1]
    cols = [c.strip() for c in last.split(",")]
    assert cols[0] == "11200"
    assert cols[-1] == "1.405994e-08"


def test_golden_covers_all_boundary_methods_and_solvers():
    bcs = {META[n]["bc"] for n in META}
    solvers = {META[n]["solver"] for n in META}
    assert bcs == {0, 1, 2, 3, 4} and solvers == {1, 2, 3}
