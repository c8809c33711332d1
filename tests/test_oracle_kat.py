"""Known answers of the reference's own unit tests, checked on the oracle.

The reference ships Python mirrors of its routines with known-answer tests
(tests/test_solver.py: get_2nd_derivation and split_number;
tests/test_geometry.py: porosity and neighbourhood cases;
tests/test_evaluation.py: permeability of prescribed velocity fields).  The
same situations and expected values are restated here against the oracle's
C restatement; the oracle itself is pinned bit for bit against the reference
program (tests/test_oracle_golden.py).
"""
import numpy as np
import pytest

from oracle.oracle import OracleProblem, second_derivative, split_code

RE = 0.01  # constants.h: Reynolds number of the pseudo-time scheme


# ---------------------------------------------------------------- split_number
@pytest.mark.parametrize("code,cases", [(0, (0, 0, 0)), (6, (0, 0, 6)), (30, (0, 3, 0)),
                                        (200, (2, 0, 0)), (111, (1, 1, 1)), (666, (6, 6, 6)),
                                        (246, (2, 4, 6)), (135, (1, 3, 5)), (1, (0, 0, 1)),
                                        (600, (6, 0, 0))])
def test_split_code(code, cases):
    assert split_code(code) == cases


def test_split_code_round_trip():
    for x in range(7):
        for y in range(7):
            for z in range(7):
                assert split_code(100 * x + 10 * y + z) == (x, y, z)


# ---------------------------------------------------------- get_2nd_derivation
def test_case1_both_walls():
    assert second_derivative(1, 0.0, 0.0, 1.0, 0.0, 0.0) == pytest.approx(-8.0)
    assert second_derivative(1, 5.0, 5.0, 0.0, 5.0, 5.0) == pytest.approx(0.0)
    assert second_derivative(1, 99.0, 99.0, 2.0, 99.0, 99.0) == pytest.approx(-16.0)


def test_case2_and_case3_one_fluid_neighbour():
    assert second_derivative(2, 0.0, 0.0, 1.0, 3.0, 0.0) == pytest.approx(8 / 3 * 3 - 16 / 3)
    assert second_derivative(2, 0.0, 0.0, 1.0, 2.0, 0.0) == pytest.approx(0.0)
    assert second_derivative(3, 0.0, 3.0, 1.0, 0.0, 0.0) == pytest.approx(8 / 3 * 3 - 16 / 3)
    assert second_derivative(2, 0.0, 0.0, 2.0, 4.0, 0.0) == pytest.approx(
        second_derivative(3, 0.0, 4.0, 2.0, 0.0, 0.0))


def test_case4_and_case5_two_fluid_neighbours():
    assert second_derivative(4, 0.0, 0.0, 1.0, 2.0, 3.0) == pytest.approx(4.0 - 5.0 - 0.6)
    assert second_derivative(5, 3.0, 2.0, 1.0, 0.0, 0.0) == pytest.approx(4.0 - 0.6 - 5.0)
    assert second_derivative(4, 0.0, 0.0, 2.0, 4.0, 6.0) == pytest.approx(
        second_derivative(5, 6.0, 4.0, 2.0, 0.0, 0.0))


def test_case6_central_difference():
    assert second_derivative(6, 0.0, 1.0, 0.0, 1.0, 0.0) == pytest.approx(2.0)   # x^2
    assert second_derivative(6, 0.0, -1.0, 0.0, 1.0, 0.0) == pytest.approx(0.0)  # x
    assert second_derivative(6, 5.0, 5.0, 5.0, 5.0, 5.0) == pytest.approx(0.0)
    assert second_derivative(6, 99.0, 1.0, 2.0, 3.0, 99.0) == \
        second_derivative(6, -1.0, 1.0, 2.0, 3.0, -1.0)


# ------------------------------------------------------ porosity, neighbourhood
def test_porosity_known_answers():
    assert OracleProblem(np.zeros((6, 6, 6), np.uint8)).permeability().porosity == 1.0
    half = np.zeros((6, 6, 6), np.uint8)
    half[:3] = 1
    assert OracleProblem(half).permeability().porosity == pytest.approx(0.5)
    chan = np.ones((4, 6, 6), np.uint8)
    chan[:, 1:5, 1:5] = 0  # 16 of 36 voxels per plane are fluid
    assert OracleProblem(chan, 3).permeability().porosity == pytest.approx(16 / 36)
    one = np.zeros((5, 5, 5), np.uint8)
    one[2, 2, 2] = 1
    assert OracleProblem(one).permeability().porosity == pytest.approx(124 / 125)


def test_neighbourhood_solid_and_walls():
    g = np.ones((6, 6, 6), np.uint8)
    assert (OracleProblem(g).nhood() == -1).all()  # all solid
    chan = np.ones((4, 8, 8), np.uint8)
    chan[:, 2:6, 2:6] = 0
    nh = OracleProblem(chan, 3).nhood()
    assert (nh[chan == 1] == -1).all() and (nh[chan == 0] >= 0).all()
    # first fluid voxel in x next to the channel wall: wall left, two fluid right
    assert nh[1, 3, 2] // 100 == 4
    assert nh[1, 3, 5] // 100 == 5


# -------------------------------------------------- permeability of set fields
def permeability(u=None, v=None, w=None, dx=1e-6, porosity=-1.0, geom=None):
    g = np.zeros((6, 6, 6), np.uint8) if geom is None else geom
    orc = OracleProblem(g, 0, 2, dx, porosity=porosity)
    z = np.zeros(g.shape)
    orc.set_fields(z if u is None else u, z if v is None else v, z if w is None else w)
    return orc.permeability()


def test_uniform_velocities():
    one = np.ones((6, 6, 6))
    r = permeability(w=one)
    assert r.wk33 == pytest.approx(1e-12 / RE) and r.wk13 == 0.0 and r.wk23 == 0.0
    r = permeability(u=one)
    assert r.wk13 == pytest.approx(1e-12 / RE) and r.wk23 == 0.0 and r.wk33 == 0.0
    r = permeability()
    assert (r.wk13, r.wk23, r.wk33, r.wmean_velz, r.wmax_velz) == (0.0, 0.0, 0.0, 0.0, 0.0)


def test_scaling_with_porosity_and_voxel_size():
    one = np.ones((6, 6, 6))
    assert permeability(w=one, porosity=0.5).wk33 == pytest.approx(
        0.5 * permeability(w=one, porosity=1.0).wk33)
    assert permeability(w=one, dx=2.0).wk33 == pytest.approx(4.0 * permeability(w=one, dx=1.0).wk33)


def test_mean_and_max_velz():
    w = np.full((6, 6, 6), 3.0)
    r = permeability(w=w, dx=2.0)
    assert r.wmean_velz == pytest.approx(6.0) and r.wmax_velz == pytest.approx(6.0)
    w = np.ones((6, 6, 6))
    w[3:] = 2.0
    r = permeability(w=w, dx=1.0)
    assert r.wmax_velz == pytest.approx(2.0) and r.wmean_velz == pytest.approx(1.5)


def test_all_solid_follows_the_program():
    """The Python mirror returns zeros for an all-solid domain; the reference
    program zeroes the sums but still divides by the zero fluid count
    (src/evaluation.cc:154, 205-209), so its permeabilities are NaN (which is
    what ends its loop).  The oracle follows the program."""
    r = permeability(geom=np.ones((6, 6, 6), np.uint8))
    assert np.isnan(r.wk13) and np.isnan(r.wk23) and np.isnan(r.wk33) and np.isnan(r.wmean_velz)
    assert r.wmax_velz == 0.0
