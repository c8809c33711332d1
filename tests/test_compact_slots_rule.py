"""The compact store's six-slot rule, checked on the CPU against the padded
store it replaces.

pm_compact.cuh stores, per fluid voxel and axis, two neighbour positions
chosen by the axis' neighbourhood case (L = l, or rr in case 4; R = r, or ll
in case 5; the zero slot where nothing is stored).  The sweep then reads
(ll, l, r, rr) = (R, L, R, L) for the wall stencils, the true l / r (0 where
solid) for the along-axis terms and the divergence, and L for the pressure
difference (taken only where l is fluid).  Here the neighbourhood cases come
from the oracle (the reference's eval_geometry), the padded store's values are
emulated from random corrections with the halo rules of the padded sweep
(periodic images one period away, zeros on wall faces and where no image
exists), and every value the update uses must be the padded one -- on axes of
length 1 and 2, rows longer than one 32-bit mask word and every boundary
family.
"""
import numpy as np
import pytest

from oracle.oracle import OracleProblem
from poremaps_gb300 import synth

PER = {0: (1, 1, 1), 1: (0, 0, 1), 2: (0, 0, 1), 3: (0, 0, 0), 4: (0, 0, 0)}


def wrap(q, n, per):
    if q < 0:
        return q + n, bool(per) and q + n >= 0
    if q >= n:
        return q - n, bool(per) and q - n < n
    return q, True


def left_fluid(k):
    return k in (3, 5, 6)


def right_fluid(k):
    return k in (2, 4, 6)


@pytest.mark.parametrize("shape", [(1, 6, 9), (2, 3, 5), (7, 1, 33), (3, 5, 2), (4, 4, 1),
                                   (5, 9, 65), (2, 2, 2), (1, 1, 1)])
@pytest.mark.parametrize("bc", [0, 1, 2, 3, 4])
def test_six_slots_reproduce_the_padded_stencil(shape, bc):
    nz, ny, nx = shape
    g = synth.random_solid(shape, 0.3, 7 * sum(shape) + bc)
    nh = OracleProblem(g, bc, 2).nhood()
    per = PER[bc]
    lin = np.flatnonzero(g.ravel() == 0)
    nl = lin.size
    pos = -np.ones(g.size, np.int64)
    pos[lin] = np.arange(nl)
    rng = np.random.default_rng(1)
    e = np.concatenate([rng.standard_normal(nl) + 1.0, [0.0]])  # the zero slot last
    n = (nx, ny, nz)
    for i, L in enumerate(lin):
        z, r = divmod(int(L), ny * nx)
        y, x = divmod(r, nx)
        code = int(nh[z, y, x])
        cases = (code // 100, (code // 10) % 10, code % 10)
        c = (x, y, z)
        for ax, k in enumerate(cases):
            def at(d, slot):
                q, ok = wrap(c[ax] + d, n[ax], per[ax])
                if not ok:
                    return (nl if slot else 0.0)
                cc = list(c)
                cc[ax] = q
                p = int(pos[(cc[2] * ny + cc[1]) * nx + cc[0]])
                if slot:
                    assert p >= 0, "a slot points at a solid voxel"
                    return p
                return 0.0 if p < 0 else e[p]
            sl = at(-1, True) if left_fluid(k) else (at(2, True) if k == 4 else nl)
            sr = at(1, True) if right_fluid(k) else (at(-2, True) if k == 5 else nl)
            vl, vr = e[sl], e[sr]
            l, rr_, ll, rrr = at(-1, False), at(1, False), at(-2, False), at(2, False)
            # along-axis terms and the divergence
            assert (vl if left_fluid(k) else 0.0) == l
            assert (vr if right_fluid(k) else 0.0) == rr_
            # the wall stencil's picks (case_pick) with (ll, l, r, rr) = (R, L, R, L)
            a_got = vl if k in (3, 5, 6) else vr
            b_got = vl if k == 4 else vr
            a_pad = l if k in (3, 5, 6) else rr_
            b_pad = rrr if k == 4 else (ll if k == 5 else rr_)
            if k != 1:
                assert a_got == a_pad
            if k in (4, 5, 6):
                assert b_got == b_pad
            # the pressure difference (left neighbour fluid)
            if left_fluid(k):
                assert vl == l
