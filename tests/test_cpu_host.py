"""Host-side tests that need no GPU: the C-ABI library loads and exports every
symbol of include/poremaps.h, the .inp parser and .raw reader behave like the
reference's (read_problem_params.cc:50-156, geometry.cc:58-126), and the
oracle's building blocks mirror the reference's own unit tests (stencil
coefficients, neighbourhood cases, permeability/convergence formulae)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import poremaps_gb300 as pm
from oracle.oracle import OracleProblem
from poremaps_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "poremaps.h")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(pm.LIB_PATH):
        from poremaps_gb300 import build

        build.build()
    return pm.load_library()


def header_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:pm_status|const char\*|double|uint64_t|size_t)\s+(pm_\w+)\(",
                                 src, re.M)))


def test_header_symbols_exported(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(pm.EXPORTS)


def test_version_and_defaults(lib):
    assert b"sm_103a" in lib.pm_version()
    p = pm.default_params()
    assert p.eps == 1e-6 and p.porosity == -1.0 and p.it_eval == 100
    assert p.order == pm.ORDER_DEFAULT and p.precision == pm.PREC_FP64
    assert p.eps_fixed_point == 0.0


TEMPLATE = """dom_decomposition 0 0 0
boundary_method 2
geometry_file_name dir/ptube_54_54_50_vs_2e-05.raw
size_x_y_z  54 54 50
voxel_size  2e-05
max_iter    100000001
it_eval    100
it_write   200
log_file_name permeability_ptube.log
solving_algorithm 3
eps 1e-07
porosity 1.0
dom_interest 1 2 3 4 5 6
write_output 1 1 0 0
"""


def test_read_params_fixed_order(lib, tmp_path):
    f = tmp_path / "a.inp"
    f.write_text(TEMPLATE)
    p = pm.read_params(str(f))
    assert list(p.size) == [54, 54, 50] and p.boundary_method == 2
    assert p.geometry_file_name == b"dir/ptube_54_54_50_vs_2e-05.raw"
    assert p.voxel_size == 2e-05 and p.max_iter == 100000001
    assert p.it_eval == 100 and p.it_write == 200 and p.solving_algorithm == 3
    assert p.eps == 1e-07 and p.porosity == 1.0
    assert list(p.dom_interest) == [1, 2, 3, 4, 5, 6] and list(p.write_output) == [1, 1, 0, 0]


def test_read_params_whitespace_runs(lib, tmp_path):
    # fscanf patterns: a blank in the pattern matches any run of white space
    f = tmp_path / "b.inp"
    f.write_text(TEMPLATE.replace("size_x_y_z  54", "size_x_y_z\t \t54").replace("\n", "\n\n"))
    p = pm.read_params(str(f))
    assert list(p.size) == [54, 54, 50]


def test_read_params_errors(lib, tmp_path):
    with pytest.raises(pm.PMError) as e:
        pm.read_params(str(tmp_path / "missing.inp"))
    assert e.value.status == 2
    f = tmp_path / "c.inp"
    f.write_text(TEMPLATE.replace("boundary_method", "bc_method"))
    with pytest.raises(pm.PMError) as e:
        pm.read_params(str(f))
    assert e.value.status == 1


def test_read_geometry(lib, tmp_path):
    g = synth.random_solid((5, 4, 3), 0.3, 1)
    path = tmp_path / "g.raw"
    g.tofile(path)
    out = np.empty(g.size, np.uint8)
    size = (C.c_int * 3)(3, 4, 5)
    assert lib.pm_read_geometry(str(path).encode(), size, out.ctypes.data) == 0
    assert np.array_equal(out.reshape(g.shape), g)
    size2 = (C.c_int * 3)(3, 4, 6)  # file too short
    assert lib.pm_read_geometry(str(path).encode(), size2, out.ctypes.data) == 2


def test_last_error_copy(lib):
    """The message of the last failing call, copied into a caller buffer:
    truncated and NUL-terminated, full length returned."""
    with pytest.raises(pm.PMError):
        pm.Problem(np.zeros((4, 4, 4), np.uint8), None, boundary_method=5)
    msg = lib.pm_last_error()
    assert b"boundary_method" in msg
    buf = C.create_string_buffer(b"x" * 16, 16)
    n = lib.pm_last_error_copy(buf, 16)
    assert n == len(msg) and buf.value == msg[:15] and buf.raw[15:16] == b"\0"
    big = C.create_string_buffer(n + 8)
    assert lib.pm_last_error_copy(big, n + 8) == n and big.value == msg
    assert lib.pm_last_error_copy(None, 0) == n


def test_problem_create_validates_before_touching_the_device(lib):
    g = np.zeros((4, 4, 4), np.uint8)
    for kw in (dict(boundary_method=5), dict(solving_algorithm=4), dict(it_eval=0),
               dict(solving_algorithm=1, precision="mixed"), dict(eps_fixed_point=-1e-9),
               dict(eps_fixed_point=float("nan"))):
        with pytest.raises(pm.PMError) as e:
            pm.Problem(g, None, **kw)
        assert e.value.status == 1


# ---- reference unit-test semantics restated on the oracle (tests/test_solver.py,
# test_geometry.py, test_evaluation.py of the reference) ----

def test_neighbourhood_all_fluid_is_666():
    orc = OracleProblem(np.zeros((8, 8, 8), np.uint8), 0, 2)
    assert (orc.nhood() == 666).all()


def test_neighbourhood_cases_line():
    # x-line fluid pattern (1 = solid) around the probed voxels, periodic off
    g = np.ones((5, 5, 9), np.uint8)
    g[2, 2, 1:8] = 0
    g[2, 2, 4] = 1            # split into two fluid runs of length 3
    orc = OracleProblem(g, 3, 2)
    nh = orc.nhood()[2, 2]
    cx = nh // 100
    # run x=1..3: left wall at 0 -> case 4 (l solid, r, rr fluid), middle 6? no:
    # x=1: l solid, r fluid, rr fluid -> 4; x=2: l,r fluid -> 6; x=3: ll fluid, r solid -> 5
    assert list(cx[1:4]) == [4, 6, 5]
    assert list(cx[5:8]) == [4, 6, 5]
    g2 = np.ones((5, 5, 6), np.uint8)
    g2[2, 2, 2:4] = 0         # two fluid voxels: case 2 then case 3
    assert list((OracleProblem(g2, 3, 2).nhood()[2, 2] // 100)[2:4]) == [2, 3]
    g3 = np.ones((5, 5, 5), np.uint8)
    g3[2, 2, 2] = 0           # isolated voxel: case 1 in every direction
    assert OracleProblem(g3, 3, 2).nhood()[2, 2, 2] == 111


def test_porosity_and_permeability_scaling():
    g = synth.random_solid((10, 8, 6), 0.3, 4)
    a = OracleProblem(g, 0, 2, 1e-5)
    a.iterate(50)
    b = OracleProblem(g, 0, 2, 2e-5)
    b.iterate(50)
    assert abs(a.permeability().porosity - (1 - g.mean())) < 1e-15
    # k scales with dx^2 (evaluation.cc:205-207)
    assert abs(b.permeability().wk33 / a.permeability().wk33 - 4.0) < 1e-12
    c = OracleProblem(g, 0, 2, 1e-5, porosity=0.5)
    c.iterate(50)
    assert abs(c.permeability().wk33 / a.permeability().wk33 - 0.5 / (1 - g.mean())) < 1e-12


def test_convergence_formula():
    g = synth.random_solid((10, 8, 6), 0.3, 4)
    a = OracleProblem(g, 0, 2)
    a.iterate(20)
    conv, k = a.convergence(0.0)
    assert conv == 1.0 and k > 0
    conv2, k2 = a.convergence(k)
    assert conv2 == 0.0 and k2 == k


def test_synthetic_generators():
    c = synth.cylinder()
    assert c.shape == (64, 48, 48) and abs((1 - c.mean()) - 0.548611) < 1e-6
    s = synth.sphere_pack((32, 32, 32), rmin=2, rmax=5, solid_fraction=0.65, seed=3)
    assert 0.64 <= s.mean() <= 0.70 and synth.percolates_z(s)
    gf = synth.gaussian_field((32, 32, 32), 2.0, 0.2, seed=1)
    assert synth.percolates_z(gf) and (gf == 0).mean() <= 0.2 + 1e-6


def test_footprint_counts_each_kernels_stores(lib):
    """pm_problem_footprint (what the server admits requests by) is host
    arithmetic: the FP64 state alone for FP64; the compact store for a pinned
    compact kernel; kernel 13 adds its 16-byte records per voxel; autotuning
    (kernel -1) holds both stores and the records while it times them; the
    padded store for the padded kernels.  Growing the domain grows it."""
    shape = (40, 30, 50)
    nvox = 40 * 30 * 50
    f64 = pm.footprint(shape, precision="fp64")
    c10 = pm.footprint(shape, precision="mixed", kernel=10)
    c13 = pm.footprint(shape, precision="mixed", kernel=13)
    pad = pm.footprint(shape, precision="mixed", kernel=6)
    tune = pm.footprint(shape, precision="mixed", kernel=-1)
    assert f64 < c10 < c13 and f64 < pad
    assert c13 - c10 == 16 * (nvox + 1)
    assert tune >= max(c13, pad) and tune < c13 + pad
    # doubling every axis: 8x the voxels, a little less of the padded halo
    assert pm.footprint((80, 60, 100), precision="mixed", kernel=10) > 5 * (c10 - (1 << 20))
    for k in (8, 9, 11, 12):
        assert pm.footprint(shape, precision="mixed", kernel=k) == c10
