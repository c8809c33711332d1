"""Drop-in behaviour on the GPU: the poremaps_gpu program and the writers
against the golden output of the reference program itself, the full
calc_flow of the small cylinder configuration to convergence, the
dom_interest permeability, and the tensor driver's axis mapping."""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import poremaps_gb300 as pm
from oracle.oracle import OracleProblem
from poremaps_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = np.load(os.path.join(HERE, "golden", "golden.npz"), allow_pickle=False)
META = json.loads(str(GOLDEN["__meta__"]))
CLI_CASES = ["rand_bc0_s1", "rand_bc0_s3", "rand_bc2_s1", "rand_bc4_s3", "rand_dofi",
             "rand_porosity_given", "spheres_converged", "channel_24_14_50"]
PREFIXES = ["velx_", "vely_", "velz_", "press_", "voxel_neighborhood_", "domain_decomp_"]


def run_cli(name, tmp_path, extra=()):
    c = META[name]
    g = make_golden.geometry(c["geom"])
    nz, ny, nx = g.shape
    g.tofile(tmp_path / "geom.raw")
    (tmp_path / "in.inp").write_text(make_golden.inp_text(c, nx, ny, nz))
    r = subprocess.run([pm.CLI_PATH, "in.inp", *extra], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return make_golden.blank_tps((tmp_path / "run.log").read_text())


@pytest.mark.parametrize("name", CLI_CASES)
def test_cli_reference_order_matches_reference_program(name, tmp_path):
    """poremaps_gpu --order reference --arith exact writes the same log rows
    and byte-identical field files as the reference program."""
    log = run_cli(name, tmp_path, ["--order", "reference", "--arith", "exact"])
    assert log == str(GOLDEN[f"{name}/log"])
    for pre in PREFIXES:
        raw = (tmp_path / (pre + "geom.raw")).read_bytes()
        assert hashlib.sha256(raw).hexdigest() == str(GOLDEN[f"{name}/sha_{pre}"]), pre


def test_cli_default_order_converges_to_reference_k(tmp_path):
    """Default (red-black, FMA) run of the converged sphere case: the final
    permeability agrees with the reference program's log to its 7 digits."""
    log = run_cli("spheres_converged", tmp_path)
    last = [c.strip() for c in log.strip().splitlines()[-1].split(",")]
    ref = [c.strip() for c in str(GOLDEN["spheres_converged/log"]).strip().splitlines()[-1].split(",")]
    assert abs(float(last[-1]) - float(ref[-1])) <= 2e-6 * abs(float(ref[-1]))


def test_cli_mixed_precision_converges_to_reference_k(tmp_path):
    """poremaps_gpu --precision mixed (FP32 sweeps + FP64 defect correction)
    on the converged sphere case: the final permeability agrees with the
    reference program's log to its 7 digits."""
    log = run_cli("spheres_converged", tmp_path, ["--precision", "mixed"])
    last = [c.strip() for c in log.strip().splitlines()[-1].split(",")]
    ref = [c.strip() for c in str(GOLDEN["spheres_converged/log"]).strip().splitlines()[-1].split(",")]
    assert abs(float(last[-1]) - float(ref[-1])) <= 2e-6 * abs(float(ref[-1]))
    for pre in ("velz_", "press_"):
        assert (tmp_path / (pre + "geom.raw")).stat().st_size == 8 * 20 * 20 * 20


def test_cli_eps_fixed_point(tmp_path):
    """poremaps_gpu --precision mixed --eps-fixed-point 1e-30: the run goes on
    past the reference's eps stop to the rounding floor of conv and ends
    there; its permeability is the reference program's to its 7 digits."""
    log = run_cli("spheres_converged", tmp_path,
                  ["--precision", "mixed", "--eps-fixed-point", "1e-30"])
    rows = [r for r in log.strip().splitlines() if not r.startswith("#")]
    ref_rows = [r for r in str(GOLDEN["spheres_converged/log"]).strip().splitlines()
                if not r.startswith("#")]
    last = [c.strip() for c in rows[-1].split(",")]
    ref = [c.strip() for c in ref_rows[-1].split(",")]
    assert len(rows) > len(ref_rows) and int(last[0]) < 200000 - 1
    assert float(last[1]) < 1e-10
    assert abs(float(last[-1]) - float(ref[-1])) <= 2e-6 * abs(float(ref[-1]))


def test_c1_cylinder_full_calc_flow_reference_order():
    """48x48x64 cylinder r=20, GS, eps 1e-6: the reference stops at iteration
    64,200 with wk33 = 1.070459e-08 m^2 (Hagen-Poiseuille 1.0908e-08)."""
    g = synth.cylinder(48, 48, 64, 20.0)
    with pm.Problem(g, None, boundary_method=0, solving_algorithm=2, voxel_size=2e-5,
                    eps=1e-6, order="reference", arith=pm.ARITH_EXACT) as p:
        r = p.solve()
    last = [c.strip() for c in str(GOLDEN["c1_cylinder/log"]).strip().splitlines()[-1].split(",")]
    assert r.iterations == int(last[0]) == 64200
    assert f"{r.wk33:e}" == last[-1]
    hp = np.pi * (20 * 2e-5) ** 4 / (8 * (48 * 2e-5) ** 2)
    assert abs(r.wk33 - hp) / hp < 0.03


def test_dom_interest_permeability():
    g = synth.random_solid((18, 12, 14), 0.2, 8)
    di = (2, 9, 1, 10, 3, 17)
    with pm.Problem(g, None, boundary_method=0, solving_algorithm=2, order="reference",
                    arith=pm.ARITH_EXACT, dom_interest=di) as p:
        p.iterate(400)
        r = p.permeability()
    orc = OracleProblem(g, 0, 2, dom_interest=di)
    orc.iterate(400, "reference")
    ro = orc.permeability()
    for a in ("k13", "k23", "k33", "wk13", "wk23", "wk33", "wmax_velz", "wmean_velz"):
        assert abs(getattr(r, a) - getattr(ro, a)) <= 1e-12 * abs(ro.wk33) + 1e-300, a
    assert r.k33 != 0.0


def test_writers_and_neighbourhood(tmp_path, monkeypatch):
    g = synth.random_solid((10, 9, 8), 0.3, 3)
    monkeypatch.chdir(tmp_path)
    with pm.Problem(g, None, boundary_method=1, solving_algorithm=2, voxel_size=3e-5,
                    geometry_file_name="sample.raw", write_output=(1, 1, 1, 1)) as p:
        p.iterate(30)
        u, v, w, pp = p.fields()
        nh = p.nhood()
        p.write_outputs()
    assert np.array_equal(np.fromfile("velx_sample.raw", np.float64).reshape(g.shape), u * 3e-5)
    assert np.array_equal(np.fromfile("press_sample.raw", np.float64).reshape(g.shape), pp)
    assert np.array_equal(np.fromfile("voxel_neighborhood_sample.raw", np.int32).reshape(g.shape),
                          nh)
    assert not np.fromfile("domain_decomp_sample.raw", np.int32).any()
    assert np.array_equal(nh, OracleProblem(g, 1, 2).nhood())


def test_tensor_axis_mapping():
    """A duct along x carries flow only for a pressure drop along x: K[0,0]
    is its permeability and matches the z-duct solved directly."""
    n = 12
    duct_x = np.ones((n, n, n), np.uint8)
    duct_x[4:8, 4:8, :] = 0          # open along x (axis 2 of the z,y,x array)
    duct_z = np.ones((n, n, n), np.uint8)
    duct_z[:, 4:8, 4:8] = 0          # same duct along z
    kw = dict(boundary_method=0, solving_algorithm=2, eps=1e-9, voxel_size=1e-5, porosity=1.0,
              max_iter=20000)
    K, res = pm.solve_tensor(duct_x, None, **kw)
    with pm.Problem(duct_z, None, **kw) as p:
        kz = p.solve().wk33
    assert abs(K[0, 0] - kz) <= 1e-9 * kz
    off = np.abs(K - np.diag(np.diag(K))).max()
    # no path along y or z: those responses vanish up to the stopping error
    assert abs(K[1, 1]) <= 1e-6 * kz and abs(K[2, 2]) <= 1e-6 * kz and off <= 1e-6 * kz


def test_cli_report_full_precision(tmp_path):
    """poremaps_gpu --report out.json: the report's iteration count is the
    log's last row and its wk33, printed at full precision, rounds to the
    log's 7 digits and equals, bit for bit, the oracle's run of the same
    case in the reference order."""
    name = "spheres_converged"
    run_cli(name, tmp_path, ["--order", "reference", "--arith", "exact",
                             "--report", "rep.json"])
    rep = json.loads((tmp_path / "rep.json").read_text())
    last = [c.strip() for c in str(GOLDEN[f"{name}/log"]).strip().splitlines()[-1].split(",")]
    r = rep["result"]
    assert rep["status"] == "ok" and r["converged"] == 1
    assert r["iterations"] == int(last[0])
    assert f"{r['wk33']:e}" == last[-1]
    c = META[name]
    orc = OracleProblem(make_golden.geometry(c["geom"]), c["bc"], c["solver"], c.get("dx", 1e-5))
    ro = orc.calc_flow(c["max_iter"], 100, 100, c["eps"], "reference")
    assert r["wk33"] == ro.wk33 and r["wk13"] == ro.wk13 and r["wk23"] == ro.wk23


def test_cli_tensor(tmp_path):
    """poremaps_gpu --tensor: the three axis-rotated solves of the .inp's
    geometry give the reference program's tensor (16^3 sphere pack, SOR) to
    1e-6 of its scale, and the report carries all nine components."""
    c = META["tensor_s3_z"]
    g = make_golden.geometry(dict(make_golden.TENSOR_GEOM))
    nz, ny, nx = g.shape
    g.tofile(tmp_path / "geom.raw")
    (tmp_path / "in.inp").write_text(make_golden.inp_text(dict(c, max_iter=400000), nx, ny, nz))
    r = subprocess.run([pm.CLI_PATH, "in.inp", "--tensor", "--report", "rep.json"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rep = json.loads((tmp_path / "rep.json").read_text())
    K = np.array(rep["tensor_m2"]).reshape(3, 3)
    K_ref = np.zeros((3, 3))
    slots = {"x": ((1, 0), (2, 0), (0, 0)), "y": ((2, 1), (0, 1), (1, 1)),
             "z": ((0, 2), (1, 2), (2, 2))}
    for rot in "xyz":
        last = [v.strip() for v in
                str(GOLDEN[f"tensor_s3_{rot}/log"]).strip().splitlines()[-1].split(",")]
        for (i, j), lv in zip(slots[rot], last[-3:]):
            K_ref[i, j] = float(lv)
    scale = np.abs(np.diag(K_ref)).max()
    assert np.abs(K - K_ref).max() <= 2e-6 * scale
    assert len(rep["solves"]) == 3 and all(s["converged"] == 1 for s in rep["solves"])
    assert not (tmp_path / "run.log").exists()
