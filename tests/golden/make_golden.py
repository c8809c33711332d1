"""Generate the golden vectors in tests/golden/golden.npz by running the
reference POREMAPS program itself (its own src/*.cc, built unmodified against
the MPI shim by `make -C oracle ref`) on small seeded geometries.

Run in a container where the reference sources exist:
    make -C oracle ref REF_SRC=<reference checkout>/src && python tests/golden/make_golden.py [--slow]

Each case stores the log text (TPS column blanked: it is wall-clock time), the
SHA-256 of every field file the program writes, and for the smallest cases
the field arrays themselves.  --slow adds the long-running cases (the
48x48x64 cylinder at eps 1e-6, ~64k iterations, a few minutes of CPU).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import run_reference_binary  # noqa: E402
from poremaps_gb300 import synth  # noqa: E402


def channel(nx=24, ny=14, nz=50, frame=2):
    g = np.ones((nz, ny, nx), np.uint8)
    g[:, frame:ny - frame, frame:nx - frame] = 0
    return g


def rotate(g, rot):
    """Axis rotation of README.md:221-225: flow along x (z' = x, y' = z,
    x' = y) or along y (z' = y, y' = x, x' = z); the array is (z, y, x)."""
    if rot == "x":
        return np.ascontiguousarray(np.transpose(g, (2, 0, 1)))
    if rot == "y":
        return np.ascontiguousarray(np.transpose(g, (1, 2, 0)))
    return g


def geometry(spec):
    if "rot" in spec:
        return rotate(geometry({k: v for k, v in spec.items() if k != "rot"}), spec["rot"])
    kind = spec["kind"]
    if kind == "random":
        return synth.random_solid(tuple(spec["shape"]), spec["frac"], spec["seed"])
    if kind == "cylinder":
        return synth.cylinder(*spec["size"], radius=spec["radius"])
    if kind == "channel":
        return channel(*spec["size"])
    if kind == "spheres":
        return synth.sphere_pack(tuple(spec["shape"]), rmin=spec["rmin"], rmax=spec["rmax"],
                                 solid_fraction=spec["solid"], seed=spec["seed"])
    raise ValueError(kind)


def inp_text(c, nx, ny, nz):
    di = " ".join(str(v) for v in c.get("dom_interest", [0] * 6))
    dd = " ".join(str(v) for v in c.get("dims", [0, 0, 0]))
    return (f"dom_decomposition {dd}\n"
            f"boundary_method {c['bc']}\n"
            f"geometry_file_name geom.raw\n"
            f"size_x_y_z  {nx} {ny} {nz}\n"
            f"voxel_size  {c.get('dx', 1e-5)}\n"
            f"max_iter    {c['max_iter']}\n"
            f"it_eval    {c.get('it_eval', 100)}\n"
            f"it_write   {c.get('it_write', 100)}\n"
            f"log_file_name run.log\n"
            f"solving_algorithm {c['solver']}\n"
            f"eps {c['eps']}\n"
            f"porosity {c.get('porosity', -1.0)}\n"
            f"dom_interest {di}\n"
            f"write_output 1 1 1 1\n")


R = {"kind": "random", "shape": [16, 10, 12], "frac": 0.2, "seed": 1}
R2 = {"kind": "random", "shape": [14, 12, 10], "frac": 0.25, "seed": 2}
CASES = [
    dict(name="rand_bc0_s1", geom=R, bc=0, solver=1, max_iter=1250, eps=1e-12, fields=True),
    dict(name="rand_bc0_s2", geom=R, bc=0, solver=2, max_iter=1250, eps=1e-12, fields=True),
    dict(name="rand_bc0_s3", geom=R, bc=0, solver=3, max_iter=1250, eps=1e-12, fields=True),
    dict(name="rand_bc1_s2", geom=R2, bc=1, solver=2, max_iter=1150, eps=1e-12, fields=True),
    dict(name="rand_bc2_s1", geom=R2, bc=2, solver=1, max_iter=1150, eps=1e-12, fields=True),
    dict(name="rand_bc3_s2", geom=R2, bc=3, solver=2, max_iter=1150, eps=1e-12, fields=True),
    dict(name="rand_bc4_s3", geom=R2, bc=4, solver=3, max_iter=1150, eps=1e-12, fields=True),
    dict(name="rand_dofi", geom=R, bc=0, solver=2, max_iter=1300, eps=1e-12, fields=False,
         dom_interest=[2, 8, 1, 7, 3, 12]),
    dict(name="rand_porosity_given", geom=R, bc=2, solver=2, max_iter=1101, eps=1e-12,
         fields=False, porosity=0.75, it_eval=50, it_write=100),
    dict(name="rand_slabs2", geom=R, bc=0, solver=2, max_iter=1200, eps=1e-12, fields=False,
         ranks=2, dims=[1, 1, 2]),
    dict(name="rand_slabs3_bc4", geom=R2, bc=4, solver=1, max_iter=1200, eps=1e-12,
         fields=False, ranks=3, dims=[1, 1, 3]),
    dict(name="spheres_converged", geom={"kind": "spheres", "shape": [20, 20, 20], "rmin": 2,
                                          "rmax": 4, "solid": 0.6, "seed": 5},
         bc=0, solver=2, max_iter=200000, eps=1e-8, fields=False),
    dict(name="channel_24_14_50", geom={"kind": "channel", "size": [24, 14, 50]}, bc=0, solver=2,
         max_iter=100000001, eps=1e-7, fields=False, porosity=1.0, dx=5e-5),
]
TENSOR_GEOM = {"kind": "spheres", "shape": [16, 16, 16], "rmin": 1.5, "rmax": 3.0, "solid": 0.55,
               "seed": 11}
TENSOR = [dict(name=f"tensor_s{solver}_{rot}", geom=dict(TENSOR_GEOM, rot=rot), bc=0,
               solver=solver, max_iter=400000, eps=1e-10 if solver == 3 else 1e-9, fields=False)
          for solver in (1, 2, 3) for rot in ("x", "y", "z")]
SLOW = [
    dict(name="c1_cylinder", geom={"kind": "cylinder", "size": [48, 48, 64], "radius": 20.0},
         bc=0, solver=2, max_iter=100000001, eps=1e-6, fields=False, dx=2e-5),
]


def blank_tps(log: str) -> str:
    out = []
    for line in log.splitlines():
        if line.startswith("#"):
            out.append(line)
            continue
        cols = [c.strip() for c in line.split(",")]
        cols[2] = "*"
        out.append(", ".join(cols))
    return "\n".join(out) + "\n"


def run_case(c):
    g = geometry(c["geom"])
    nz, ny, nx = g.shape
    with tempfile.TemporaryDirectory() as d:
        g.tofile(os.path.join(d, "geom.raw"))
        with open(os.path.join(d, "in.inp"), "w") as f:
            f.write(inp_text(c, nx, ny, nz))
        r = run_reference_binary("in.inp", d, nranks=c.get("ranks", 1), timeout=3600)
        if r.returncode != 0:
            raise RuntimeError(f"{c['name']}: reference exited {r.returncode}\n{r.stderr}")
        out = {"log": blank_tps(open(os.path.join(d, "run.log")).read())}
        for pre, dt in (("velx_", np.float64), ("vely_", np.float64), ("velz_", np.float64),
                        ("press_", np.float64), ("voxel_neighborhood_", np.int32),
                        ("domain_decomp_", np.int32)):
            raw = open(os.path.join(d, pre + "geom.raw"), "rb").read()
            out["sha_" + pre] = hashlib.sha256(raw).hexdigest()
            if c.get("fields") and pre != "domain_decomp_":
                out[pre] = np.frombuffer(raw, dt).reshape(nz, ny, nx)
    return out


def main():
    cases = CASES + TENSOR + (SLOW if "--slow" in sys.argv else [])
    if "--only-tensor" in sys.argv:
        cases = TENSOR
    path = os.path.join(HERE, "golden.npz")
    old = dict(np.load(path, allow_pickle=False)) if os.path.exists(path) else {}
    store = dict(old)
    meta = json.loads(str(old["__meta__"])) if "__meta__" in old else {}
    for c in cases:
        print("case", c["name"], flush=True)
        res = run_case(c)
        for k, v in res.items():
            store[f"{c['name']}/{k}"] = np.array(v) if isinstance(v, str) else v
        meta[c["name"]] = {k: v for k, v in c.items() if k != "fields"} | {"fields": bool(c.get("fields"))}
    store["__meta__"] = np.array(json.dumps(meta))
    np.savez_compressed(path, **store)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
