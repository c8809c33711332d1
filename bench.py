#!/usr/bin/env python3
"""Benchmark of the POREMAPS pseudo-time Stokes sweep on GB300.

Workload (default): a 128^3 periodic overlapping-sphere pack (radii U[4,10]
voxels, solid fraction 0.65, z-percolating, seeded), voxel size 1e-5 m,
boundary_method 0, SOR (solving_algorithm 3), eps 1e-6, full permeability
tensor through the three axis-rotated problems.  One step = one it_eval block
(100 sweeps + the convergence evaluation) on each of the three rotated
problems, all resident in HBM.  Headline form: FP32 correction sweeps + FP64
defect correction (mixed); the plain FP64 form is measured beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs N independent replicas (torchrun, one rank per GPU): the solver
does not shard, so there is no data-path collective; the barrier and the
max-over-ranks timing use torch.distributed.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

SWEEPS_PER_BLOCK = 100
ALGO_BYTES_MIXED_INNER = 48.125  # read e (4 x 4 B) + read r (4 x 4 B) + write e (4 x 4 B) + 1 bit
ALGO_BYTES_FP64 = 64.125         # read 4 x 8 B + write 4 x 8 B + 1 bit


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the batched-stream (c4) and request-stream (c5) legs that the "
                         "default single-GPU run adds to its line")
    ap.add_argument("--c4-samples", type=int, default=256)
    ap.add_argument("--relaunch-sweeps", type=int, default=0,
                    help="c4/c5: 1 = the server launches every FP32 sweep separately instead "
                         "of one persistent kernel per round")
    ap.add_argument("--c5-requests", type=int, default=48)
    ap.add_argument("--c5-max-axis", type=int, default=192)
    ap.add_argument("--workload", choices=["c2", "c3", "c4", "c5"], default="c2",
                    help="c2: 128^3 tensor workload (default); c3: one 512^3 sample "
                         "(HBM-streaming roofline); c4: batched uneven samples; c5: serving "
                         "stream with Poisson arrivals")
    ap.add_argument("--samples", type=int, default=64, help="c4/c5: number of requests")
    ap.add_argument("--max-axis", type=int, default=128, help="c5: largest axis length")
    ap.add_argument("--kernel", type=int, default=-1,
                    help="profile case: correction-sweep kernel (-1 autotune)")
    ap.add_argument("--brick", type=int, nargs=3, default=[0, 0, 0],
                    help="profile case: fluid-list brick order for kernels 1/2")
    ap.add_argument("--converge", action="store_true",
                    help="c3: also solve every form to eps 1e-6 and compare k")
    ap.add_argument("--max-iter", type=int, default=100000, help="c3 --converge: iteration cap")
    ap.add_argument("--eps-fixed-point", type=float, default=0.0,
                    help="c3 --converge: pm_params.eps_fixed_point (0: stop at eps 1e-6 as "
                         "calc_flow; > 0: run every form on to that threshold or to the "
                         "rounding floor of conv)")
    ap.add_argument("--write-traffic", default=None, metavar="NCU_CSV",
                    help="write the traffic record of --kernel/--brick from an ncu CSV and exit")
    ap.add_argument("--write-fp64-record", default=None, metavar="NCU_CSV",
                    help="write the FP64-pipe record of the FP64 Jacobi sweep from an ncu CSV")
    ap.add_argument("--profile-case", choices=["mixed", "fp64", "steps"], default=None,
                    help="run two it_eval blocks of one resident problem and exit (a small, "
                         "self-contained case for ncu captures)")
    return ap.parse_args()


def workload(size: int):
    from poremaps_gb300 import synth

    g = synth.sphere_pack((size, size, size), rmin=4.0, rmax=10.0, solid_fraction=0.65,
                          seed=2024)
    # flow along z (as stored), along x (z' = x, y' = z, x' = y), along y (z' = y, y' = x, x' = z)
    rots = [np.ascontiguousarray(g), np.ascontiguousarray(np.transpose(g, (2, 0, 1))),
            np.ascontiguousarray(np.transpose(g, (1, 2, 0)))]
    return g, rots


def config_dict(size, g):
    return {"workload": f"sphere-pack {size}^3 (radii U[4,10], solid 0.65, seed 2024), SOR, "
                        "boundary_method 0, eps 1e-6, 3 axis-rotated problems (tensor)",
            "size": [size, size, size], "porosity": round(float(1 - g.mean()), 6),
            "solving_algorithm": 3, "boundary_method": 0, "voxel_size": 1e-5,
            "sweeps_per_step": 3 * SWEEPS_PER_BLOCK, "order": "jacobi",
            "streams": "the three rotated problems run concurrently, one CUDA stream each",
            "l2": "256 MB buffer written between timed steps",
            "parallelism": "replicas (one independent domain per GPU)"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            c = [x.strip() for x in ln.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax = max(smax, float(c[2]))
            except ValueError:
                continue
            for n, v in zip(names, c[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU side
def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def write_case(d, g, max_iter=100000001, bc=0, solver=3):
    nz, ny, nx = g.shape
    g.tofile(os.path.join(d, "geom.raw"))
    with open(os.path.join(d, "in.inp"), "w") as f:
        f.write(f"dom_decomposition 1 1 1\nboundary_method {bc}\ngeometry_file_name geom.raw\n"
                f"size_x_y_z  {nx} {ny} {nz}\nvoxel_size  1e-05\nmax_iter    {max_iter}\n"
                f"it_eval    100\nit_write   100\nlog_file_name run.log\n"
                f"solving_algorithm {solver}\n"
                f"eps 1e-06\nporosity -1.0\ndom_interest 0 0 0 0 0 0\nwrite_output 0 0 0 0\n")


def oracle_cli():
    path = os.path.join(ROOT, "oracle", "_build", "oracle_cli")
    if not os.path.exists(path):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True,
                       stdout=subprocess.DEVNULL)
    return path


def cpu_run(g, sweeps: int, cores: int):
    """The CPU restatement of the reference sweep (bitwise equal to the
    reference program) on `cores` z-slabs, one thread each: the reference run
    with dom_decomposition 1 1 cores."""
    with tempfile.TemporaryDirectory() as d:
        write_case(d, g)
        r = subprocess.run([oracle_cli(), "in.inp", "--slabs", str(cores), "--threads",
                            str(cores), "--sweeps", str(sweeps)], cwd=d, capture_output=True,
                           text=True, check=True)
        return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_cores(nz: int) -> int:
    n = os.cpu_count() or 1
    return max(1, min(n, nz // 2))


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    g, _ = workload(args.size)
    cores = cpu_cores(g.shape[0])
    times = []
    for i in range(args.warmup + args.steps):
        r = cpu_run(g, SWEEPS_PER_BLOCK, cores)
        if i >= args.warmup:
            times.append(r["seconds"])
    sec = statistics.mean(times)
    glups = g.size * SWEEPS_PER_BLOCK / sec / 1e9
    sample = (f"{SWEEPS_PER_BLOCK} sweeps of the unrotated {args.size}^3 problem per step "
              f"(reference order, {cores} z-slabs)")
    out = {"metric": "GLUP/s", "value": glups, "unit": "GLUP/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "impl": "reference", "config": config_dict(args.size, g),
           "cpu_baseline": {"value": glups, "unit": "GLUP/s", "cores": cores, "kind": "port",
                            "sample": sample},
           "e2e": {"value": glups, "unit": "GLUP/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    out["config"]["sweeps_per_step"] = SWEEPS_PER_BLOCK
    out["config"]["order"] = "reference (in-place lexicographic, per slab)"
    for k in ("streams", "l2"):  # notes about the GPU arm's step
        out["config"].pop(k, None)
    print(json.dumps(out), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch

    import poremaps_gb300 as pm
    from poremaps_gb300.replicas import Replicas

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    pm.set_device(local)
    rep = Replicas("nccl")
    world, rank = rep.world, rep.rank

    def barrier():
        rep.barrier()
        torch.cuda.synchronize()

    max_over_ranks = rep.max

    g, rots = workload(args.size)
    nvox = g.size
    flush = torch.empty(256 * 2**20 // 4, dtype=torch.float32, device="cuda")
    common = dict(solving_algorithm=3, boundary_method=0, voxel_size=1e-5, eps=1e-6,
                  it_eval=SWEEPS_PER_BLOCK, it_write=SWEEPS_PER_BLOCK, order="jacobi")

    def timed_form(precision: str, steps: int, warmup: int):
        probs = [pm.Problem(r, None, precision=precision, **common) for r in rots]
        perm = [0.0, 0.0, 0.0]
        conv = [0.0, 0.0, 0.0]
        # one step: one it_eval block of each rotated problem, the three
        # issued concurrently on their own streams (as pm_solve_tensor runs
        # them), timed with CUDA events from a common start to a joined end
        for _ in range(warmup):
            _, conv, perm = pm.block_group_timed(probs, SWEEPS_PER_BLOCK, True, perm)
        barrier()
        launches0 = pm.kernel_launches()
        total_ms = 0.0
        with ClockSampler(local) as clk:
            for _ in range(steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                ms, conv, perm = pm.block_group_timed(probs, SWEEPS_PER_BLOCK, True, perm)
                total_ms += ms
            barrier()
        launches = pm.kernel_launches() - launches0
        ms_step = max_over_ranks(total_ms / steps)
        return probs, perm, ms_step, launches, clk.summary()

    # headline: mixed precision
    probs_mx, perm_mx, ms_mx, launches_mx, clocks = timed_form("mixed", args.steps, args.warmup)
    lups_step = 3 * SWEEPS_PER_BLOCK * nvox
    value = world * lups_step / (ms_mx * 1e-3) / 1e9
    kernel_ms = probs_mx[2].kernel_time(0, 50)
    kid = probs_mx[2].kernel()
    kshort, kdesc = KERNELS[kid]
    kname = f"{kshort} ({kdesc})"
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = nvox * ALGO_BYTES_MIXED_INNER / (kernel_ms * 1e-3) / 1e9
    brick = list(probs_mx[2].brick())
    traffic, traffic_note = kernel_traffic(kid, brick, args.size, nvox)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "frac_dram": (traffic / (kernel_ms * 1e-3) / 1e9 / peak) if traffic else None,
                "traffic_source": traffic_note,
                "model": "achieved/frac: dense model (every voxel of the unpadded domain, "
                         f"{ALGO_BYTES_MIXED_INNER} B); frac_dram: the chosen kernel's measured "
                         "DRAM bytes per launch over the same CUDA-event launch time. The "
                         "fluid-list sweep skips solid regions, so the dense model can exceed 1",
                "kernel": kname, "kernel_choice": "autotuned at problem creation",
                "kernel_id": kid, "brick": brick,
                "kernels_per_rotation": [[KERNELS[p.kernel()][0], list(p.brick())]
                                         for p in probs_mx],
                "algorithmic_bytes_per_lup": ALGO_BYTES_MIXED_INNER,
                "kernel_ms": kernel_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst, of measured)" if peaks
                               else "fallback 6.8 TB/s (of fallback)"}
    phi = float(1 - g.mean())  # every rotation has the same fluid count
    forms = {"mixed": {"glups": value, "fluid_glups": value * phi, "ms_per_step": ms_mx,
                       "inner_kernel_ms": kernel_ms}}

    k_rel = None
    if not args.no_fp64:
        probs_64, perm_64, ms_64, _, _ = timed_form("fp64", max(2, args.steps // 2),
                                                    max(1, args.warmup))
        k64 = probs_64[2].kernel_time(0, 10)
        glups64 = world * lups_step / (ms_64 * 1e-3) / 1e9
        forms["fp64"] = {"glups": glups64, "fluid_glups": glups64 * phi, "ms_per_step": ms_64,
                         "sweep_kernel_ms": k64,
                         "hbm_frac_of_measured": nvox * ALGO_BYTES_FP64 / (k64 * 1e-3) / 1e9 / peak,
                         "fp64_pipe": fp64_pipe_record(args.size, k64),
                         "note": "FP64 sweeps are bound by the FP64 pipe of GB300, not by HBM"}
        for p in probs_64:
            p.close()
    # k of the mixed form against the FP64 form after the same 1200 iterations
    # (same ordering, same trajectory in exact arithmetic)
    if not args.no_fp64:
        ks = []
        for prec in ("mixed", "fp64"):
            with pm.Problem(rots[2], None, precision=prec, **common) as p:
                p.iterate(1200)
                ks.append(p.permeability())
        k_rel_components = {a: abs(getattr(ks[0], a) - getattr(ks[1], a)) / abs(ks[1].wk33)
                            for a in ("wk13", "wk23", "wk33")}
        k_rel = max(k_rel_components.values())
    res_mx = [p.permeability() for p in probs_mx]
    for p in probs_mx:
        p.close()

    # end to end: the C-ABI tensor call from host geometry to host K
    # (one untimed call, then the mean of E2E_CALLS calls: a call takes ~40 ms)
    e2e_iters = 1200
    e2e_times = []
    for i in range(1 + E2E_CALLS):
        barrier()
        t0 = time.perf_counter()
        K, res3 = pm.solve_tensor(g, None, max_iter=e2e_iters, precision="mixed", **common)
        t1 = time.perf_counter()
        if i >= 1:
            e2e_times.append(t1 - t0)
    e2e_s = max_over_ranks(statistics.mean(e2e_times))
    checks = len([it for it in range(1001, e2e_iters) if it % SWEEPS_PER_BLOCK == 0])
    e2e = {"value": world * 3 * e2e_iters * nvox / e2e_s / 1e9, "unit": "GLUP/s",
           "h2d_bytes_per_step": 3 * nvox,
           "d2h_bytes_per_step": 3 * (checks + 1) * 9 * 8 + 9 * 8,
           "seconds_per_step": e2e_s,
           "step": f"pm_solve_tensor, {e2e_iters} iterations per rotated problem, host geometry "
                   f"in, host tensor out; mean of {E2E_CALLS} calls after one untimed call"}
    if not args.no_fp64:
        # the same call for the plain FP64 form (the reference's precision)
        t64 = []
        for i in range(1 + E2E_CALLS_FP64):
            barrier()
            t0 = time.perf_counter()
            K64, _ = pm.solve_tensor(g, None, max_iter=e2e_iters, precision="fp64", **common)
            t1 = time.perf_counter()
            if i >= 1:
                t64.append(t1 - t0)
        s64 = max_over_ranks(statistics.mean(t64))
        forms["fp64"]["e2e"] = {"value": world * 3 * e2e_iters * nvox / s64 / 1e9,
                                "unit": "GLUP/s", "seconds_per_step": s64,
                                "h2d_bytes_per_step": e2e["h2d_bytes_per_step"],
                                "d2h_bytes_per_step": e2e["d2h_bytes_per_step"],
                                "tensor_rel_diff_vs_mixed":
                                    float(np.abs(K64 - K).max() / np.abs(np.diag(K64)).max())}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = cpu_cores(g.shape[0])
        sweeps = 200
        r = cpu_run(g, sweeps, cores)
        cpu = {"value": r["mlups"] / 1e3, "unit": "GLUP/s", "cores": cores, "kind": "port",
               "sample": f"{sweeps} reference-order sweeps of the unrotated {args.size}^3 "
                         f"problem on {cores} z-slab threads (oracle restatement, bitwise equal "
                         f"to the reference program), {r['seconds']:.2f} s"}

    if rank == 0:
        out = {"metric": "GLUP/s", "value": value, "unit": "GLUP/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mx,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32+f64", "data": "synthetic", "config": config_dict(args.size, g),
               "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
               "gpu_launches": int(launches_mx), "forms": forms,
               "tensor_k_m2": K.tolist(),
               "mixed_wk33_after_timed_blocks": [r.wk33 for r in res_mx]}
        if k_rel is not None:
            out["k_rel_diff_vs_fp64"] = k_rel
            out["k_rel_diff_vs_fp64_components"] = k_rel_components
        if world == 1 and not args.no_serving:
            # the serving target: batched mixed vs plain FP64 solves/h on the
            # uneven stream, and latency percentiles on a request stream
            out["c4"] = c4_result(args.c4_samples, with_cpu=not args.no_cpu_baseline)
            out["c5"] = c5_result(args.c5_requests, args.c5_max_axis)
        print(json.dumps(out), flush=True)
    rep.close()
    return 0


def kernel_traffic(kid, brick, size, nvox):
    """DRAM bytes per launch of the chosen correction sweep from its committed
    ncu capture (profiles/*_traffic.json), only when that capture is of the
    same kernel id and fluid-list order and of the kernel sources as they are
    now (their SHA-256 is recorded at capture time); otherwise None, with the
    reason."""
    import hashlib

    tpath = os.path.join(ROOT, "profiles", f"{KERNELS[kid][0]}_sphere{size}_traffic.json")
    if not os.path.exists(tpath):
        return None, f"no ncu capture of {KERNELS[kid][0]} on this workload"
    t = json.load(open(tpath))
    if t.get("kernel_id") != kid or list(t.get("brick", [])) != list(brick):
        return None, (f"capture is of kernel {t.get('kernel_id')} brick {t.get('brick')}, "
                      f"the autotuner chose {kid} brick {brick}")
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        h.update(open(os.path.join(ROOT, f), "rb").read())
    if t.get("sources") != KERNEL_SOURCES or h.hexdigest() != t.get("sources_sha256"):
        return None, "kernel sources changed since the capture"
    return t["dram_bytes_per_launch"] * nvox / t["nvox"], t["source"]


# Sources of each correction-sweep kernel: a traffic capture is valid while
# their SHA-256 is the one recorded with it.
KERNEL_SOURCES = ["poremaps_gb300/csrc/pm_fast.cu", "poremaps_gb300/csrc/pm_compact.cu",
                  "poremaps_gb300/csrc/pm_compact.cuh", "poremaps_gb300/csrc/pm_stencil.cuh",
                  "poremaps_gb300/csrc/pm_internal.h"]


FP64_SOURCES = ["poremaps_gb300/csrc/pm_fast.cu", "poremaps_gb300/csrc/pm_stencil.cuh",
                "poremaps_gb300/csrc/pm_internal.h"]


def _sources_sha(files):
    import hashlib

    h = hashlib.sha256()
    for f in files:
        h.update(open(os.path.join(ROOT, f), "rb").read())
    return h.hexdigest()


def _ncu_rows(csv_path, kname):
    """(launch id -> {metric: value}) of the launches of kernel kname in an
    ncu --csv log."""
    import csv

    with open(csv_path) as f:
        rows = [r for r in csv.reader(f) if len(r) > 10]
    head = rows[0]
    ci = {n: head.index(n) for n in ("ID", "Kernel Name", "Metric Name", "Metric Unit",
                                     "Metric Value")}
    scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "ns": 1e-3, "us": 1.0,
             "ms": 1e3, "%": 1.0, "inst": 1.0, "": 1.0}
    per = {}
    for r in rows[1:]:
        if kname not in r[ci["Kernel Name"]]:
            continue
        v = float(r[ci["Metric Value"]].replace(",", "")) * scale.get(r[ci["Metric Unit"]], 1.0)
        per.setdefault(r[ci["ID"]], {})[r[ci["Metric Name"]]] = v
    return per


def write_fp64_record(csv_path, size):
    """FP64-pipe record of the FP64 Jacobi sweep (k_sweep64_pf) from an ncu CSV
    of `bench.py --profile-case fp64` with the metrics
    sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active,
    sm__inst_executed_pipe_fp64.sum and gpu__time_duration.sum."""
    per = _ncu_rows(csv_path, "k_sweep64_pf")
    if not per:
        raise SystemExit(f"no k_sweep64_pf launches in {csv_path}")
    first = per[sorted(per, key=int)[0]]  # the Jacobi sweep's launches come first
    out = {"kernel": "k_sweep64_pf", "workload": f"{size}^3 sphere pack (bench default), FP64 "
                                                "Jacobi, one rotated problem",
           "fp64_pipe_active_pct": first["sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active"],
           "fp64_warp_instructions": first["sm__inst_executed_pipe_fp64.sum"],
           "duration_us": first["gpu__time_duration.sum"],
           "sources": FP64_SOURCES, "sources_sha256": _sources_sha(FP64_SOURCES),
           "source": "ncu --metrics sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active,"
                     "sm__inst_executed_pipe_fp64.sum,gpu__time_duration.sum --clock-control none "
                     "-k regex:k_sweep64_pf -s 2 -c 1 python bench.py --profile-case fp64; "
                     "one launch, cold caches"}
    path = os.path.join(ROOT, "profiles", f"k_sweep64_pf_sphere{size}_fp64pipe.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out))
    return 0


def fp64_pipe_record(size, kernel_ms):
    """The FP64 Jacobi sweep's FP64-pipe utilisation: measured by ncu on one
    cold launch, and scaled to the warm event time of this run (the pipe does
    the same work in less time when the caches are warm)."""
    path = os.path.join(ROOT, "profiles", f"k_sweep64_pf_sphere{size}_fp64pipe.json")
    if not os.path.exists(path):
        return None
    t = json.load(open(path))
    if t.get("sources") != FP64_SOURCES or t.get("sources_sha256") != _sources_sha(FP64_SOURCES):
        return {"stale": "kernel sources changed since the capture"}
    return {"active_pct_ncu_cold": t["fp64_pipe_active_pct"],
            "active_frac_at_event_time": t["fp64_pipe_active_pct"] / 100.0 *
            (t["duration_us"] * 1e-3) / kernel_ms,
            "fp64_warp_instructions_per_sweep": t["fp64_warp_instructions"],
            "source": t["source"]}


def write_traffic(csv_path, kid, brick, size):
    """Turn an ncu CSV of the chosen correction sweep (the metrics
    dram__bytes_read.sum and dram__bytes_write.sum, launches of
    `bench.py --profile-case mixed --kernel K --brick ...`) into
    profiles/<kernel>_sphere<size>_traffic.json, keyed to the kernel id, the
    list order and the SHA-256 of the kernel sources."""
    import csv
    import hashlib

    per = {}
    with open(csv_path) as f:
        rows = [r for r in csv.reader(f) if len(r) > 10]
    head = rows[0]
    ci = {n: head.index(n) for n in ("ID", "Kernel Name", "Metric Name", "Metric Unit",
                                     "Metric Value")}
    scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    kshort = KERNELS[kid][0]
    for r in rows[1:]:
        if kshort not in r[ci["Kernel Name"]]:
            continue
        m = r[ci["Metric Name"]]
        if m in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            v = float(r[ci["Metric Value"]].replace(",", "")) * scale[r[ci["Metric Unit"]]]
            per[r[ci["ID"]]] = per.get(r[ci["ID"]], 0.0) + v
    if not per:
        raise SystemExit(f"no {kshort} launches with DRAM metrics in {csv_path}")
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        h.update(open(os.path.join(ROOT, f), "rb").read())
    out = {"kernel": kshort, "kernel_id": kid, "brick": list(brick),
           "workload": f"{size}^3 sphere pack (bench default), mixed, one rotated problem",
           "nvox": size ** 3, "dram_bytes_per_launch": statistics.mean(per.values()),
           "launches": len(per), "sources": KERNEL_SOURCES, "sources_sha256": h.hexdigest(),
           "source": "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum "
                     f"--clock-control none -k regex:{kshort} -s 5 -c 2 python bench.py "
                     f"--profile-case mixed --kernel {kid} --brick {' '.join(map(str, brick))}; "
                     "mean over the captured launches, cold caches, the bench's problem size"}
    path = os.path.join(ROOT, "profiles", f"{kshort}_sphere{size}_traffic.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out))
    return 0


# timed end-to-end tensor calls (mixed ~40 ms each, FP64 ~150 ms each)
E2E_CALLS = 8
E2E_CALLS_FP64 = 3

KERNELS = {0: ("k_zmarch_inner", "32x16 tiles, TMA z-march FP32 correction sweep"),
           3: ("k_zmarch_inner", "32x8 tiles, TMA z-march FP32 correction sweep"),
           1: ("k_dc_inner", "fluid-list FP32 correction sweep"),
           2: ("k_dc_inner_occ", "fluid-list FP32 correction sweep, 4 blocks/SM"),
           4: ("k_brick_inner", "TMA brick tiles, FP32 correction sweep"),
           5: ("k_dc_inner_pf", "persistent fluid-list FP32 correction sweep, 4 blocks/SM"),
           6: ("k_dc_inner_pf", "persistent fluid-list FP32 correction sweep, 3 blocks/SM"),
           7: ("k_dc_inner_pf", "persistent fluid-list FP32 correction sweep, 2 blocks/SM"),
           8: ("k_dc_inner_c", "persistent FP32 correction sweep over the compact fluid store, "
                               "3 blocks/SM"),
           9: ("k_dc_inner_c", "persistent FP32 correction sweep over the compact fluid store, "
                               "4 blocks/SM"),
           10: ("k_dc_inner_c", "persistent FP32 correction sweep over the compact fluid store, "
                                "5 blocks/SM, no slot prefetch"),
           11: ("k_dc_inner_cb", "persistent FP32 correction sweep over the compact fluid store, "
                                 "slots staged in shared memory by bulk copies, 5 blocks/SM"),
           12: ("k_dc_inner_cb", "persistent FP32 correction sweep over the compact fluid store, "
                                 "slots staged in shared memory by bulk copies, 4 blocks/SM"),
           13: ("k_dc_inner_cr", "persistent FP32 correction sweep over the compact fluid store, "
                                 "16-byte packed neighbour records, 5 blocks/SM")}


def run_profile_case(args):
    import poremaps_gb300 as pm

    if args.profile_case == "steps":
        # the headline's timed loop alone: the three rotated mixed problems,
        # --warmup + --steps concurrent it_eval blocks (for a launch list)
        g, rots = workload(args.size)
        probs = [pm.Problem(r, None, precision="mixed", solving_algorithm=3, boundary_method=0,
                            voxel_size=1e-5, eps=1e-6, it_eval=SWEEPS_PER_BLOCK,
                            it_write=SWEEPS_PER_BLOCK, order="jacobi") for r in rots]
        perm = [0.0, 0.0, 0.0]
        for _ in range(args.warmup + args.steps):
            _, _, perm = pm.block_group_timed(probs, SWEEPS_PER_BLOCK, True, perm)
        for p in probs:
            p.close()
        return 0
    if args.workload == "c3":
        # the c3 medium at --size (a few GB on the device at 256^3): two
        # it_eval blocks of the mixed form, or of FP64 Jacobi and red-black
        from poremaps_gb300 import synth

        g = synth.gaussian_field((args.size,) * 3, 3.0, 0.20, seed=3)
        kw = dict(boundary_method=2, solving_algorithm=2, voxel_size=5e-6)
        forms = ([dict(precision="mixed", order="jacobi", kernel=args.kernel, brick=args.brick)]
                 if args.profile_case == "mixed" else
                 [dict(precision="fp64", order="jacobi"), dict(precision="fp64", order="redblack")])
        for extra in forms:
            with pm.Problem(g, None, **extra, **kw) as p:
                for _ in range(2):
                    p.block_timed(SWEEPS_PER_BLOCK, True)
        return 0
    g, rots = workload(args.size)
    with pm.Problem(rots[2], None, precision=args.profile_case, solving_algorithm=3,
                    boundary_method=0, voxel_size=1e-5, order="jacobi", kernel=args.kernel,
                    brick=args.brick) as p:
        for _ in range(2):
            p.block_timed(SWEEPS_PER_BLOCK, True)
        if args.profile_case == "mixed":
            print(json.dumps({"kernel": KERNELS[p.kernel()][0], "brick": p.brick()}), flush=True)
    if args.profile_case == "fp64":  # and the red-black FP64 form (the default order)
        with pm.Problem(rots[2], None, precision="fp64", solving_algorithm=3, boundary_method=0,
                        voxel_size=1e-5, order="redblack") as p:
            for _ in range(2):
                p.block_timed(SWEEPS_PER_BLOCK, True)
    return 0


# ------------------------------------------------------------------ serving workloads
def c4_samples(n: int, seed: int = 4):
    """Uneven samples: each axis from {32,48,64,96,128}; half sphere packs
    (radii U[2,8]), half thresholded Gaussian fields (sigma U[1.5,4]); target
    porosity U[0.15,0.5]; boundary_method 0 or 1; per-sample seeds."""
    from poremaps_gb300 import synth

    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        shape = tuple(int(v) for v in rng.choice([32, 48, 64, 96, 128], 3))
        phi = float(rng.uniform(0.15, 0.5))
        bc = int(rng.integers(0, 2))
        if i % 2 == 0:
            g = synth.sphere_pack(shape, rmin=2.0, rmax=8.0, solid_fraction=1 - phi,
                                  seed=seed * 100003 + i)
        else:
            g = synth.gaussian_field(shape, float(rng.uniform(1.5, 4.0)), phi,
                                     seed=seed * 100003 + i)
        out.append((g, bc))
    return out


def c5_samples(n: int, max_axis: int, seed: int = 5):
    """Serving stream: axes log-uniform in [32, max_axis], generators as c4,
    porosity U[0.12,0.45], boundary_method in {0,1,2}.  A Gaussian draw that
    does not percolate along z at its porosity (low porosity, large sigma,
    long z) is redrawn with the porosity raised in steps of 0.02."""
    from poremaps_gb300 import synth

    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        shape = tuple(int(round(np.exp(rng.uniform(np.log(32), np.log(max_axis))))) for _ in range(3))
        phi = float(rng.uniform(0.12, 0.45))
        bc = int(rng.integers(0, 3))
        if i % 2 == 0:
            g = synth.sphere_pack(shape, rmin=2.0, rmax=8.0, solid_fraction=1 - phi,
                                  seed=seed * 100003 + i)
        else:
            g = synth.gaussian_field(shape, float(rng.uniform(1.5, 4.0)), phi,
                                     seed=seed * 100003 + i, relax=0.02)
        out.append((g, bc))
    return out


SERVE_KW = dict(solving_algorithm=2, voxel_size=1e-5, eps=1e-6, it_eval=100, it_write=100,
                max_iter=200000)
# Below this |wk33| (1e-10 dx^2) a sample's permeability is numerically zero
# (e.g. a percolating cluster whose throats are one voxel wide): the fields
# are round-off around a zero-flow state and a relative error means nothing.
K_ZERO = 1e-10 * SERVE_KW["voxel_size"] ** 2


def k_errors(pairs):
    """pairs: (mixed result, fp64 result) per sample.  Relative error of the
    three components (over |wk33|) where k is not numerically zero; absolute
    values listed for the rest."""
    rel, zero = [], []
    for i, (m, r) in enumerate(pairs):
        d = max(abs(m.wk13 - r.wk13), abs(m.wk23 - r.wk23), abs(m.wk33 - r.wk33))
        if abs(r.wk33) < K_ZERO:
            zero.append({"index": i, "fp64_wk33": r.wk33, "mixed_wk33": m.wk33, "abs_diff": d})
            rel.append(0.0)
        else:
            rel.append(d / abs(r.wk33))
    nz = [x for i, x in enumerate(rel) if not any(z["index"] == i for z in zero)]
    return rel, {"max": max(nz) if nz else 0.0, "median": float(np.median(nz)) if nz else 0.0,
                 "samples_above_1e-6": sum(x > 1e-6 for x in nz),
                 "numerically_zero_k": {"threshold_m2": K_ZERO, "samples": zero}}


def unconverged(results):
    """Indices of the requests that reached max_iter without meeting the stop
    rule: they count neither as solves nor in the latency percentiles."""
    return [i for i, r in enumerate(results) if not r.converged]


def c4_result(n_samples: int, relaunch: int = 0, with_cpu: bool = True):
    """The batched uneven stream (configuration 4) through the mixed-precision
    server against the plain FP64 form solving the samples one by one."""
    import poremaps_gb300 as pm

    t_gen = time.perf_counter()
    reqs = c4_samples(n_samples)
    t_gen = time.perf_counter() - t_gen
    nvox = sum(g.size for g, _ in reqs)
    # batched mixed-precision server
    srv = pm.Server(precision="mixed", use_graphs=1, autotune=1, relaunch_sweeps=relaunch)
    t0 = time.perf_counter()
    tickets = {srv.submit(g, boundary_method=bc, **SERVE_KW): i for i, (g, bc) in enumerate(reqs)}
    done = {}
    while len(done) < len(reqs):
        srv.step()
        for c in srv.poll():
            done[tickets[c.ticket]] = c
    t_mx = time.perf_counter() - t0
    busy, wall, lups = srv.stats()
    shape = srv.launch_shape()  # the autotuner's choice for the last resident set
    srv.close()
    # plain FP64 GPU form, one sample after another (Jacobi order, FMA form: the
    # fastest FP64 form and the same ordering as the mixed form)
    t0 = time.perf_counter()
    plain = []
    for g, bc in reqs:
        with pm.Problem(g, None, boundary_method=bc, precision="fp64", order="jacobi",
                        **SERVE_KW) as p:
            plain.append(p.solve())
    t_64 = time.perf_counter() - t0
    rel, kerr = k_errors([(done[i].result, r) for i, r in enumerate(plain)])
    cpu = c4_cpu_estimate(reqs, [r.iterations for r in plain]) if with_cpu else None
    if cpu:
        cpu["batched_mixed_speedup"] = (3600.0 * len(reqs) / t_mx) / cpu["solves_per_h"]
    unc_mx = unconverged([done[i].result for i in range(len(reqs))])
    unc_64 = unconverged(plain)
    out = {"metric": "solves/h", "value": 3600.0 * len(reqs) / t_mx, "unit": "solves/h",
           "n_gpus": 1, "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic",
           "config": {"workload": f"{len(reqs)} uneven samples (axes from {{32,48,64,96,128}}), "
                                  "half sphere packs r U[2,8], half Gaussian sigma U[1.5,4], "
                                  "porosity U[0.15,0.5], bc 0/1, GS, eps 1e-6",
                      "total_voxels": nvox, "generation_s": t_gen},
           "batched_mixed": {"solves_per_h": 3600.0 * len(reqs) / t_mx, "seconds": t_mx,
                             "converged_solves_per_h":
                                 3600.0 * (len(reqs) - len(unc_mx)) / t_mx,
                             "unconverged_at_max_iter": unc_mx,
                             "device_busy_ms": busy, "glups_busy": lups / (busy * 1e6),
                             "launch_shape_last": shape},
           "plain_fp64": {"solves_per_h": 3600.0 * len(reqs) / t_64, "seconds": t_64,
                          "converged_solves_per_h": 3600.0 * (len(reqs) - len(unc_64)) / t_64,
                          "unconverged_at_max_iter": unc_64},
           "speedup_vs_plain_fp64": t_64 / t_mx,
           "k_rel_err_vs_plain_fp64": kerr,
           "cpu_reference_estimate": cpu,
           "iterations": {"min": min(c.result.sweeps for c in done.values()),
                          "max": max(c.result.sweeps for c in done.values())}}
    order = sorted(range(len(rel)), key=lambda i: -rel[i])
    out["failed"] = [{"index": i, "status": done[i].status} for i in range(len(reqs))
                     if done[i].status != 0]
    out["worst_samples"] = [
        {"index": i, "shape": list(reqs[i][0].shape), "boundary_method": reqs[i][1],
         "porosity": round(float(1 - reqs[i][0].mean()), 4), "rel_err": rel[i],
         "status": done[i].status,
         "mixed": {"iterations": done[i].result.iterations,
                   "converged": bool(done[i].result.converged), "wk33": done[i].result.wk33},
         "fp64": {"iterations": plain[i].iterations, "converged": bool(plain[i].converged),
                  "wk33": plain[i].wk33}} for i in order[:5]]
    return out


def c4_cpu_estimate(reqs, iterations, cores=None, sweeps=100):
    """Solves/h of the reference's CPU path on the c4 stream, as the reference
    would serve it on this host: one np=1 process per core, each solving one
    sample.  A subsample of the stream (every k-th sample, one per core) runs
    `sweeps` reference-order sweeps of the oracle restatement (bitwise the
    reference program) at once, one process per sample, which gives the
    per-core MLUP/s under full load; each sample's solve is then
    voxels x iterations at that rate, with the iterations the plain FP64 GPU
    form needed for it (Jacobi order; the reference's in-place order needs
    counts of the same size: 0.76-1.00 of them, mean 0.95, on the six
    smallest samples of this stream run to eps 1e-6 on the CPU oracle)."""
    n = len(reqs)
    cores = cores or min(16, os.cpu_count() or 1)
    pick = list(range(0, n, max(1, n // cores)))[:cores]
    cli = oracle_cli()
    with tempfile.TemporaryDirectory() as root:
        procs = []
        for i in pick:
            d = os.path.join(root, str(i))
            os.makedirs(d)
            g, bc = reqs[i]
            write_case(d, g, bc=bc, solver=SERVE_KW["solving_algorithm"])
            procs.append((i, subprocess.Popen([cli, "in.inp", "--sweeps", str(sweeps)], cwd=d,
                                              stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                              text=True)))
        rates = []
        for i, pr in procs:
            out, _ = pr.communicate()
            if pr.returncode != 0:
                raise RuntimeError(f"oracle_cli failed on c4 sample {i}")
            r = json.loads(out.strip().splitlines()[-1])
            rates.append(reqs[i][0].size * sweeps / r["seconds"])
    rate = float(np.mean(rates))  # lattice updates per second per core
    core_s = sum(g.size * it for (g, _), it in zip(reqs, iterations)) / rate
    sph = 3600.0 * n / (core_s / cores)
    return {"solves_per_h": sph, "unit": "solves/h", "cores": cores, "kind": "port",
            "mlups_per_core": rate / 1e6,
            "sample": f"{len(pick)} of the {n} samples, {sweeps} reference-order sweeps each, "
                      f"one single-threaded process per sample at once; every sample's solve "
                      f"extrapolated as voxels x the plain FP64 GPU form's iterations at the "
                      f"mean per-core rate, {cores} cores"}


def run_c4(args):
    import poremaps_gb300 as pm

    pm.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    print(json.dumps(c4_result(args.samples, args.relaunch_sweeps)), flush=True)
    return 0


def pcts(lat, skip=()):
    keep = np.array([x for i, x in enumerate(lat) if i not in set(skip)])
    if keep.size == 0:
        return {"p50_s": None, "p99_s": None}
    return {"p50_s": float(np.percentile(keep, 50)), "p99_s": float(np.percentile(keep, 99))}


def c5_result(n_requests: int, max_axis: int, relaunch: int = 0):
    """A serving stream (configuration 5): Poisson arrivals through the
    mixed-precision server, and the plain FP64 form serving the same arrivals
    one request at a time."""
    import poremaps_gb300 as pm

    reqs = c5_samples(n_requests, max_axis)
    # arrival rate: keep the device busy -- mean inter-arrival = 0.6 x the mean
    # solve time estimated from the first request alone (scaled by voxels)
    rng = np.random.default_rng(55)
    srv = pm.Server(precision="mixed", use_graphs=1, autotune=1, relaunch_sweeps=relaunch)
    probe = time.perf_counter()
    t = {srv.submit(reqs[0][0], boundary_method=reqs[0][1], **SERVE_KW): 0}
    while srv.step():
        pass
    srv.poll()
    solo = time.perf_counter() - probe
    gaps = rng.exponential(0.6 * solo * np.mean([g.size for g, _ in reqs]) / reqs[0][0].size,
                           len(reqs))
    arrive = np.cumsum(gaps) - gaps[0]
    t0 = time.perf_counter()
    tickets, done, nxt = {}, {}, 0
    while len(done) < len(reqs):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and arrive[nxt] <= now:
            g, bc = reqs[nxt]
            tickets[srv.submit(g, boundary_method=bc, **SERVE_KW)] = nxt
            nxt += 1
        if srv.step() == 0 and nxt < len(reqs):
            time.sleep(max(0.0, min(0.01, arrive[nxt] - (time.perf_counter() - t0))))
        for c in srv.poll():
            done[tickets[c.ticket]] = c
    total = time.perf_counter() - t0
    busy, wall, lups = srv.stats()
    srv.close()
    lat = np.array([done[i].finish_ms - done[i].submit_ms for i in range(len(reqs))]) / 1e3
    # the plain FP64 GPU form on the same arrivals: one request at a time,
    # first come first served; each service time is a real solve on the GPU
    # (host geometry in, result out), the queueing follows from the arrivals
    free_at, lat64, fp64_res, fp64_objs = 0.0, [], [], []
    for i, (g, bc) in enumerate(reqs):
        s0 = time.perf_counter()
        with pm.Problem(g, None, boundary_method=bc, precision="fp64", order="jacobi",
                        **SERVE_KW) as p:
            r = p.solve()
        fp64_res.append({"iterations": r.iterations, "sweeps": r.sweeps,
                         "converged": bool(r.converged), "k": [r.wk13, r.wk23, r.wk33]})
        svc = time.perf_counter() - s0
        start = max(arrive[i], free_at)
        free_at = start + svc
        lat64.append(free_at - arrive[i])
        fp64_objs.append(r)
    rel, kerr = k_errors([(done[i].result, r) for i, r in enumerate(fp64_objs)])
    lat64 = np.array(lat64)
    unc_mx = unconverged([done[i].result for i in range(len(reqs))])
    unc_64 = unconverged(fp64_objs)
    span64 = free_at - arrive[0]
    out = {"metric": "p99 time-to-permeability", "value": float(np.percentile(lat, 99)),
           "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f32+f64",
           "data": "synthetic",
           "config": {"workload": f"{len(reqs)} requests, Poisson arrivals, axes log-uniform in "
                                  f"[32,{max_axis}], porosity U[0.12,0.45], bc 0/1/2, GS, "
                                  "eps 1e-6, mixed-precision server"},
           "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
           "converged_only": pcts(lat, unc_mx),
           "solves_per_h": 3600.0 * len(reqs) / total,
           "converged_solves_per_h": 3600.0 * (len(reqs) - len(unc_mx)) / total,
           "unconverged_at_max_iter": unc_mx,
           "device_busy_frac": (busy / 1e3) / total,
           "plain_fp64": {"p50_s": float(np.percentile(lat64, 50)),
                          "p99_s": float(np.percentile(lat64, 99)),
                          "converged_only": pcts(lat64, unc_64),
                          "solves_per_h": 3600.0 * len(reqs) / span64,
                          "converged_solves_per_h": 3600.0 * (len(reqs) - len(unc_64)) / span64,
                          "unconverged_at_max_iter": unc_64,
                          "service": "one request at a time, FIFO, same arrivals"},
           "k_rel_err_vs_plain_fp64": kerr,
           "failed": [{"index": i, "status": done[i].status} for i in range(len(reqs))
                      if done[i].status != 0]}
    order = sorted(range(len(rel)), key=lambda i: -rel[i])
    out["worst_samples"] = [
        {"index": i, "shape": list(reqs[i][0].shape), "boundary_method": reqs[i][1],
         "porosity": round(float(1 - reqs[i][0].mean()), 4), "rel_err": rel[i],
         "status": done[i].status,
         "mixed": {"iterations": done[i].result.iterations, "sweeps": done[i].result.sweeps,
                   "converged": bool(done[i].result.converged),
                   "k": [done[i].result.wk13, done[i].result.wk23, done[i].result.wk33]},
         "fp64": fp64_res[i]} for i in order[:4]]
    return out


def run_c5(args):
    import poremaps_gb300 as pm

    pm.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    print(json.dumps(c5_result(args.samples, args.max_axis, args.relaunch_sweeps)), flush=True)
    return 0


def run_c3(args):
    """One large sample: iid N(0,1) -> periodic Gaussian filter sigma 3 ->
    fluid = lowest 20 % -> largest z-percolating cluster; boundary_method 2,
    GS update (solving_algorithm 2); FP64 red-black, FP64 Jacobi and the mixed
    form timed over it_eval blocks, and the correction sweep's roofline with a
    working set far above L2."""
    import poremaps_gb300 as pm
    from poremaps_gb300 import synth

    local = int(os.environ.get("LOCAL_RANK", "0"))
    pm.set_device(local)
    n = args.size if args.size != 128 else 512
    t0 = time.perf_counter()
    g = synth.gaussian_field((n, n, n), 3.0, 0.20, seed=3)
    t_gen = time.perf_counter() - t0
    kw = dict(boundary_method=2, solving_algorithm=2, voxel_size=5e-6, eps=1e-6, it_eval=100,
              it_write=100)
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    forms = {}
    for name, extra in (("mixed", dict(precision="mixed", order="jacobi")),
                        ("fp64_jacobi", dict(precision="fp64", order="jacobi")),
                        ("fp64_redblack", dict(precision="fp64", order="redblack"))):
        with pm.Problem(g, None, **extra, **kw) as p:
            perm = 0.0
            for _ in range(max(1, args.warmup)):
                _, _, perm = p.block_timed(SWEEPS_PER_BLOCK, True, perm)
            ms = []
            for _ in range(max(2, args.steps // 2)):
                t, _, perm = p.block_timed(SWEEPS_PER_BLOCK, True, perm)
                ms.append(t)
            kms = p.kernel_time(0, 10)
            f = {"glups": g.size * SWEEPS_PER_BLOCK / (statistics.mean(ms) * 1e-3) / 1e9,
                 "ms_per_block": statistics.mean(ms), "sweep_kernel_ms": kms}
            if name == "mixed":
                f["kernel"] = p.kernel()
                f["brick"] = list(p.brick())
                f["roofline"] = {"bound": "hbm", "achieved": g.size * ALGO_BYTES_MIXED_INNER /
                                 (kms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s"}
                f["roofline"]["frac"] = f["roofline"]["achieved"] / peak
            else:
                f["hbm_frac_of_measured"] = g.size * ALGO_BYTES_FP64 / (kms * 1e-3) / 1e9 / peak
            forms[name] = f
    converged = None
    if args.converge:
        # every form to eps 1e-6 (calc_flow's stop rule), or on to
        # eps_fixed_point: iterations, device time and each permeability
        # component against the FP64 runs
        converged = {}
        for name, extra in (("mixed", dict(precision="mixed", order="jacobi")),
                            ("fp64_jacobi", dict(precision="fp64", order="jacobi")),
                            ("fp64_redblack", dict(precision="fp64", order="redblack"))):
            with pm.Problem(g, None, max_iter=args.max_iter,
                            eps_fixed_point=args.eps_fixed_point, **extra, **kw) as p:
                r = p.solve()
            converged[name] = {"iterations": r.iterations, "converged": bool(r.converged),
                               "conv": r.conv, "device_s": r.device_ms / 1e3,
                               "k_m2": [r.wk13, r.wk23, r.wk33]}
        # the FP64 oracle of the mixed form is the FP64 form in the same
        # (Jacobi) order; red-black is another trajectory, and two orders that
        # stop at different iterations differ by the drift the stop rule leaves
        def rel(a, b):
            return [abs(x - y) / abs(b[2]) for x, y in zip(a, b)]
        jac, rb = converged["fp64_jacobi"]["k_m2"], converged["fp64_redblack"]["k_m2"]
        converged["mixed"]["k_rel_err_vs_fp64_jacobi"] = rel(converged["mixed"]["k_m2"], jac)
        converged["mixed"]["k_rel_err_vs_fp64_redblack"] = rel(converged["mixed"]["k_m2"], rb)
        converged["fp64_jacobi"]["k_rel_err_vs_fp64_redblack"] = rel(jac, rb)
    out = {"metric": "GLUP/s", "value": forms["mixed"]["glups"], "unit": "GLUP/s", "n_gpus": 1,
           "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic",
           "config": {"workload": f"Gaussian field {n}^3 (sigma 3, porosity 0.20, largest "
                                  "z-percolating cluster), boundary_method 2, GS, it_eval blocks",
                      "porosity": float(1 - g.mean()), "generation_s": t_gen},
           "forms": forms}
    if converged is not None:
        key = ("to_eps_1e-6" if args.eps_fixed_point <= 0
               else f"to_eps_fixed_point_{args.eps_fixed_point:g}")
        out[key] = converged
    print(json.dumps(out), flush=True)
    return 0


def main():
    args = parse()
    if args.write_traffic:
        return write_traffic(args.write_traffic, args.kernel, args.brick, args.size)
    if args.write_fp64_record:
        return write_fp64_record(args.write_fp64_record, args.size)
    if args.profile_case:
        return run_profile_case(args)
    if args.workload == "c3":
        return run_c3(args)
    if args.workload == "c4":
        return run_c4(args)
    if args.workload == "c5":
        return run_c5(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
