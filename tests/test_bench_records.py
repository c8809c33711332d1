"""bench.py's measured records (CPU): a traffic or FP64-pipe record is used
only for the kernel id, list order and kernel sources it was captured with;
any other kernel or a changed source gives no figure and says why."""
import importlib
import json
import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture()
def bench_copy(tmp_path, monkeypatch):
    """bench.py pointed at a copy of the kernel sources with a fresh record."""
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    for f in set(bench.KERNEL_SOURCES) | set(bench.FP64_SOURCES):
        dst = tmp_path / f
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy(os.path.join(ROOT, f), dst)
    (tmp_path / "profiles").mkdir()
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    rec = {"kernel": "k_dc_inner_c", "kernel_id": 9, "brick": [0, 0, 0], "nvox": 1000,
           "dram_bytes_per_launch": 5000.0, "sources": bench.KERNEL_SOURCES,
           "sources_sha256": bench._sources_sha(bench.KERNEL_SOURCES), "source": "test"}
    (tmp_path / "profiles" / "k_dc_inner_c_sphere10_traffic.json").write_text(json.dumps(rec))
    fp = {"fp64_pipe_active_pct": 80.0, "fp64_warp_instructions": 1e6, "duration_us": 50.0,
          "sources": bench.FP64_SOURCES, "sources_sha256": bench._sources_sha(bench.FP64_SOURCES),
          "source": "test"}
    (tmp_path / "profiles" / "k_sweep64_pf_sphere10_fp64pipe.json").write_text(json.dumps(fp))
    return bench, tmp_path


def test_traffic_record_used_for_its_kernel(bench_copy):
    bench, _ = bench_copy
    t, why = bench.kernel_traffic(9, [0, 0, 0], 10, 2000)
    assert t == 10000.0 and why == "test"  # scaled by the voxels of the run


def test_traffic_record_refused_for_another_kernel_or_order(bench_copy):
    bench, _ = bench_copy
    t, why = bench.kernel_traffic(8, [0, 0, 0], 10, 1000)
    assert t is None and "kernel 9" in why
    t, why = bench.kernel_traffic(9, [32, 8, 8], 10, 1000)
    assert t is None and "brick" in why


def test_traffic_record_refused_after_a_source_change(bench_copy):
    bench, root = bench_copy
    f = root / bench.KERNEL_SOURCES[0]
    f.write_text(f.read_text() + "\n// changed\n")
    t, why = bench.kernel_traffic(9, [0, 0, 0], 10, 1000)
    assert t is None and "changed" in why


def test_fp64_pipe_record(bench_copy):
    bench, root = bench_copy
    r = bench.fp64_pipe_record(10, 0.1)  # warm 100 us against 50 us cold
    assert r["active_pct_ncu_cold"] == 80.0 and abs(r["active_frac_at_event_time"] - 0.4) < 1e-12
    f = root / bench.FP64_SOURCES[0]
    f.write_text(f.read_text() + "\n// changed\n")
    assert "stale" in bench.fp64_pipe_record(10, 0.1)


def test_c4_cpu_estimate_extrapolates_measured_rates():
    """The c4 leg's CPU figure: the oracle restatement's reference-order
    sweeps on a subsample, one process per sample, extrapolated to the whole
    stream by voxels x iterations at the measured per-core rate."""
    import numpy as np
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    from poremaps_gb300 import synth
    reqs = [(synth.random_solid((10, 12, 14), 0.3, s), s % 2) for s in range(4)]
    iters = [1000, 2000, 1500, 3000]
    est = bench.c4_cpu_estimate(reqs, iters, cores=2, sweeps=20)
    assert est["cores"] == 2 and est["kind"] == "port" and est["mlups_per_core"] > 0
    rate = est["mlups_per_core"] * 1e6
    core_s = sum(g.size * it for (g, _), it in zip(reqs, iters)) / rate
    assert np.isclose(est["solves_per_h"], 3600.0 * len(reqs) / (core_s / 2))
    assert "2 of the 4 samples" in est["sample"]
