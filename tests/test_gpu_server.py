"""The batched / continuously batching server (pm_server_*) on the GPU.

* each request's result equals the single-problem path (same kernels, same
  correction schedule) and is bitwise identical alone and in the mix;
* CUDA-graph capture and the autotuner change nothing in the results;
* admission respects the HBM budget, requests submitted while others run are
  admitted as memory frees up, finished ones retire without stalling others.
"""
import numpy as np
import pytest

import poremaps_gb300 as pm
from poremaps_gb300 import synth

pytestmark = pytest.mark.gpu

KW = dict(boundary_method=0, solving_algorithm=2, voxel_size=1e-5, eps=1e-6, it_eval=100,
          it_write=100, max_iter=60000)


def samples(n=6, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        shape = tuple(int(v) for v in rng.choice([12, 16, 20, 24], 3))
        if i % 2 == 0:
            g = synth.sphere_pack(shape, rmin=1.5, rmax=3.0, solid_fraction=0.55, seed=seed + i)
        else:
            g = synth.gaussian_field(shape, 1.5, 0.4, seed=seed + i)
        out.append(g)
    return out


def run_server(geoms, precision="mixed", use_graphs=1, autotune=0, budget=0, kw=None,
               submit_later=(), relaunch_sweeps=0, shape=None, shapes_seen=None):
    kw = dict(KW, **(kw or {}))
    s = pm.Server(precision=precision, use_graphs=use_graphs, autotune=autotune,
                  hbm_budget_bytes=budget, relaunch_sweeps=relaunch_sweeps)
    if shape is not None:
        s.set_launch_shape(*shape)
    tickets = {}
    for i, g in enumerate(geoms):
        if i not in submit_later:
            tickets[s.submit(g, **kw)] = i
    steps = 0
    results = {}
    max_resident = 0
    while True:
        active = s.step()
        steps += 1
        if steps == 3:
            for i in submit_later:
                tickets[s.submit(geoms[i], **kw)] = i
            active = 1
        for c in s.poll():
            results[tickets[c.ticket]] = c
        if shapes_seen is not None:
            shapes_seen.append(s.launch_shape())
        if active == 0 and len(results) == len(geoms):
            break
        assert steps < 5000
    s.close()
    return results


def single(g, precision="mixed", kw=None):
    kw = dict(KW, **(kw or {}))
    with pm.Problem(g, None, order="jacobi", precision=precision, **kw) as p:
        return p.solve()


def test_server_matches_single_problem():
    geoms = samples(6, seed=1)
    res = run_server(geoms)
    for i, g in enumerate(geoms):
        c = res[i]
        assert c.status == 0
        r = single(g)
        assert c.result.converged and r.converged
        assert c.result.iterations == r.iterations and c.result.sweeps == r.sweeps
        for a in ("wk13", "wk23", "wk33", "wmax_velz", "wmean_velz"):
            assert getattr(c.result, a) == getattr(r, a), (i, a)


def test_alone_and_in_the_mix_identical():
    geoms = samples(5, seed=2)
    mix = run_server(geoms)
    for i, g in enumerate(geoms[:3]):
        alone = run_server([g])[0]
        for a in ("iterations", "sweeps", "wk13", "wk23", "wk33", "conv"):
            assert getattr(alone.result, a) == getattr(mix[i].result, a), (i, a)


def test_graphs_and_autotune_do_not_change_results():
    geoms = samples(4, seed=3)
    base = run_server(geoms, use_graphs=0, autotune=0)
    for cfg in (dict(use_graphs=1, autotune=0), dict(use_graphs=1, autotune=1)):
        other = run_server(geoms, **cfg)
        for i in range(len(geoms)):
            assert other[i].result.iterations == base[i].result.iterations
            assert other[i].result.wk33 == base[i].result.wk33


def footprint(g):
    """Device bytes the server admits one request of this geometry by."""
    with pm.Server(precision="mixed") as s:
        return s.request_bytes(g, **KW)


def test_budget_limits_resident_set_and_all_finish():
    geoms = samples(6, seed=4)
    budget = int(2.5 * max(footprint(g) for g in geoms))
    res = run_server(geoms, budget=budget)
    assert len(res) == len(geoms) and all(c.status == 0 for c in res.values())
    # some request had to wait for an earlier one to retire
    admits = sorted((c.admit_ms, c.finish_ms) for c in res.values())
    assert any(a > min(f for _, f in admits) for a, _ in admits)


def test_requests_arriving_while_others_run():
    geoms = samples(5, seed=5)
    res = run_server(geoms, submit_later=(3, 4))
    for i, g in enumerate(geoms):
        assert res[i].status == 0
        assert res[i].result.wk33 == single(g).wk33


def test_server_fp64_form():
    geoms = samples(3, seed=6)
    res = run_server(geoms, precision="fp64")
    for i, g in enumerate(geoms):
        r = single(g, precision="fp64")
        assert res[i].result.iterations == r.iterations
        assert res[i].result.wk33 == r.wk33


def test_mixed_server_k_within_1e6_of_fp64():
    geoms = samples(3, seed=7)
    kw = dict(eps=1e-9)
    mx = run_server(geoms, kw=kw)
    for i, g in enumerate(geoms):
        r64 = single(g, precision="fp64", kw=kw)
        for a in ("wk13", "wk23", "wk33"):
            assert abs(getattr(mx[i].result, a) - getattr(r64, a)) <= 1e-6 * abs(r64.wk33)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_iteration_cap_matches_single_problem(precision):
    """Requests that stop on max_iter (eps too small to be met) run iterations
    0 .. max_iter-1 as calc_flow does -- also when max_iter is not a block
    boundary, or is shorter than one block -- and give the single-problem
    result bit for bit."""
    geoms = samples(3, seed=8)
    caps = [1550, 250, 1301]
    s = pm.Server(precision=precision, use_graphs=1, autotune=0)
    tickets = {}
    for i, (g, cap) in enumerate(zip(geoms, caps)):
        tickets[s.submit(g, **dict(KW, eps=1e-30, max_iter=cap))] = i
    res = {}
    for _ in range(1000):
        active = s.step()
        for c in s.poll():
            res[tickets[c.ticket]] = c
        if active == 0 and len(res) == len(geoms):
            break
    s.close()
    assert len(res) == len(geoms)
    for i, (g, cap) in enumerate(zip(geoms, caps)):
        r = single(g, precision=precision, kw=dict(eps=1e-30, max_iter=cap))
        c = res[i]
        assert c.status == 0 and not c.result.converged and not r.converged
        assert c.result.sweeps == r.sweeps == cap
        assert c.result.iterations == r.iterations
        for a in ("wk13", "wk23", "wk33", "wmax_velz", "wmean_velz"):
            assert getattr(c.result, a) == getattr(r, a), (i, a)


def test_mixed_solvers_in_one_batch():
    """Requests with different update formulas (GS and SOR) share the batched
    launches through the generic kernels; each result equals its
    single-problem run bit for bit."""
    geoms = samples(4, seed=9)
    solvers = [2, 3, 3, 2]
    s = pm.Server(precision="mixed", use_graphs=1, autotune=0)
    tickets = {}
    for i, (g, sv) in enumerate(zip(geoms, solvers)):
        tickets[s.submit(g, **dict(KW, solving_algorithm=sv))] = i
    res = {}
    for _ in range(5000):
        active = s.step()
        for c in s.poll():
            res[tickets[c.ticket]] = c
        if active == 0 and len(res) == len(geoms):
            break
    s.close()
    assert len(res) == len(geoms)
    for i, (g, sv) in enumerate(zip(geoms, solvers)):
        r = single(g, kw=dict(solving_algorithm=sv))
        c = res[i]
        assert c.status == 0 and c.result.iterations == r.iterations
        for a in ("wk13", "wk23", "wk33"):
            assert getattr(c.result, a) == getattr(r, a), (i, a)


def test_server_eps_fixed_point_matches_single_problem():
    """The fixed-point stop rule in the server.  A threshold well above the
    rounding floor of conv stops at the same iteration as pm_solve.  Below the
    floor the run ends by stagnation, and where exactly depends on conv's last
    bits, which the server sums in another order (per-item partials) than
    pm_solve: both stop within a few windows of evaluations of each other, on
    the same fixed point."""
    geoms = samples(3, seed=4)
    kw = dict(eps_fixed_point=1e-11, max_iter=200000)
    res = run_server(geoms, kw=kw)
    for i, g in enumerate(geoms):
        c, r = res[i], single(g, kw=kw)
        assert c.status == 0 and c.result.converged and r.converged
        assert c.result.iterations == r.iterations and c.result.sweeps == r.sweeps
        assert c.result.wk33 == r.wk33 and c.result.conv < 1e-11
    kw = dict(eps_fixed_point=1e-30, max_iter=200000)
    res = run_server(geoms, kw=kw)
    for i, g in enumerate(geoms):
        c, r = res[i], single(g, kw=kw)
        assert c.status == 0 and c.result.converged and r.converged
        assert c.result.iterations < 100000 and abs(c.result.iterations - r.iterations) <= 5000
        assert abs(c.result.wk33 - r.wk33) <= 1e-12 * abs(r.wk33)


def drain(s, tickets, limit=5000):
    out, steps = {}, 0
    while len(out) < len(tickets):
        s.step()
        steps += 1
        for c in s.poll():
            out[tickets[c.ticket]] = c
        assert steps < limit
    return out


def test_request_larger_than_budget_fails_with_nomem():
    """A request whose footprint exceeds the whole budget completes at once
    with PM_ERR_NOMEM while a resident request keeps running; a small one
    behind it still completes."""
    big = synth.sphere_pack((64, 64, 64), rmin=2.0, rmax=4.0, solid_fraction=0.55, seed=3)
    small = samples(2, seed=4)
    budget = footprint(small[0]) + footprint(small[1]) + 4096
    assert footprint(big) > budget
    s = pm.Server(precision="mixed", hbm_budget_bytes=budget)
    tickets = {s.submit(small[0], **KW): "a"}
    s.step()  # "a" resident
    tickets[s.submit(big, **KW)] = "big"
    tickets[s.submit(small[1], **KW)] = "b"
    res = drain(s, tickets)
    s.close()
    assert res["big"].status == pm.PM_ERR_NOMEM
    assert res["a"].status == 0 and res["b"].status == 0
    r = single(small[1])
    assert res["b"].result.wk33 == r.wk33 and res["b"].result.iterations == r.iterations


def _backfill_case(max_bypass):
    a = synth.sphere_pack((32, 32, 32), rmin=1.5, rmax=3.0, solid_fraction=0.55, seed=21)
    b = synth.sphere_pack((28, 28, 30), rmin=1.5, rmax=3.0, solid_fraction=0.55, seed=22)
    c1 = synth.sphere_pack((12, 12, 12), rmin=1.5, rmax=3.0, solid_fraction=0.55, seed=23)
    c2 = synth.sphere_pack((12, 14, 12), rmin=1.5, rmax=3.0, solid_fraction=0.55, seed=24)
    budget = footprint(a) + footprint(c1) + footprint(c2) + 4096
    assert footprint(b) < footprint(a) and footprint(a) + footprint(b) > budget
    s = pm.Server(precision="mixed", hbm_budget_bytes=budget, max_bypass=max_bypass)
    tickets = {}
    for name, g in (("a", a), ("b", b), ("c1", c1), ("c2", c2)):
        tickets[s.submit(g, **KW)] = name
    res = drain(s, tickets)
    s.close()
    assert all(c.status == 0 for c in res.values())
    for name, g in (("b", b), ("c1", c1)):
        assert res[name].result.wk33 == single(g).wk33
    return {k: c.admit_ms for k, c in res.items()}


def test_backfill_admits_past_a_head_that_does_not_fit():
    """a is resident, b does not fit beside it: c1 and c2 behind b fit and are
    admitted before b (default backfill)."""
    t = _backfill_case(0)
    assert t["c1"] < t["b"] and t["c2"] < t["b"]


def test_backfill_bypass_limit_and_strict_fifo():
    """With max_bypass 1 only c1 passes b; with backfill off (-1) neither does."""
    t = _backfill_case(1)
    assert t["c1"] < t["b"] <= t["c2"]
    t = _backfill_case(-1)
    assert t["b"] <= t["c1"] and t["b"] <= t["c2"]


def test_cancel_queued_and_resident():
    """Cancelling a resident and a queued request frees them; the others
    finish with the results they have alone."""
    geoms = samples(4, seed=6)
    s = pm.Server(precision="mixed", max_resident=2)
    tickets = {s.submit(g, **KW): i for i, g in enumerate(geoms)}
    inv = {i: t for t, i in tickets.items()}
    s.step()  # 0 and 1 resident, 2 and 3 queued
    assert s.cancel(inv[0]) == 0
    assert s.cancel(inv[3]) == 0
    assert s.cancel(10**9) == pm.PM_ERR_NOT_FOUND
    res = drain(s, tickets)
    assert s.cancel(inv[1]) == pm.PM_ERR_NOT_FOUND  # already completed
    s.close()
    assert res[0].status == pm.PM_ERR_CANCELLED and res[3].status == pm.PM_ERR_CANCELLED
    for i in (1, 2):
        r = single(geoms[i])
        assert res[i].status == 0 and res[i].result.wk33 == r.wk33
        assert res[i].result.iterations == r.iterations


def test_allocation_failure_is_reported_and_recovered():
    """A failed device allocation during set-up (injected on the host) gives
    PM_ERR_NOMEM from pm_problem_create and in the server's completion;
    nothing leaks and the next requests run normally."""
    g = samples(2, seed=8)
    # a mixed problem makes two or three device allocations: its fixed
    # buffers, then the correction store(s)
    for nth in (1, 2):
        pm.debug_fail_alloc(nth)
        with pytest.raises(RuntimeError, match="PM_ERR_NOMEM"):
            pm.Problem(g[0], None, precision="mixed", order="jacobi", **KW)
    pm.debug_fail_alloc(0)
    ref = single(g[1])
    s = pm.Server(precision="mixed")
    pm.debug_fail_alloc(2)
    tickets = {s.submit(x, **KW): i for i, x in enumerate(g)}
    res = drain(s, tickets)
    pm.debug_fail_alloc(0)
    s.close()
    assert res[0].status == pm.PM_ERR_NOMEM
    assert res[1].status == 0 and res[1].result.wk33 == ref.wk33


@pytest.mark.parametrize("use_graphs", [1, 0])
def test_persistent_round_equals_one_launch_per_sweep(use_graphs):
    """The round's FP32 sweeps as one persistent kernel walking the tile
    queue give the same fields as one launch per sweep, bit for bit, with
    samples of very different sizes resident together."""
    geoms = samples(5, seed=12) + [synth.sphere_pack((40, 36, 44), rmin=1.5, rmax=3.0,
                                                     solid_fraction=0.55, seed=13)]
    a = run_server(geoms, use_graphs=use_graphs, relaunch_sweeps=0)
    b = run_server(geoms, use_graphs=use_graphs, relaunch_sweeps=1)
    for i in range(len(geoms)):
        assert a[i].status == 0 and b[i].status == 0
        assert a[i].result.iterations == b[i].result.iterations
        for f in ("wk13", "wk23", "wk33", "wmax_velz"):
            assert getattr(a[i].result, f) == getattr(b[i].result, f), (i, f)


def test_round_wait_that_runs_out_reports_an_error():
    """A wait of the persistent sweep kernel that can never be satisfied
    (test hook) runs out after its poll limit: the kernel sets its error flag
    and returns, pm_server_step reports PM_ERR_CUDA, and the device stays
    usable -- a new server then solves the same samples normally."""
    geoms = samples(2, seed=14)
    pm.debug_round_wait(1 << 20, 2048)
    try:
        s = pm.Server(precision="mixed")
        for g in geoms:
            s.submit(g, **KW)
        with pytest.raises(pm.PMError) as ei:
            for _ in range(5):
                s.step()
        assert ei.value.status == 3 and "timed out" in str(ei.value)
        s.close()
    finally:
        pm.debug_round_wait(0, 0)
    res = run_server(geoms)
    for i, g in enumerate(geoms):
        assert res[i].status == 0 and res[i].result.wk33 == single(g).wk33


def test_launch_shapes_give_identical_results():
    """The persistent round at 256 threads x 4 CTAs per SM and at 128 threads
    x 8, with different work-item sizes and block sizes of the other batched
    kernels, and the autotuned shape: the same results bit for bit.  Every
    shape the autotuner picks is one of its candidates."""
    geoms = samples(5, seed=7)
    outs = []
    for shape in ((8192, 4, 256, 256), (512, 8, 128, 128), (2048, 3, 128, 512)):
        seen = []
        outs.append(run_server(geoms, shape=shape, shapes_seen=seen))
        assert all(tuple(d.values()) == shape for d in seen)
    seen = []
    outs.append(run_server(geoms, autotune=1, shapes_seen=seen))
    for d in seen:
        assert d["item_voxels"] in (2048, 8192, 32768) and d["threads"] == 256
        assert (d["round_threads"], d["round_ctas_per_sm"]) in (
            (256, 2), (256, 3), (256, 4), (128, 4), (128, 6), (128, 8))
    for other in outs[1:]:
        for i in range(len(geoms)):
            a, b = outs[0][i].result, other[i].result
            assert a.iterations == b.iterations
            for f in ("wk13", "wk23", "wk33", "wmax_velz", "wmean_velz"):
                assert getattr(a, f) == getattr(b, f), (i, f)


def test_launch_shape_rejects_invalid_shapes():
    s = pm.Server(precision="mixed")
    for bad in ((0, 4, 256, 256), (8192, 5, 256, 256), (8192, 9, 128, 256),
                (8192, 4, 192, 256), (8192, 4, 256, 96)):
        with pytest.raises(pm.PMError):
            s.set_launch_shape(*bad)
    s.close()
