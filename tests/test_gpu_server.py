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
               submit_later=()):
    kw = dict(KW, **(kw or {}))
    s = pm.Server(precision=precision, use_graphs=use_graphs, autotune=autotune,
                  hbm_budget_bytes=budget)
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


def footprint(shape):
    """Device bytes of one mixed-precision request (mirrors the library's layout)."""
    nz, ny, nx = shape
    NX, NY, NZ = nx + 4, ny + 4, nz + 4
    up = lambda a, b: (a + b - 1) // b * b  # noqa: E731
    a64 = up(14 + NX, 16) * NY * NZ + 64
    a4 = up(6 + NX, 8) * NY * NZ + 16
    ac = up(14 + NX, 16) * NY * NZ + 256
    n = nx * ny * nz
    return ac + 4 * n + 64 * a64 + 48 * a4 + 8 * n + (1 << 20)


def test_budget_limits_resident_set_and_all_finish():
    geoms = samples(6, seed=4)
    budget = int(2.5 * max(footprint(g.shape) for g in geoms))
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
