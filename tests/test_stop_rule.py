"""The stop rule of the solve loop and the server (pm_api_internal.h), on the
host: calc_flow's `conv < eps` (calc_flow.cc:92-168) and the eps_fixed_point
extension (threshold, or stagnation at the rounding floor of conv), replayed
on synthetic convergence traces through the library's own inline functions."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path_factory.mktemp("stop") / "stop_rule_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", CUDA_INC,
                    os.path.join(HERE, "stop_rule_check.cpp"), "-o", exe], check=True)
    return exe


def run(exe, eps, efp, trace):
    text = "".join("nan\n" if math.isnan(c) else f"{c:.17g}\n" for c in trace)
    out = subprocess.run([exe, repr(eps), repr(efp)], input=text, capture_output=True, text=True,
                         check=True).stdout.split()
    if out == ["none"]:
        return None
    return int(out[1]), bool(int(out[3]))


def geometric(start, factor, n):
    return [start * factor ** i for i in range(n)]


def test_reference_rule(checker):
    assert run(checker, 1e-6, 0.0, [1e-3, 1e-5, 2e-6, 5e-7, 1e-8]) == (3, True)
    assert run(checker, 1e-6, 0.0, [1e-3, float("nan"), 1e-9]) == (1, False)
    assert run(checker, 1e-6, 0.0, [1e-3] * 50) is None
    # the reference rule ignores stagnation entirely
    assert run(checker, 1e-6, 0.0, [1e-3] * 5 + [2e-6] * 100) is None


def test_fixed_point_threshold(checker):
    trace = geometric(1e-3, 0.8, 200)
    k = next(i for i, c in enumerate(trace) if c < 1e-12)
    assert run(checker, 1e-6, 1e-12, trace) == (k, True)
    # eps alone would have stopped far earlier
    assert run(checker, 1e-6, 0.0, trace)[0] < k


def test_no_stop_while_conv_wanders_above_the_floor(checker):
    """A medium whose conv wanders around 1e-7 for thousands of evaluations
    (weakly damped pressure waves) is not at its fixed point: no stop."""
    rng = np.random.default_rng(1)
    trace = geometric(1e-3, 0.9, 90) + list(1e-7 * (1 + 2 * rng.random(3000)))
    assert min(trace) < 1e-6
    assert run(checker, 1e-6, 1e-30, trace) is None


def test_stagnation_at_the_rounding_floor(checker):
    rng = np.random.default_rng(2)
    decay = geometric(1e-3, 0.7, 90)
    floor_at = next(i for i, c in enumerate(decay) if c < 1e-13)
    trace = decay[:floor_at] + list(1e-16 * (1 + 9 * rng.random(2000)))
    stop, conv = run(checker, 1e-6, 1e-30, trace)
    assert conv and floor_at <= stop < floor_at + 200


def test_a_dip_does_not_stop_the_run(checker):
    """One evaluation where the change of k passes through zero lowers no
    window maximum: the run goes on to the floor."""
    rng = np.random.default_rng(3)
    trace = geometric(1e-3, 0.7, 90)
    trace[40] = 1e-25
    floor_at = next(i for i, c in enumerate(trace) if c < 1e-13 and i != 40)
    trace = trace[:floor_at] + list(1e-16 * (1 + 9 * rng.random(2000)))
    stop, conv = run(checker, 1e-6, 1e-30, trace)
    assert conv and stop >= floor_at


def test_nan_stops_unconverged_with_fixed_point(checker):
    assert run(checker, 1e-6, 1e-30, [1e-3, 1e-4, float("nan")]) == (2, False)
