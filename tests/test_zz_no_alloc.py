"""The allocation-free sums entry point (pm_reduce_fields_noalloc) against the
regular permeability entry point (pm_compute_permeability).

pm_reduce_fields_noalloc serves callers that cannot let the library allocate
device memory (HBM reserved up front by their own admission control, or a host
framework that owns every allocation); its only scratch is a fixed device
array of the library.  This test gives it device buffers it owns itself,
turns its nine sums into permeabilities with the reference's formulas
(evaluation.cc:192-210) and checks them against pm_compute_permeability on
the same state, within the 1e-12 relative tolerance of the GPU parity tests,
on two calls in a row (the shared scratch keeps the previous call's contents).
The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

import poremaps_gb300 as pm
from poremaps_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RE = 0.01


def k_from_sums(s, geom, di, phi, dx):
    fluid = geom == 0
    nz, ny, nx = geom.shape
    z, y, x = np.nonzero(fluid)
    box = (x >= di[0]) & (x <= di[1]) & (y >= di[2]) & (y <= di[3]) & (z >= di[4]) & (z <= di[5])
    wfl, fl = int(fluid.sum()), int(box.sum())
    p0f, pef = int((box & (z == di[4])).sum()), int((box & (z == di[5])).sum())
    pgrad = ((s[8] / pef) - (s[7] / p0f)) / (di[5] - di[4])
    return {
        "k13": (s[4] / fl) * (1.0 / RE) * phi * (1.0 / pgrad) * (dx * dx),
        "k23": (s[5] / fl) * (1.0 / RE) * phi * (1.0 / pgrad) * (dx * dx),
        "k33": (s[6] / fl) * (1.0 / RE) * phi * (1.0 / pgrad) * (dx * dx),
        "wk13": (s[0] / wfl) * (1.0 / RE) * phi * (dx * dx),
        "wk23": (s[1] / wfl) * (1.0 / RE) * phi * (dx * dx),
        "wk33": (s[2] / wfl) * (1.0 / RE) * phi * (dx * dx),
        "wmean_velz": s[2] / wfl * dx,
        "wmax_velz": s[3] * dx,
    }


def test_noalloc_sums_match_permeability_entry_point():
    geom = synth.random_solid((24, 20, 16), 0.25, 17)
    nz, ny, nx = geom.shape
    di = (2, 12, 3, 15, 4, nz - 1)  # zmax on the last interior plane (pressure 3)
    dx = 1e-5
    with pm.Problem(geom, None, boundary_method=0, solving_algorithm=2, voxel_size=dx,
                    dom_interest=di, order="jacobi") as pr:
        pr.iterate(300)
        ref = pr.permeability()
        u, v, w, p = pr.fields()
        phi = pr.porosity()
    dev = torch.device("cuda", 0)
    g_d = torch.from_numpy(geom.copy()).to(dev)
    f_d = [torch.from_numpy(a.copy()).to(dev) for a in (u, v, w, p)]
    sums = torch.empty(9, dtype=torch.float64, device=dev)
    size = (C.c_int * 3)(nx, ny, nz)
    dia = (C.c_int * 6)(*di)
    lib = pm.load_library()
    for call in range(2):
        sums.fill_(float("nan"))
        torch.cuda.synchronize()
        st = lib.pm_reduce_fields_noalloc(size, g_d.data_ptr(), *[t.data_ptr() for t in f_d], dia,
                                          sums.data_ptr(), None)
        assert st == 0, lib.pm_last_error()
        torch.cuda.synchronize()
        k = k_from_sums(sums.cpu().numpy(), geom, di, phi, dx)
        for name, val in k.items():
            want = getattr(ref, name)
            assert abs(val - want) <= 1e-12 * max(abs(want), 1e-300), (call, name, val, want)


def test_noalloc_rejects_sizes_beyond_the_scratch():
    lib = pm.load_library()
    size = (C.c_int * 3)(8, 200, 100)  # 20000 rows > 16384
    dummy = C.c_void_p(16)
    st = lib.pm_reduce_fields_noalloc(size, dummy, dummy, dummy, dummy, dummy, None, dummy, None)
    assert st == 1 and b"scratch" in lib.pm_last_error()


def test_noalloc_without_box_on_a_caller_stream():
    """dom_interest NULL: the box sums are 0 and the whole-domain sums still
    match pm_compute_permeability; the launch goes on a stream the caller
    owns, which the caller synchronises before reading the sums."""
    geom = synth.random_solid((18, 14, 22), 0.3, 29)
    nz, ny, nx = geom.shape
    dx = 2e-5
    with pm.Problem(geom, None, boundary_method=1, solving_algorithm=3, voxel_size=dx,
                    order="redblack") as pr:
        pr.iterate(250)
        ref = pr.permeability()
        u, v, w, p = pr.fields()
        phi = pr.porosity()
    dev = torch.device("cuda", 0)
    g_d = torch.from_numpy(geom.copy()).to(dev)
    f_d = [torch.from_numpy(a.copy()).to(dev) for a in (u, v, w, p)]
    sums = torch.empty(9, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream()
    size = (C.c_int * 3)(nx, ny, nz)
    lib = pm.load_library()
    for call in range(2):
        sums.fill_(float("nan"))
        torch.cuda.synchronize()
        st = lib.pm_reduce_fields_noalloc(size, g_d.data_ptr(), *[t.data_ptr() for t in f_d],
                                          None, sums.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.pm_last_error()
        stream.synchronize()
        s = sums.cpu().numpy()
        assert np.all(s[4:9] == 0.0), (call, s[4:9])
        wfl = int((geom == 0).sum())
        for name, val in (("wk13", s[0] / wfl / RE * phi * dx * dx),
                          ("wk23", s[1] / wfl / RE * phi * dx * dx),
                          ("wk33", s[2] / wfl / RE * phi * dx * dx),
                          ("wmax_velz", s[3] * dx)):
            want = getattr(ref, name)
            assert abs(val - want) <= 1e-12 * max(abs(want), 1e-300), (call, name, val, want)
