"""ctypes front-end of the CPU ORACLE (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  It wraps ``oracle/_build/liboracle.so`` (the C
restatement in ``pm_oracle.c``) and, where present, runs the reference's own
sources built against the MPI shim (``oracle/_ref/poremaps_ref``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
CLI_PATH = os.path.join(HERE, "_build", "oracle_cli")
REF_BIN = os.path.join(HERE, "_ref", "poremaps_ref")

ORDER = {"reference": 0, "jacobi": 1, "redblack": 2}


class OrResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("sweeps", C.c_int), ("conv", C.c_double),
                ("permeability", C.c_double), ("k13", C.c_double), ("k23", C.c_double),
                ("k33", C.c_double), ("wk13", C.c_double), ("wk23", C.c_double),
                ("wk33", C.c_double), ("wmax_velz", C.c_double), ("wmean_velz", C.c_double),
                ("porosity", C.c_double)]


def build(quiet: bool = True) -> None:
    """Compile the oracle restatement (and the shimmed reference when its
    sources are available) with the committed Makefile."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "oracle"], check=True, stdout=out)
    subprocess.run(["make", "-C", HERE, "ref-if-present"], check=True, stdout=out)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_uint, C.c_int, C.c_void_p,
                                C.c_double, C.c_double, C.POINTER(C.c_int)]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_iterate.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.or_calc_flow.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_char_p, C.POINTER(OrResult)]
        L.or_convergence.restype = C.c_double
        L.or_convergence.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.or_permeability.argtypes = [C.c_void_p, C.POINTER(OrResult)]
        L.or_porosity.restype = C.c_double
        L.or_porosity.argtypes = [C.c_void_p]
        L.or_get_fields.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.or_get_nhood.argtypes = [C.c_void_p, C.c_void_p]
        L.or_get_padded.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)] + [C.c_void_p] * 4
        L.or_threads.argtypes = [C.c_void_p, C.c_int]
        L.or_set_fields.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.or_second_derivative.restype = C.c_double
        L.or_second_derivative.argtypes = [C.c_int] + [C.c_double] * 5
        L.or_split_code.argtypes = [C.c_int, C.POINTER(C.c_int)]
        _lib = L
    return _lib


@dataclass
class Fields:
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    p: np.ndarray


class OracleProblem:
    """One domain on the CPU oracle.  ``geom`` is a (nz, ny, nx) uint8 array
    (x fastest, 0 = fluid)."""

    def __init__(self, geom: np.ndarray, bc_method: int = 0, solver: int = 2,
                 voxel_size: float = 1e-5, porosity: float = -1.0,
                 dom_interest=(0, 0, 0, 0, 0, 0), nslabs: int = 1, threads: int = 1):
        g = np.ascontiguousarray(geom, dtype=np.uint8)
        self.shape = g.shape
        nz, ny, nx = g.shape
        size = (C.c_int * 3)(nx, ny, nz)
        di = (C.c_int * 6)(*dom_interest)
        self._g = g
        self.h = lib().or_create(size, bc_method, solver, nslabs, g.ctypes.data, voxel_size,
                                 porosity, di)
        if not self.h:
            raise ValueError("oracle: invalid decomposition")
        lib().or_threads(self.h, threads)

    def close(self):
        if self.h:
            lib().or_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def iterate(self, n: int, order: str = "reference") -> None:
        lib().or_iterate(self.h, ORDER[order], n)

    def calc_flow(self, max_iter: int, it_eval: int = 100, it_write: int = 100,
                  eps: float = 1e-6, order: str = "reference", log_path: str | None = None):
        r = OrResult()
        lib().or_calc_flow(self.h, ORDER[order], max_iter, it_eval, it_write, eps,
                           log_path.encode() if log_path else None, C.byref(r))
        return r

    def convergence(self, permeability: float):
        p = C.c_double(permeability)
        conv = lib().or_convergence(self.h, C.byref(p))
        return conv, p.value

    def permeability(self) -> OrResult:
        r = OrResult()
        lib().or_permeability(self.h, C.byref(r))
        return r

    def fields(self) -> Fields:
        arr = [np.empty(self.shape, np.float64) for _ in range(4)]
        lib().or_get_fields(self.h, *[a.ctypes.data for a in arr])
        return Fields(*arr)

    def set_fields(self, u=None, v=None, w=None, p=None) -> None:
        """Interior fields (z, y, x) set directly (test hook)."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (u, v, w, p)]
        lib().or_set_fields(self.h, *[None if a is None else a.ctypes.data for a in arrs])

    def nhood(self) -> np.ndarray:
        out = np.empty(self.shape, np.int32)
        lib().or_get_nhood(self.h, out.ctypes.data)
        return out

    def padded(self, slab: int = 0) -> Fields:
        nz, ny, nx = self.shape
        dims = (C.c_int * 3)()
        n = (nx + 4) * (ny + 4) * (nz + 4) * 2  # upper bound for any slab
        arr = [np.empty(n, np.float64) for _ in range(4)]
        lib().or_get_padded(self.h, slab, dims, *[a.ctypes.data for a in arr])
        NX, NY, NZ = dims[0], dims[1], dims[2]
        return Fields(*[a[:NX * NY * NZ].reshape(NZ, NY, NX) for a in arr])


def run_reference_binary(inp_path: str, cwd: str, nranks: int = 1, timeout: float = 600):
    """Run the reference's own program (built from its sources against the
    MPI shim) on an .inp file; returns the CompletedProcess."""
    env = dict(os.environ, PM_SHIM_NP=str(nranks))
    return subprocess.run([REF_BIN, inp_path], cwd=cwd, env=env, capture_output=True,
                          text=True, timeout=timeout)


def second_derivative(case: int, ll: float, l: float, m: float, r: float, rr: float) -> float:
    """get_2nd_derivation (solver.cc:57-91) of the restatement."""
    return lib().or_second_derivative(case, ll, l, m, r, rr)


def split_code(code: int):
    """split_number (solver.cc:94-109) of the restatement: (cx, cy, cz)."""
    out = (C.c_int * 3)()
    lib().or_split_code(code, out)
    return tuple(out)
