"""poremaps_gb300 -- GB300 (sm_103a) POREMAPS pseudo-time Stokes permeability solver.

Python front-end over the C ABI of ``include/poremaps.h`` (ctypes).  All
compute runs in the native library ``_build/libporemaps_gb300.so``; there is
no CPU fallback: importing this package without the built library raises.

Mirror of the reference program's interface (krachdd/poremaps):
  read_params      <- read_problem_params (src/read_problem_params.cc:50-156)
  Problem          <- the state set up in src/main_stokes_solver.cc:195-276
  Problem.solve    <- calc_flow (src/calc_flow.cc:53-169)
  Problem.iterate  <- one calc_flow iteration (central_diff5 + halo exchange + reapply)
  Problem.convergence / permeability <- src/evaluation.cc:54-262
  run_inp          <- the POREMAPS program (src/main_stokes_solver.cc:57-416)
  solve_tensor     <- the three axis-rotated runs of README.md:215-227
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libporemaps_gb300.so")
CLI_PATH = os.path.join(HERE, "_build", "poremaps_gpu")

ORDER_DEFAULT, ORDER_REFERENCE, ORDER_JACOBI, ORDER_REDBLACK = -1, 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
ARITH_EXACT, ARITH_FAST = 0, 1
ORDERS = {"default": -1, "reference": 0, "jacobi": 1, "redblack": 2}
PRECISIONS = {"fp64": 0, "mixed": 1}
ARITHS = {"exact": 0, "fast": 1}

STATUS = {0: "PM_OK", 1: "PM_ERR_INVALID", 2: "PM_ERR_IO", 3: "PM_ERR_CUDA", 4: "PM_ERR_NOMEM",
          5: "PM_ERR_NONFINITE", 6: "PM_ERR_BUSY", 7: "PM_ERR_NOT_FOUND", 8: "PM_ERR_CANCELLED"}
PM_ERR_NOMEM = 4
PM_ERR_NOT_FOUND = 7
PM_ERR_CANCELLED = 8


class PMError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("dom_decomposition", C.c_int * 3), ("boundary_method", C.c_int),
                ("geometry_file_name", C.c_char * 400), ("size", C.c_int * 3),
                ("voxel_size", C.c_double), ("max_iter", C.c_int), ("it_eval", C.c_int),
                ("it_write", C.c_int), ("log_file_name", C.c_char * 400),
                ("solving_algorithm", C.c_uint), ("eps", C.c_double), ("porosity", C.c_double),
                ("dom_interest", C.c_int * 6), ("write_output", C.c_int * 4),
                ("order", C.c_int), ("precision", C.c_int), ("arith", C.c_int),
                ("write_log", C.c_int), ("mixed_inner", C.c_int), ("kernel", C.c_int),
                ("brick", C.c_int * 3), ("eps_fixed_point", C.c_double)]


class Result(C.Structure):
    _fields_ = [("iterations", C.c_int), ("sweeps", C.c_int), ("converged", C.c_int),
                ("conv", C.c_double), ("permeability", C.c_double), ("k13", C.c_double),
                ("k23", C.c_double), ("k33", C.c_double), ("wk13", C.c_double),
                ("wk23", C.c_double), ("wk33", C.c_double), ("wmax_velz", C.c_double),
                ("wmean_velz", C.c_double), ("porosity", C.c_double), ("device_ms", C.c_double),
                ("wall_ms", C.c_double), ("glups", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_resident", C.c_int),
                ("precision", C.c_int), ("use_graphs", C.c_int), ("autotune", C.c_int),
                ("max_bypass", C.c_int), ("relaunch_sweeps", C.c_int)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int), ("result", Result),
                ("submit_ms", C.c_double), ("admit_ms", C.c_double), ("finish_ms", C.c_double)]


# Every symbol declared in include/poremaps.h (checked by the CPU tests).
EXPORTS = ["pm_last_error", "pm_last_error_copy", "pm_version", "pm_params_default", "pm_read_params",
           "pm_read_geometry", "pm_problem_create", "pm_problem_destroy", "pm_solve",
           "pm_iterate", "pm_compute_convergence", "pm_compute_permeability", "pm_get_porosity",
           "pm_get_iteration", "pm_get_fields", "pm_set_fields", "pm_resume_outputs",
           "pm_get_neighborhood", "pm_write_outputs",
           "pm_run_inp", "pm_solve_tensor", "pm_set_device", "pm_problem_reset",
           "pm_block_timed", "pm_block_group_timed", "pm_kernel_time", "pm_kernel_launches", "pm_get_kernel", "pm_get_brick", "pm_reduce_fields_noalloc",
           "pm_server_create", "pm_server_destroy",
           "pm_server_submit", "pm_server_step", "pm_server_poll", "pm_server_stats",
           "pm_server_clock_ms", "pm_server_cancel", "pm_debug_fail_alloc",
           "pm_problem_footprint", "pm_server_request_bytes", "pm_debug_round_wait",
           "pm_debug_tma_fail", "pm_server_launch_shape", "pm_server_set_launch_shape"]

_lib = None


def load_library(path: str = LIB_PATH):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"poremaps_gb300 native library missing: {path} "
                          "(run __graft_entry__.build() or python poremaps_gb300/build.py)")
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "pm_last_error": (C.c_char_p, []),
        "pm_last_error_copy": (C.c_size_t, [C.c_char_p, C.c_size_t]),
        "pm_version": (C.c_char_p, []),
        "pm_params_default": (C.c_int, [P(Params)]),
        "pm_read_params": (C.c_int, [C.c_char_p, P(Params)]),
        "pm_read_geometry": (C.c_int, [C.c_char_p, P(C.c_int), vp]),
        "pm_problem_create": (C.c_int, [P(Params), vp, P(vp)]),
        "pm_problem_destroy": (C.c_int, [vp]),
        "pm_solve": (C.c_int, [vp, P(Result)]),
        "pm_iterate": (C.c_int, [vp, C.c_int]),
        "pm_compute_convergence": (C.c_int, [vp, P(C.c_double), P(C.c_double)]),
        "pm_compute_permeability": (C.c_int, [vp, P(Result)]),
        "pm_get_porosity": (C.c_int, [vp, P(C.c_double)]),
        "pm_get_iteration": (C.c_int, [vp, P(C.c_int)]),
        "pm_get_fields": (C.c_int, [vp, vp, vp, vp, vp]),
        "pm_set_fields": (C.c_int, [vp, vp, vp, vp, vp, C.c_int]),
        "pm_resume_outputs": (C.c_int, [vp, C.c_int]),
        "pm_get_neighborhood": (C.c_int, [vp, vp]),
        "pm_write_outputs": (C.c_int, [vp]),
        "pm_run_inp": (C.c_int, [C.c_char_p, P(Params), P(Result)]),
        "pm_solve_tensor": (C.c_int, [P(Params), vp, P(C.c_double), P(Result)]),
        "pm_set_device": (C.c_int, [C.c_int]),
        "pm_problem_reset": (C.c_int, [vp]),
        "pm_block_timed": (C.c_int, [vp, C.c_int, C.c_int, P(C.c_double), P(C.c_double),
                                     P(C.c_double)]),
        "pm_block_group_timed": (C.c_int, [P(vp), C.c_int, C.c_int, C.c_int, P(C.c_double),
                                           P(C.c_double), P(C.c_double)]),
        "pm_kernel_time": (C.c_int, [vp, C.c_int, C.c_int, P(C.c_double)]),
        "pm_kernel_launches": (C.c_uint64, []),
        "pm_get_kernel": (C.c_int, [vp, P(C.c_int)]),
        "pm_get_brick": (C.c_int, [vp, P(C.c_int)]),
        "pm_reduce_fields_noalloc": (C.c_int, [P(C.c_int), vp, vp, vp, vp, vp, P(C.c_int), vp,
                                               vp]),
        "pm_server_create": (C.c_int, [P(ServerConfig), P(vp)]),
        "pm_server_destroy": (C.c_int, [vp]),
        "pm_server_submit": (C.c_int, [vp, P(Params), vp, P(C.c_uint64)]),
        "pm_server_step": (C.c_int, [vp, P(C.c_int)]),
        "pm_server_poll": (C.c_int, [vp, P(Completion), C.c_int, P(C.c_int)]),
        "pm_server_stats": (C.c_int, [vp, P(C.c_double), P(C.c_double), P(C.c_uint64)]),
        "pm_server_clock_ms": (C.c_double, [vp]),
        "pm_server_cancel": (C.c_int, [vp, C.c_uint64]),
        "pm_debug_fail_alloc": (C.c_int, [C.c_int]),
        "pm_debug_round_wait": (C.c_int, [C.c_uint, C.c_int]),
        "pm_debug_tma_fail": (C.c_int, [C.c_int]),
        "pm_problem_footprint": (C.c_int, [P(Params), P(C.c_size_t)]),
        "pm_server_request_bytes": (C.c_int, [vp, P(Params), P(C.c_size_t)]),
        "pm_server_launch_shape": (C.c_int, [vp, P(C.c_int)]),
        "pm_server_set_launch_shape": (C.c_int, [vp, P(C.c_int)]),
    }
    for name, (res, args) in sig.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _lib = L
    return L


def footprint(shape, **kw) -> int:
    """pm_problem_footprint: device bytes of a problem of this (nz, ny, nx)
    shape and these parameters."""
    nz, ny, nx = shape
    p = default_params(**kw)
    p.size[0], p.size[1], p.size[2] = nx, ny, nz
    b = C.c_size_t()
    _check(load_library().pm_problem_footprint(C.byref(p), C.byref(b)))
    return b.value


def debug_fail_alloc(nth: int) -> None:
    """pm_debug_fail_alloc: the nth device allocation of problem set-up from
    now on fails as out of memory (0 clears)."""
    _check(load_library().pm_debug_fail_alloc(int(nth)))


def debug_round_wait(extra: int, polls: int) -> None:
    """pm_debug_round_wait: the server's persistent sweep waits for `extra`
    items that never finish, with at most `polls` polls (0, 0 restores)."""
    _check(load_library().pm_debug_round_wait(int(extra), int(polls)))


def debug_tma_fail(on: bool) -> None:
    """pm_debug_tma_fail: z-march launches report a timed-out first wait."""
    _check(load_library().pm_debug_tma_fail(int(bool(on))))


def _check(st: int):
    if st != 0:
        raise PMError(st, load_library().pm_last_error().decode(errors="replace"))


def default_params(**kw) -> Params:
    p = Params()
    _check(load_library().pm_params_default(C.byref(p)))
    for k, v in kw.items():
        if k == "order" and isinstance(v, str):
            v = ORDERS[v]
        if k == "precision" and isinstance(v, str):
            v = PRECISIONS[v]
        if k == "arith" and isinstance(v, str):
            v = ARITHS[v]
        if k in ("geometry_file_name", "log_file_name"):
            v = v.encode() if isinstance(v, str) else v
        if k in ("size", "dom_interest", "write_output", "dom_decomposition", "brick"):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
            continue
        setattr(p, k, v)
    return p


def read_params(path: str) -> Params:
    p = Params()
    _check(load_library().pm_read_params(path.encode(), C.byref(p)))
    return p


class Problem:
    """One device-resident domain.  ``geom``: (nz, ny, nx) uint8 (x fastest,
    0 fluid, nonzero solid)."""

    def __init__(self, geom: np.ndarray, params: Params | None = None, **kw):
        g = np.ascontiguousarray(geom, dtype=np.uint8)
        nz, ny, nx = g.shape
        if params is None:
            params = default_params(**kw)
        else:
            params = Params.from_buffer_copy(params)
            for k, v in kw.items():
                setattr(params, k, ORDERS.get(v, v) if k == "order" and isinstance(v, str) else v)
        params.size[0], params.size[1], params.size[2] = nx, ny, nz
        self.params = params
        self.shape = g.shape
        self.h = C.c_void_p()
        _check(load_library().pm_problem_create(C.byref(params), g.ctypes.data, C.byref(self.h)))

    def close(self):
        if self.h:
            load_library().pm_problem_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def iterate(self, n: int) -> None:
        _check(load_library().pm_iterate(self.h, n))

    def solve(self) -> Result:
        r = Result()
        st = load_library().pm_solve(self.h, C.byref(r))
        if st not in (0, 5):
            _check(st)
        return r

    def convergence(self, permeability: float = 0.0):
        p = C.c_double(permeability)
        c = C.c_double()
        _check(load_library().pm_compute_convergence(self.h, C.byref(p), C.byref(c)))
        return c.value, p.value

    def permeability(self) -> Result:
        r = Result()
        _check(load_library().pm_compute_permeability(self.h, C.byref(r)))
        return r

    def porosity(self) -> float:
        v = C.c_double()
        _check(load_library().pm_get_porosity(self.h, C.byref(v)))
        return v.value

    def fields(self):
        arr = [np.empty(self.shape, np.float64) for _ in range(4)]
        _check(load_library().pm_get_fields(self.h, *[a.ctypes.data for a in arr]))
        return arr  # u, v, w, p

    @property
    def iteration(self) -> int:
        v = C.c_int()
        _check(load_library().pm_get_iteration(self.h, C.byref(v)))
        return v.value

    def set_fields(self, u, v, w, p, iteration: int = 0) -> None:
        """Restart from interior fields (lattice units, as fields() returns)."""
        arr = [np.ascontiguousarray(a, np.float64) for a in (u, v, w, p)]
        for a in arr:
            if a.shape != self.shape:
                raise ValueError(f"field shape {a.shape} != {self.shape}")
        _check(load_library().pm_set_fields(self.h, *[a.ctypes.data for a in arr], int(iteration)))

    def resume_outputs(self, iteration: int) -> None:
        """Restart from the field files write_outputs() left in the working directory."""
        _check(load_library().pm_resume_outputs(self.h, int(iteration)))

    def nhood(self) -> np.ndarray:
        out = np.empty(self.shape, np.int32)
        _check(load_library().pm_get_neighborhood(self.h, out.ctypes.data))
        return out

    def write_outputs(self) -> None:
        _check(load_library().pm_write_outputs(self.h))

    def reset(self) -> None:
        _check(load_library().pm_problem_reset(self.h))

    def block_timed(self, n: int, check: bool = True, permeability: float = 0.0):
        """n iterations (+ convergence check); returns (device_ms, conv, permeability)."""
        k = C.c_double(permeability)
        conv = C.c_double()
        ms = C.c_double()
        _check(load_library().pm_block_timed(self.h, n, int(check), C.byref(k), C.byref(conv),
                                             C.byref(ms)))
        return ms.value, conv.value, k.value

    def kernel(self) -> int:
        """Correction-sweep kernel in use (mixed form)."""
        k = C.c_int()
        _check(load_library().pm_get_kernel(self.h, C.byref(k)))
        return k.value

    def brick(self):
        """Brick order of the fluid list chosen for this problem."""
        b = (C.c_int * 3)()
        _check(load_library().pm_get_brick(self.h, b))
        return tuple(b)

    def kernel_time(self, kernel: int = 0, n: int = 20) -> float:
        v = C.c_double()
        _check(load_library().pm_kernel_time(self.h, kernel, n, C.byref(v)))
        return v.value


def set_device(device: int) -> None:
    _check(load_library().pm_set_device(device))


def block_group_timed(problems, n: int, check: bool = True, permeability=None):
    """One block of n iterations of every problem, concurrently on their
    streams; returns (device_ms, conv list, permeability list)."""
    m = len(problems)
    hs = (C.c_void_p * m)(*[p.h for p in problems])
    k = (C.c_double * m)(*(permeability or [0.0] * m))
    conv = (C.c_double * m)()
    ms = C.c_double()
    _check(load_library().pm_block_group_timed(hs, m, n, int(check), k, conv, C.byref(ms)))
    return ms.value, list(conv), list(k)


def kernel_launches() -> int:
    return int(load_library().pm_kernel_launches())


def run_inp(path: str, **overrides) -> Result:
    ov = default_params(**overrides)
    r = Result()
    st = load_library().pm_run_inp(path.encode(), C.byref(ov), C.byref(r))
    if st not in (0, 5):
        _check(st)
    return r


def solve_tensor(geom: np.ndarray, params: Params | None = None, **kw):
    """Full permeability tensor K (3x3, m^2; K[i, j] = response along axis i to
    the pressure drop along axis j) from three axis-rotated solves."""
    g = np.ascontiguousarray(geom, dtype=np.uint8)
    nz, ny, nx = g.shape
    p = default_params(**kw) if params is None else Params.from_buffer_copy(params)
    p.size[0], p.size[1], p.size[2] = nx, ny, nz
    K = (C.c_double * 9)()
    res = (Result * 3)()
    st = load_library().pm_solve_tensor(C.byref(p), g.ctypes.data, K, res)
    if st not in (0, 5):
        _check(st)
    return np.array(list(K)).reshape(3, 3), list(res)


class Server:
    """Batched / continuously batching solver (pm_server_* of the C ABI)."""

    def __init__(self, precision: str | int = "mixed", hbm_budget_bytes: int = 0,
                 max_resident: int = 0, use_graphs: int = 1, autotune: int = 0,
                 max_bypass: int = 0, relaunch_sweeps: int = 0):
        cfg = ServerConfig(hbm_budget_bytes, max_resident,
                           PRECISIONS.get(precision, precision), use_graphs, autotune,
                           max_bypass, relaunch_sweeps)
        self.h = C.c_void_p()
        _check(load_library().pm_server_create(C.byref(cfg), C.byref(self.h)))

    def submit(self, geom: np.ndarray, params: Params | None = None, **kw) -> int:
        g = np.ascontiguousarray(geom, dtype=np.uint8)
        nz, ny, nx = g.shape
        p = default_params(**kw) if params is None else Params.from_buffer_copy(params)
        p.size[0], p.size[1], p.size[2] = nx, ny, nz
        t = C.c_uint64()
        _check(load_library().pm_server_submit(self.h, C.byref(p), g.ctypes.data, C.byref(t)))
        return t.value

    def step(self) -> int:
        a = C.c_int()
        _check(load_library().pm_server_step(self.h, C.byref(a)))
        return a.value

    def poll(self, max_n: int = 256):
        buf = (Completion * max_n)()
        n = C.c_int()
        _check(load_library().pm_server_poll(self.h, buf, max_n, C.byref(n)))
        return [buf[i] for i in range(n.value)]

    def stats(self):
        b, w, l = C.c_double(), C.c_double(), C.c_uint64()
        _check(load_library().pm_server_stats(self.h, C.byref(b), C.byref(w), C.byref(l)))
        return b.value, w.value, l.value

    def clock_ms(self) -> float:
        return load_library().pm_server_clock_ms(self.h)

    def launch_shape(self) -> dict:
        """pm_server_launch_shape: the batched sweeps' current launch shape."""
        v = (C.c_int * 4)()
        _check(load_library().pm_server_launch_shape(self.h, v))
        return {"item_voxels": v[0], "round_ctas_per_sm": v[1], "round_threads": v[2],
                "threads": v[3]}

    def set_launch_shape(self, item_voxels: int, round_ctas_per_sm: int, round_threads: int,
                         threads: int) -> None:
        """pm_server_set_launch_shape: pin the launch shape (no autotuning)."""
        v = (C.c_int * 4)(item_voxels, round_ctas_per_sm, round_threads, threads)
        _check(load_library().pm_server_set_launch_shape(self.h, v))

    def request_bytes(self, geom: np.ndarray, **kw) -> int:
        """pm_server_request_bytes: the footprint this server admits the
        request by."""
        nz, ny, nx = geom.shape
        p = default_params(**kw)
        p.size[0], p.size[1], p.size[2] = nx, ny, nz
        b = C.c_size_t()
        _check(load_library().pm_server_request_bytes(self.h, C.byref(p), C.byref(b)))
        return b.value

    def cancel(self, ticket: int) -> int:
        """pm_server_cancel: returns the status (0, or PM_ERR_NOT_FOUND when the
        ticket has already completed)."""
        return load_library().pm_server_cancel(self.h, C.c_uint64(ticket))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def close(self):
        if self.h:
            load_library().pm_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
