"""tcstencil_gb300 — GB300 (sm_103a) engine for TCStencil's 2-D Jacobi sweeps.

Python mirror of the C-ABI in include/tcs.h (ctypes over the in-tree
libtcs.so).  The reference's interface is kept: `host_code(h_A, h_B, h_C, N, n)`
per stencil (layout16/host_*.cu, baseline/host_*.cu), with the same argument
meaning; the extended interface adds non-square grids, update rectangles,
multi-step plans, split precision and device-resident state.

There is no CPU fallback: if the native library is missing, every entry point
raises.  Build it with `tcstencil_gb300.build.build()`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

__all__ = [
    "STENCILS", "ENGINES", "PRECISIONS", "RADIUS", "TcsError", "lib", "host_code",
    "host_star2d1r", "host_star2d2r", "host_box2d1r", "host_box2d2r", "host_cc_star2d1r",
    "host_cc_star2d2r", "host_cc_box2d1r", "host_cc_box2d2r", "sweep_step", "Plan",
    "sweep_host", "brick_elems", "plane_elems", "device_error", "sweep_steps_noalloc",
]

STENCILS = {"star2d1r": 0, "star2d2r": 1, "box2d1r": 2, "box2d2r": 3}
RADIUS = {"star2d1r": 1, "star2d2r": 2, "box2d1r": 1, "box2d2r": 2}
ENGINES = {"tensor": 0, "cudacore": 1}
PRECISIONS = {"f16": 0, "split": 1, "f32": 2}

(TCS_OK, TCS_ERR_INVALID, TCS_ERR_CUDA, TCS_ERR_UNSUPPORTED, TCS_ERR_NOMEM, TCS_ERR_TIMEOUT,
 TCS_ERR_CANCELLED) = range(7)

LIB_PATH = _build.LIB


class TcsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class StepArgs(ctypes.Structure):
    _fields_ = [("ny", ctypes.c_int), ("nx", ctypes.c_int), ("stencil", ctypes.c_int),
                ("engine", ctypes.c_int), ("precision", ctypes.c_int), ("y0", ctypes.c_int),
                ("y1", ctypes.c_int), ("x0", ctypes.c_int), ("x1", ctypes.c_int),
                ("coeffs", ctypes.POINTER(ctypes.c_float))]


class Problem(ctypes.Structure):
    _fields_ = [("ny", ctypes.c_int), ("nx", ctypes.c_int), ("stencil", ctypes.c_int),
                ("engine", ctypes.c_int), ("precision", ctypes.c_int), ("y0", ctypes.c_int),
                ("y1", ctypes.c_int), ("x0", ctypes.c_int), ("x1", ctypes.c_int),
                ("coeffs", ctypes.POINTER(ctypes.c_float))]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_active", ctypes.c_int),
                ("round_steps", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("failed", ctypes.c_longlong), ("rounds", ctypes.c_longlong),
                ("point_updates", ctypes.c_longlong), ("algorithmic_bytes", ctypes.c_longlong),
                ("gpu_busy_s", ctypes.c_double), ("budget_bytes", ctypes.c_size_t),
                ("peak_bytes_in_use", ctypes.c_size_t), ("active", ctypes.c_int),
                ("queued", ctypes.c_int), ("sched_total_s", ctypes.c_double * 4),
                ("sched_max_s", ctypes.c_double * 4), ("launch_total_s", ctypes.c_double * 3),
                ("launch_max_s", ctypes.c_double * 3), ("cancelled", ctypes.c_longlong)]


# int hook(size_t bytes, const char *what, void *user): non-zero fails the allocation
ALLOC_HOOK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_void_p)


_lib = None

# name -> (restype, argtypes) for every function include/tcs.h declares
_P, _I, _F, _SZ, _U16 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t, ctypes.c_uint16
_HOST = [_P, _P, _P, _I, _I]
SIGNATURES = {
    "tcs_status_string": (ctypes.c_char_p, [_I]),
    "tcs_last_error": (ctypes.c_char_p, []),
    "tcs_stencil_radius": (_I, [_I]),
    "tcs_brick_elems": (_SZ, [_I, _I]),
    "tcs_plane_elems": (_SZ, [_I, _I, _I]),
    "tcs_device_error": (_I, [_P]),
    "host_star2d1r": (None, _HOST), "host_star2d2r": (None, _HOST),
    "host_box2d1r": (None, _HOST), "host_box2d2r": (None, _HOST),
    "host_cc_star2d1r": (None, _HOST), "host_cc_star2d2r": (None, _HOST),
    "host_cc_box2d1r": (None, _HOST), "host_cc_box2d2r": (None, _HOST),
    "tcs_host_code": (_I, _HOST + [_I, _I, _I, _I, _I, _I]),
    "tcs_padding_2d": (_I, [_P, _P, _I, _I, _U16, _P]),
    "tcs_brick_layout_2d": (_I, [_P, _P, _I, _I, _P]),
    "tcs_reverse_layout_2d": (_I, [_P, _P, _I, _I, _P]),
    "tcs_pack_f16": (_I, [_P, _I, _I, _I, _F, _P, _P]),
    "tcs_unpack_f16": (_I, [_P, _I, _I, _I, _P, _P]),
    "tcs_pack_f32": (_I, [_P, _I, _I, _I, _F, _P, _P]),
    "tcs_unpack_f32": (_I, [_P, _I, _I, _I, _P, _P]),
    "tcs_pack_split": (_I, [_P, _I, _I, _I, _F, _I, _P, _P, _P]),
    "tcs_unpack_split": (_I, [_P, _P, _I, _I, _I, _I, _P, _P]),
    "tcs_max_abs_f32": (_I, [_P, _SZ, ctypes.POINTER(ctypes.c_float), _P]),
    "tcs_split_scale_exp": (_I, [_F]),
    "tcs_plan_scale_exp": (_I, [_P, ctypes.POINTER(_I)]),
    "tcs_init_coe_star": (_I, [_P, _I, _P, _P]),
    "tcs_init_coe_box": (_I, [_P, _I, _P]),
    "tcs_sweep_step": (_I, [ctypes.POINTER(StepArgs), _P, _P, _P, _P, _P]),
    "tcs_plan_create": (_I, [ctypes.POINTER(Problem), ctypes.POINTER(_P)]),
    "tcs_plan_destroy": (_I, [_P]),
    "tcs_plan_upload": (_I, [_P, _P, _I, _P]),
    "tcs_plan_download": (_I, [_P, _P, _I, _P]),
    "tcs_plan_run": (_I, [_P, _I, _I, _P]),
    "tcs_plan_state": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_SZ)]),
    "tcs_plan_set_coeffs": (_I, [_P, _P]),
    "tcs_plan_set_temporal_depth": (_I, [_P, _I]),
    "tcs_plan_set_multistep": (_I, [_P, _I]),
    "tcs_plan_set_tile_width": (_I, [_P, _I]),
    "tcs_plan_tile_width": (_I, [_P, ctypes.POINTER(_I)]),
    "tcs_plan_launches": (_I, [_P, _I, _P]),
    "tcs_sweep_host": (_I, [_P, _P, ctypes.POINTER(Problem), _I]),
    "tcs_noalloc_scratch_bytes": (_SZ, []),
    "tcs_sweep_steps_noalloc": (_I, [ctypes.POINTER(StepArgs), _P, _P, _I, _P]),
    "tcs_release_cache": (None, []),
    "tcs_batch_create": (_I, [ctypes.POINTER(_P)]),
    "tcs_batch_destroy": (_I, [_P]),
    "tcs_batch_add": (_I, [_P, ctypes.POINTER(Problem), _I, ctypes.POINTER(_I)]),
    "tcs_batch_upload": (_I, [_P, _I, _P, _I, _P]),
    "tcs_batch_download": (_I, [_P, _I, _P, _I, _P]),
    "tcs_batch_run": (_I, [_P, _I, _P]),
    "tcs_batch_info": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_I),
                            ctypes.POINTER(_I)]),
    "tcs_batch_set_gate": (_I, [_P, _I, _P, ctypes.c_uint]),
    "tcs_pipe_create": (_I, [ctypes.POINTER(Problem), ctypes.POINTER(_P)]),
    "tcs_pipe_destroy": (_I, [_P]),
    "tcs_pipe_submit": (_I, [_P, _P, _P, _I]),
    "tcs_pipe_wait": (_I, [_P]),
    "tcs_batch_set_wait_limit": (_I, [_P, ctypes.c_double]),
    "tcs_drift_create": (_I, [ctypes.POINTER(Problem), ctypes.POINTER(_P)]),
    "tcs_drift_destroy": (_I, [_P]),
    "tcs_drift_upload": (_I, [_P, _P, _I, _P]),
    "tcs_drift_run": (_I, [_P, _I, _P]),
    "tcs_drift_compare": (_I, [_P, _P, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double), _P]),
    "tcs_drift_state": (_I, [_P, ctypes.POINTER(_P)]),
    "tcs_drift_download": (_I, [_P, _P, _P]),
    "tcs_server_create": (_I, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "tcs_server_destroy": (_I, [_P]),
    "tcs_server_submit": (_I, [_P, ctypes.POINTER(Problem), _I, _P, _P,
                               ctypes.POINTER(ctypes.c_longlong)]),
    "tcs_server_poll": (_I, [_P, ctypes.c_longlong, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "tcs_server_wait": (_I, [_P, ctypes.c_longlong, ctypes.c_double]),
    "tcs_server_times": (_I, [_P, ctypes.c_longlong, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "tcs_server_clock": (ctypes.c_double, [_P]),
    "tcs_server_cancel": (_I, [_P, ctypes.c_longlong]),
    "tcs_set_alloc_hook": (_I, [ALLOC_HOOK, _P]),
    "tcs_set_guard_bytes": (_I, [_SZ]),
    "tcs_guard_check": (_I, [ctypes.POINTER(ctypes.c_longlong)]),
    "tcs_alloc_stats": (_I, [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_SZ)]),
    "tcs_server_get_stats": (_I, [_P, ctypes.POINTER(ServerStats)]),
}


def lib() -> ctypes.CDLL:
    """The loaded native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA engine with tcstencil_gb300.build.build() "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int) -> None:
    if status != TCS_OK:
        L = lib()
        raise TcsError(status, f"{L.tcs_status_string(status).decode()}: "
                               f"{L.tcs_last_error().decode()}")


def _ptr(x) -> int | None:
    """Device/host address of a torch tensor, numpy array or int (None -> NULL)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(f"cannot take the address of {type(x)}")


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def _coeffs(coeffs, stencil: str) -> np.ndarray:
    n = 2 * RADIUS[stencil] + 1
    c = np.ascontiguousarray(coeffs, dtype=np.float32).reshape(-1)
    if c.size != n * n:
        raise ValueError(f"{stencil} needs {n}x{n} coefficients, got {c.size}")
    return c


def brick_elems(ny: int, nx: int) -> int:
    """Elements of the reference's layout16 bricks of an ny x nx grid."""
    return lib().tcs_brick_elems(ny, nx)


def plane_elems(ny: int, nx: int, precision: str = "f16") -> int:
    """Elements of one engine plane (panel layout, see include/tcs.h)."""
    return lib().tcs_plane_elems(ny, nx, PRECISIONS[precision])


def device_error() -> int:
    """Reads and clears the device error word (raises TcsError on a timeout)."""
    code = ctypes.c_int(0)
    _check(lib().tcs_device_error(ctypes.byref(code)))
    return code.value


# --------------------------------------------------------------- drop-in --
def host_code(h_A: np.ndarray, h_B: np.ndarray, h_C: np.ndarray, N: int, n: int,
              stencil: str, engine: str = "tensor", run_times: int = 500,
              skip_times: int = 400, step_times: int = 1, tile_size: int = 1) -> None:
    """The reference's host_code(h_A, h_B, h_C, N, n) (layout16/host_star2d1r.cu:129),
    with the common/param.hpp macros as keyword arguments."""
    for a, shape in ((h_A, (N, N)), (h_C, (N, N)), (h_B, (n, n))):
        if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"] or a.size != shape[0] * shape[1]:
            raise ValueError("host_code takes C-contiguous float32 arrays")
    _check(lib().tcs_host_code(_ptr(h_A), _ptr(h_B), _ptr(h_C), N, n, STENCILS[stencil],
                               ENGINES[engine], run_times, skip_times, step_times, tile_size))


def _drop_in(stencil, engine):
    def f(h_A, h_B, h_C, N, n, **kw):
        host_code(h_A, h_B, h_C, N, n, stencil, engine, **kw)
    f.__name__ = ("host_cc_" if engine == "cudacore" else "host_") + stencil
    f.__doc__ = f"host_code of the reference's {stencil} ({engine} form)."
    return f


host_star2d1r = _drop_in("star2d1r", "tensor")
host_star2d2r = _drop_in("star2d2r", "tensor")
host_box2d1r = _drop_in("box2d1r", "tensor")
host_box2d2r = _drop_in("box2d2r", "tensor")
host_cc_star2d1r = _drop_in("star2d1r", "cudacore")
host_cc_star2d2r = _drop_in("star2d2r", "cudacore")
host_cc_box2d1r = _drop_in("box2d1r", "cudacore")
host_cc_box2d2r = _drop_in("box2d2r", "cudacore")


# --------------------------------------------------------------- extended --
def _rect(rect):
    return (0, 0, 0, 0) if rect is None else tuple(int(v) for v in rect)


def sweep_step(d_in, d_out, ny: int, nx: int, stencil: str, coeffs, engine: str = "tensor",
               precision: str = "f16", rect=None, d_in_lo=None, d_out_lo=None,
               stream=None) -> None:
    """One step on caller-owned device planes (tcs_sweep_step)."""
    c = _coeffs(coeffs, stencil)
    y0, y1, x0, x1 = _rect(rect)
    a = StepArgs(ny, nx, STENCILS[stencil], ENGINES[engine], PRECISIONS[precision], y0, y1, x0,
                 x1, c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    _check(lib().tcs_sweep_step(ctypes.byref(a), _ptr(d_in), _ptr(d_in_lo), _ptr(d_out),
                                _ptr(d_out_lo), _stream(stream)))


def sweep_steps_noalloc(d_in, d_out, ny: int, nx: int, stencil: str, coeffs, steps: int,
                        engine: str = "tensor", rect=None, stream=None) -> None:
    """`steps` FP16 sweep steps from d_in to d_out with no device allocation
    (tcs_sweep_steps_noalloc): for callers that may not call cudaMalloc where
    they sweep (allocator-free loops, device memory owned by a pool or budget
    they do not control).  The ping-pong plane is a 32 MiB static device array
    shared by all calls on a GPU, so overlapping calls race; make the first
    call on a device before any stream capture."""
    c = _coeffs(coeffs, stencil)
    y0, y1, x0, x1 = _rect(rect)
    a = StepArgs(ny, nx, STENCILS[stencil], ENGINES[engine], PRECISIONS["f16"], y0, y1, x0, x1,
                 c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    _check(lib().tcs_sweep_steps_noalloc(ctypes.byref(a), _ptr(d_in), _ptr(d_out), steps,
                                         _stream(stream)))


class Plan:
    """Device-resident sweep of one grid (tcs_plan_*)."""

    def __init__(self, ny: int, nx: int, stencil: str, coeffs, engine: str = "tensor",
                 precision: str = "f16", rect=None, temporal_depth: int | None = None,
                 tile_w: int | None = None):
        """engine "auto" takes the autotuner's choice for this problem class
        (engine, temporal depth, launch form and tile width); temporal_depth 2
        runs steps in blocked pairs (split precision, tensor engine); tile_w
        (128, 96 or 64) is the tile width of plain FP16 tensor sweeps."""
        tuned_launch = -1
        if engine == "auto":
            from .autotune import best_config, best_launch, best_tile_width

            engine, tuned_depth = best_config(stencil, precision, ny, nx)
            if temporal_depth is None:
                temporal_depth = tuned_depth
            tuned_launch = best_launch(stencil, precision, ny, nx)
            if tile_w is None and engine == "tensor" and precision == "f16":
                tile_w = best_tile_width(stencil, ny, nx)
        self._c = _coeffs(coeffs, stencil)
        y0, y1, x0, x1 = _rect(rect)
        self.ny, self.nx, self.stencil, self.engine, self.precision = ny, nx, stencil, engine, precision
        pr = Problem(ny, nx, STENCILS[stencil], ENGINES[engine], PRECISIONS[precision], y0, y1,
                     x0, x1, self._c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        h = ctypes.c_void_p()
        _check(lib().tcs_plan_create(ctypes.byref(pr), ctypes.byref(h)))
        self._h = h
        if temporal_depth and temporal_depth != 1:
            self.set_temporal_depth(temporal_depth)
        if tuned_launch >= 0 and engine == "tensor":
            self.set_multistep(tuned_launch)
        if tile_w and tile_w != 128:
            self.set_tile_width(tile_w)

    def set_temporal_depth(self, depth: int) -> None:
        _check(lib().tcs_plan_set_temporal_depth(self._h, int(depth)))

    def launches(self, steps: int) -> int:
        """Kernel launches run(steps) makes."""
        n = ctypes.c_int(0)
        _check(lib().tcs_plan_launches(self._h, int(steps), ctypes.byref(n)))
        return n.value

    def set_multistep(self, mode: int) -> None:
        """Tensor plans (FP16 or split, temporal depth 1): run(steps) as one
        launch (1), one launch per step (0), or by grid size (-1, the
        default); same bits."""
        _check(lib().tcs_plan_set_multistep(self._h, int(mode)))

    def set_tile_width(self, tile_w: int) -> None:
        """Plain FP16 tensor plans: tiles of 128 rows by tile_w = 128, 96 or
        64 columns; same bits."""
        _check(lib().tcs_plan_set_tile_width(self._h, int(tile_w)))

    def tile_width(self) -> int:
        w = ctypes.c_int()
        _check(lib().tcs_plan_tile_width(self._h, ctypes.byref(w)))
        return w.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().tcs_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, grid, stream=None) -> None:
        """grid: ny x nx float32 (numpy = host memory, torch CUDA tensor = device)."""
        on_host = isinstance(grid, np.ndarray) or (hasattr(grid, "is_cuda") and not grid.is_cuda)
        _check(lib().tcs_plan_upload(self._h, _ptr(grid), int(on_host), _stream(stream)))

    def download(self, out, stream=None) -> None:
        on_host = isinstance(out, np.ndarray) or (hasattr(out, "is_cuda") and not out.is_cuda)
        _check(lib().tcs_plan_download(self._h, _ptr(out), int(on_host), _stream(stream)))

    def run(self, steps: int, use_graph: bool = True, stream=None) -> None:
        _check(lib().tcs_plan_run(self._h, steps, int(use_graph), _stream(stream)))

    def state(self):
        """(hi device pointer, lo device pointer or None, bytes per plane)."""
        hi, lo, nb = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
        _check(lib().tcs_plan_state(self._h, ctypes.byref(hi), ctypes.byref(lo), ctypes.byref(nb)))
        return hi.value, lo.value, nb.value

    def scale_exp(self) -> int:
        """Split plans store x 2^-E; returns E (0 for other precisions)."""
        e = ctypes.c_int(0)
        _check(lib().tcs_plan_scale_exp(self._h, ctypes.byref(e)))
        return e.value

    def set_coeffs(self, coeffs) -> None:
        self._c = _coeffs(coeffs, self.stencil)
        _check(lib().tcs_plan_set_coeffs(self._h, _ptr(self._c)))


def _on_host(a) -> bool:
    return isinstance(a, np.ndarray) or (hasattr(a, "is_cuda") and not a.is_cuda)


class Batch:
    """Many grids advanced by one persistent tensor-core launch per run
    (tcs_batch_*).  Add every grid, upload each, then run and download."""

    def __init__(self):
        h = ctypes.c_void_p()
        _check(lib().tcs_batch_create(ctypes.byref(h)))
        self._h = h
        self._coeffs = []
        self.shapes = []

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().tcs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, ny: int, nx: int, stencil: str, coeffs, steps: int, precision: str = "f16",
            rect=None) -> int:
        c = _coeffs(coeffs, stencil)
        y0, y1, x0, x1 = _rect(rect)
        pr = Problem(ny, nx, STENCILS[stencil], ENGINES["tensor"], PRECISIONS[precision], y0, y1,
                     x0, x1, c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        idx = ctypes.c_int(-1)
        _check(lib().tcs_batch_add(self._h, ctypes.byref(pr), int(steps), ctypes.byref(idx)))
        self._coeffs.append(c)
        self.shapes.append((ny, nx))
        return idx.value

    def upload(self, index: int, grid, stream=None) -> None:
        _check(lib().tcs_batch_upload(self._h, index, _ptr(grid), int(_on_host(grid)),
                                      _stream(stream)))

    def download(self, index: int, out, stream=None) -> None:
        _check(lib().tcs_batch_download(self._h, index, _ptr(out), int(_on_host(out)),
                                        _stream(stream)))

    def run(self, use_graph: bool = True, stream=None) -> None:
        _check(lib().tcs_batch_run(self._h, int(use_graph), _stream(stream)))

    def set_gate(self, index: int, d_flag, value: int) -> None:
        """Grid `index` starts once the device word at d_flag is >= value."""
        _check(lib().tcs_batch_set_gate(self._h, index, _ptr(d_flag), int(value)))

    def set_wait_limit(self, seconds: float) -> None:
        _check(lib().tcs_batch_set_wait_limit(self._h, float(seconds)))

    def info(self):
        """(point updates per run, work items per run, grids)."""
        pu, it, g = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
        _check(lib().tcs_batch_info(self._h, ctypes.byref(pu), ctypes.byref(it), ctypes.byref(g)))
        return pu.value, it.value, g.value


class Pipe:
    """Many grids of one shape through the device, double-buffered
    (tcs_pipe_*): submit(h_in, h_out, steps) returns at once; submission k's
    buffers are the pipe's until submission k + 2 or wait().  Pinned host
    buffers let the copies overlap the sweeps."""

    def __init__(self, ny: int, nx: int, stencil: str, coeffs, engine: str = "tensor",
                 precision: str = "f16", rect=None):
        self._c = _coeffs(coeffs, stencil)
        y0, y1, x0, x1 = _rect(rect)
        pr = Problem(ny, nx, STENCILS[stencil], ENGINES[engine], PRECISIONS[precision], y0, y1, x0,
                     x1, self._c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        h = ctypes.c_void_p()
        _check(lib().tcs_pipe_create(ctypes.byref(pr), ctypes.byref(h)))
        self._h = h
        self.shape = (ny, nx)
        self._held = []

    def submit(self, h_in: np.ndarray, h_out: np.ndarray, steps: int) -> None:
        for a in (h_in, h_out):
            if a.dtype != np.float32 or a.shape != self.shape or not a.flags.c_contiguous:
                raise ValueError("pipe buffers are C-contiguous float32 grids of the pipe's shape")
        _check(lib().tcs_pipe_submit(self._h, _ptr(h_in), _ptr(h_out), int(steps)))
        self._held = (self._held + [(h_in, h_out)])[-2:]

    def wait(self) -> None:
        _check(lib().tcs_pipe_wait(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().tcs_pipe_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Drift:
    """FP64 shadow of a stencil problem on the device (tcs_drift_*)."""

    def __init__(self, ny: int, nx: int, stencil: str, coeffs, rect=None):
        self._c = _coeffs(coeffs, stencil)
        y0, y1, x0, x1 = _rect(rect)
        pr = Problem(ny, nx, STENCILS[stencil], ENGINES["tensor"], PRECISIONS["f16"], y0, y1, x0,
                     x1, self._c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        h = ctypes.c_void_p()
        _check(lib().tcs_drift_create(ctypes.byref(pr), ctypes.byref(h)))
        self._h = h
        self.shape = (ny, nx)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().tcs_drift_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, grid, stream=None) -> None:
        _check(lib().tcs_drift_upload(self._h, _ptr(grid), int(_on_host(grid)), _stream(stream)))

    def run(self, steps: int, stream=None) -> None:
        _check(lib().tcs_drift_run(self._h, int(steps), _stream(stream)))

    def compare(self, d_grid, stream=None):
        """(relative L2, max abs) of a device FP32 grid against the shadow."""
        rel, mx = ctypes.c_double(), ctypes.c_double()
        _check(lib().tcs_drift_compare(self._h, _ptr(d_grid), ctypes.byref(rel),
                                       ctypes.byref(mx), _stream(stream)))
        return rel.value, mx.value

    def state(self) -> int:
        p = ctypes.c_void_p()
        _check(lib().tcs_drift_state(self._h, ctypes.byref(p)))
        return p.value

    def download(self) -> np.ndarray:
        out = np.empty(self.shape, np.float64)
        _check(lib().tcs_drift_download(self._h, _ptr(out), None))
        return out


class Server:
    """Continuous-batching request server (tcs_server_*).  submit() hands the
    host buffers to the server until the ticket completes; keep references to
    them (this wrapper does) until then."""

    def __init__(self, hbm_budget_bytes: int, max_active: int = 0, round_steps: int = 0):
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_active), int(round_steps))
        h = ctypes.c_void_p()
        _check(lib().tcs_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._held = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            _check(lib().tcs_server_destroy(self._h))
            self._h = None
            self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, grid: np.ndarray, out: np.ndarray, stencil: str, coeffs, steps: int,
               precision: str = "f16", rect=None) -> int:
        """Queues `steps` steps of a tensor-engine solve from `grid` into `out`
        (both ny x nx float32 host arrays, ideally pinned); returns the ticket."""
        assert grid.dtype == np.float32 and out.dtype == np.float32 and grid.shape == out.shape
        assert grid.flags.c_contiguous and out.flags.c_contiguous
        ny, nx = grid.shape
        c = _coeffs(coeffs, stencil)
        y0, y1, x0, x1 = _rect(rect)
        pr = Problem(ny, nx, STENCILS[stencil], ENGINES["tensor"], PRECISIONS[precision], y0, y1,
                     x0, x1, c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        t = ctypes.c_longlong()
        _check(lib().tcs_server_submit(self._h, ctypes.byref(pr), int(steps), _ptr(grid),
                                       _ptr(out), ctypes.byref(t)))
        self._held[t.value] = (grid, out)
        return t.value

    def poll(self, ticket: int):
        """(state, status): state 0 queued, 1 resident, 2 done, 3 failed."""
        st, status = ctypes.c_int(), ctypes.c_int()
        _check(lib().tcs_server_poll(self._h, ticket, ctypes.byref(st), ctypes.byref(status)))
        return st.value, status.value

    def wait(self, ticket: int, timeout: float = -1.0) -> None:
        _check(lib().tcs_server_wait(self._h, ticket, float(timeout)))
        self._held.pop(ticket, None)

    def cancel(self, ticket: int) -> None:
        """tcs_server_cancel: the ticket ends failed with TCS_ERR_CANCELLED."""
        _check(lib().tcs_server_cancel(self._h, ticket))

    def times(self, ticket: int):
        """(submitted, admitted, completed) on the server clock, seconds."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(lib().tcs_server_times(self._h, ticket, ctypes.byref(a), ctypes.byref(b),
                                      ctypes.byref(c)))
        return a.value, b.value, c.value

    def clock(self) -> float:
        return lib().tcs_server_clock(self._h)

    def stats(self) -> dict:
        o = ServerStats()
        _check(lib().tcs_server_get_stats(self._h, ctypes.byref(o)))
        return {k: (list(getattr(o, k)) if k.startswith(("sched_", "launch_")) else getattr(o, k))
                for k, _ in ServerStats._fields_}


_hook_ref = None  # the installed allocation hook's ctypes callback, kept alive


def set_alloc_hook(fn) -> None:
    """tcs_set_alloc_hook: fn(bytes, what) -> True to fail that allocation
    (TCS_ERR_NOMEM from the call that needed it); None removes the hook."""
    global _hook_ref
    if fn is None:
        _check(lib().tcs_set_alloc_hook(ALLOC_HOOK(), None))
        _hook_ref = None
        return
    cb = ALLOC_HOOK(lambda n, what, user: 1 if fn(int(n), what.decode()) else 0)
    _check(lib().tcs_set_alloc_hook(cb, None))
    _hook_ref = cb


def set_guard_bytes(n: int) -> None:
    """tcs_set_guard_bytes: canary regions of n bytes (rounded up to 256)
    around allocations made from now on; 0 turns them off."""
    _check(lib().tcs_set_guard_bytes(int(n)))


def guard_check() -> int:
    """tcs_guard_check: the number of guard regions found changed (0: none)."""
    n = ctypes.c_longlong()
    _check(lib().tcs_guard_check(ctypes.byref(n)))
    return n.value


def alloc_stats():
    """tcs_alloc_stats: (live allocations, live bytes) of the library."""
    c, b = ctypes.c_longlong(), ctypes.c_size_t()
    _check(lib().tcs_alloc_stats(ctypes.byref(c), ctypes.byref(b)))
    return c.value, b.value


def sweep_host(h_in: np.ndarray, steps: int, stencil: str, coeffs, engine: str = "tensor",
               precision: str = "f16", rect=None, h_out: np.ndarray | None = None) -> np.ndarray:
    """Host FP32 grid in, `steps` Jacobi steps, host FP32 grid out (tcs_sweep_host)."""
    h_in = np.ascontiguousarray(h_in, dtype=np.float32)
    ny, nx = h_in.shape
    out = np.empty_like(h_in) if h_out is None else h_out
    c = _coeffs(coeffs, stencil)
    y0, y1, x0, x1 = _rect(rect)
    pr = Problem(ny, nx, STENCILS[stencil], ENGINES[engine], PRECISIONS[precision], y0, y1, x0,
                 x1, c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    _check(lib().tcs_sweep_host(_ptr(h_in), _ptr(out), ctypes.byref(pr), steps))
    return out
