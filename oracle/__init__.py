"""CPU oracle for the 2-D Jacobi sweep hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this package, and only as the checker.  The tcstencil_gb300 product
never imports, loads or calls it.

`oracle.c` restates the reference's gold codes (common/gold_*.cpp), its layout
helpers (layout16/host_star2d1r.cu:33-101) and the arithmetic contracts of the
GPU engine; see its header for the file:line of each function.  `ref` (below)
loads the reference's own gold/helpers when they were compiled from the
reference sources by `make -C oracle ref`; they pin this restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def ref_src_dir() -> str:
    """Where the reference's sources are: $TCS_REF_DIR, else a TCStencil
    checkout named `reference` beside this repository."""
    return os.environ.get("TCS_REF_DIR") or os.path.abspath(
        os.path.join(HERE, "..", "..", "reference"))

STENCILS = {"star2d1r": 0, "star2d2r": 1, "box2d1r": 2, "box2d2r": 3}
RADIUS = {"star2d1r": 1, "star2d2r": 2, "box2d1r": 1, "box2d2r": 2}
SPLIT_SCALE = 2048.0

_lib = None


def build() -> str:
    """Compiles liboracle.so (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "oracle.c")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        for name in ("oracle_gold_step_f32", "oracle_step_f64", "oracle_step_f16cc",
                     "oracle_step_f32", "oracle_step_f16tc"):
            getattr(L, name).argtypes = [P, P, P, I, I, I, I, I, I, I]
            getattr(L, name).restype = I
        L.oracle_step_split.argtypes = [P, P, P, P, P, I, I, I, I, I, I, I]
        L.oracle_step_split.restype = I
        for name in ("oracle_sweep_f32", "oracle_sweep_f64", "oracle_sweep_f16cc",
                     "oracle_sweep_f16tc"):
            getattr(L, name).argtypes = [P, P, I, I, I, I, I, I, I, I]
            getattr(L, name).restype = I
        L.oracle_sweep_split.argtypes = [P, P, P, I, I, I, I, I, I, I, I, P]
        L.oracle_sweep_split.restype = I
        L.oracle_f32_to_f16.argtypes = [P, P, ctypes.c_long]
        L.oracle_f16_to_f32.argtypes = [P, P, ctypes.c_long]
        L.oracle_split_f64.argtypes = [P, P, P, ctypes.c_long, I]
        L.oracle_join_f64.argtypes = [P, P, P, ctypes.c_long, I]
        L.oracle_pad_2d.argtypes = [P, P, I, I, ctypes.c_uint16]
        L.oracle_brick_2d.argtypes = [P, P, I, I, I, ctypes.c_uint16]
        L.oracle_unbrick_2d.argtypes = [P, P, I, I, I]
        L.oracle_init_coe_star.argtypes = [P, I, P, P]
        L.oracle_init_coe_box.argtypes = [P, I, P]
        D = ctypes.c_double
        L.oracle_check_error_2d.argtypes = [I, P, P, I, I, I, I, I, D, D, P, P, P, P, P, P, I]
        L.oracle_check_error_2d.restype = D
        L.oracle_gold_loop_step.argtypes = [P, P, P, I, I, I]
        L.oracle_gold_loop_step.restype = I
        L.oracle_gold_bench_bands.argtypes = [P, P, I, I, I, I, I, I, P]
        L.oracle_gold_bench_bands.restype = ctypes.c_double
        L.oracle_stencil_taps.argtypes = [I, P, P]
        L.oracle_stencil_taps.restype = I
        _lib = L
    return _lib


def _p(a: np.ndarray) -> ctypes.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def _rect(rect):
    return (0, 0, 0, 0) if rect is None else tuple(int(v) for v in rect)


def _coef(B, stencil):
    n = 2 * RADIUS[stencil] + 1
    B = np.ascontiguousarray(B, dtype=np.float32).reshape(n, n)
    return B


# ------------------------------------------------------------ conversions --
def f32_to_f16(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint16)
    lib().oracle_f32_to_f16(_p(a), _p(out), a.size)
    return out


def f16_to_f32(h: np.ndarray) -> np.ndarray:
    h = np.ascontiguousarray(h, dtype=np.uint16)
    out = np.empty(h.shape, dtype=np.float32)
    lib().oracle_f16_to_f32(_p(h), _p(out), h.size)
    return out


def split_scale_exp(x: np.ndarray) -> int:
    """Smallest E with max|x| 2^-E <= 1 (the engine's choice; 0 for all-zero)."""
    m = float(np.max(np.abs(x))) if x.size else 0.0
    return 0 if m == 0.0 else int(np.frexp(np.float32(m))[1])


def split(x: np.ndarray, scale_exp: int = 0):
    x = np.ascontiguousarray(x, dtype=np.float64)
    hi = np.empty(x.shape, np.uint16)
    lo = np.empty(x.shape, np.uint16)
    lib().oracle_split_f64(_p(x), _p(hi), _p(lo), x.size, scale_exp)
    return hi, lo


def join(hi: np.ndarray, lo: np.ndarray, scale_exp: int = 0) -> np.ndarray:
    hi = np.ascontiguousarray(hi, np.uint16)
    lo = np.ascontiguousarray(lo, np.uint16)
    out = np.empty(hi.shape, np.float64)
    lib().oracle_join_f64(_p(hi), _p(lo), _p(out), hi.size, scale_exp)
    return out


# ---------------------------------------------------------------- layouts --
def pad_2d(a16: np.ndarray, halo: int, value16: int) -> np.ndarray:
    size = a16.shape[0]
    a16 = np.ascontiguousarray(a16, np.uint16)
    out = np.empty((size + 2 * halo, size + 2 * halo), np.uint16)
    lib().oracle_pad_2d(_p(a16), _p(out), size, halo, value16)
    return out


def brick_2d(a16: np.ndarray, b: int = 16, fill: int = 0) -> np.ndarray:
    ny, nx = a16.shape
    nby, nbx = -(-ny // b), -(-nx // b)
    a16 = np.ascontiguousarray(a16, np.uint16)
    out = np.empty(nby * nbx * b * b, np.uint16)
    lib().oracle_brick_2d(_p(a16), _p(out), ny, nx, b, fill)
    return out


def unbrick_2d(bricks: np.ndarray, ny: int, nx: int, b: int = 16) -> np.ndarray:
    bricks = np.ascontiguousarray(bricks, np.uint16)
    out = np.empty((ny, nx), np.uint16)
    lib().oracle_unbrick_2d(_p(bricks), _p(out), ny, nx, b)
    return out


def init_coe_star(B16: np.ndarray, n: int):
    B16 = np.ascontiguousarray(B16, np.uint16).reshape(-1)
    a = np.empty(256, np.uint16)
    b = np.empty(256, np.uint16)
    lib().oracle_init_coe_star(_p(B16), n, _p(a), _p(b))
    return a, b


def init_coe_box(B16: np.ndarray, n: int):
    B16 = np.ascontiguousarray(B16, np.uint16).reshape(-1)
    coe = np.empty(256 * n, np.uint16)
    lib().oracle_init_coe_box(_p(B16), n, _p(coe))
    return coe


def stencil_taps(stencil: str):
    dy = np.zeros(25, np.int32)
    dx = np.zeros(25, np.int32)
    k = lib().oracle_stencil_taps(STENCILS[stencil], _p(dy), _p(dx))
    return list(zip(dy[:k].tolist(), dx[:k].tolist()))


# ----------------------------------------------------------------- sweeps --
def gold_step(A: np.ndarray, B, stencil: str, C: np.ndarray | None = None, rect=None):
    """One FP32 gold step; cells outside the update rectangle keep C's value."""
    A = np.ascontiguousarray(A, np.float32)
    C = np.zeros_like(A) if C is None else np.ascontiguousarray(C, np.float32).copy()
    Bc = _coef(B, stencil)
    rc = lib().oracle_gold_step_f32(_p(A), _p(Bc), _p(C), A.shape[0], A.shape[1],
                                    STENCILS[stencil], *_rect(rect))
    assert rc == 0
    return C


def sweep_f32(A, B, stencil, steps, rect=None):
    g = np.ascontiguousarray(A, np.float32).copy()
    Bc = _coef(B, stencil)
    assert lib().oracle_sweep_f32(_p(g), _p(Bc), g.shape[0], g.shape[1], STENCILS[stencil],
                                  steps, *_rect(rect)) == 0
    return g


def sweep_f64(A, B, stencil, steps, rect=None):
    g = np.ascontiguousarray(A, np.float64).copy()
    n = 2 * RADIUS[stencil] + 1
    Bc = np.ascontiguousarray(B, np.float64).reshape(n, n)
    assert lib().oracle_sweep_f64(_p(g), _p(Bc), g.shape[0], g.shape[1], STENCILS[stencil],
                                  steps, *_rect(rect)) == 0
    return g


def sweep_f16cc(A16, B, stencil, steps, rect=None):
    g = np.ascontiguousarray(A16, np.uint16).copy()
    Bc = _coef(B, stencil)
    assert lib().oracle_sweep_f16cc(_p(g), _p(Bc), g.shape[0], g.shape[1], STENCILS[stencil],
                                    steps, *_rect(rect)) == 0
    return g


def sweep_f16tc(A16, B, stencil, steps, rect=None):
    g = np.ascontiguousarray(A16, np.uint16).copy()
    Bc = _coef(B, stencil)
    assert lib().oracle_sweep_f16tc(_p(g), _p(Bc), g.shape[0], g.shape[1], STENCILS[stencil],
                                    steps, *_rect(rect)) == 0
    return g


def sweep_split(hi, lo, B, stencil, steps, rect=None, scale_exp=0):
    """One run of `steps` split steps from planes in units of 2^scale_exp, with
    the engine's per-step scale; returns (hi, lo, the final exponent)."""
    h = np.ascontiguousarray(hi, np.uint16).copy()
    l = np.ascontiguousarray(lo, np.uint16).copy()
    Bc = _coef(B, stencil)
    e = ctypes.c_int(int(scale_exp))
    assert lib().oracle_sweep_split(_p(h), _p(l), _p(Bc), h.shape[0], h.shape[1],
                                    STENCILS[stencil], steps, *_rect(rect),
                                    ctypes.byref(e)) == 0
    return h, l, e.value


def sweep_f32_fixed(A, B, stencil, steps, rect=None):
    """FP32 storage: gold's arithmetic plus the fixed-border ping-pong copy."""
    return sweep_f32(A, B, stencil, steps, rect)


def check_error_2d(N, output, reference, y_lb, y_ub, x_lb, x_ub, relative=False,
                   tolerance=0.01, min_number=1e-6):
    """checkError2D / checkRelativeError2D (common/common.hpp:38-92): the RMS
    result, the final maximum and its cell, and the cells the reference
    reports with a "Values at index (j,k) differ" line, in order."""
    o = np.ascontiguousarray(output, np.float32)
    r = np.ascontiguousarray(reference, np.float32)
    cap = (y_ub - y_lb) * (x_ub - x_lb)
    mj, mk = np.zeros(max(cap, 1), np.int32), np.zeros(max(cap, 1), np.int32)
    mx = ctypes.c_double()
    j, k, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rms = lib().oracle_check_error_2d(N, _p(o), _p(r), y_lb, y_ub, x_lb, x_ub, int(relative),
                                      tolerance, min_number, ctypes.byref(mx), ctypes.byref(j),
                                      ctypes.byref(k), ctypes.byref(n), _p(mj), _p(mk), cap)
    return {"rms": rms, "max_error": mx.value, "max_at": (j.value, k.value),
            "reported": list(zip(mj[:n.value].tolist(), mk[:n.value].tolist()))}


def gold_loop_step(A: np.ndarray, B, stencil: str, C: np.ndarray | None = None):
    """One gold step in gold's own loop shape (per-tap store into the output
    cell for box stencils); the same bits as gold_step."""
    A = np.ascontiguousarray(A, np.float32)
    C = np.zeros_like(A) if C is None else np.ascontiguousarray(C, np.float32).copy()
    Bc = _coef(B, stencil)
    assert lib().oracle_gold_loop_step(_p(A), _p(Bc), _p(C), A.shape[0], A.shape[1],
                                       STENCILS[stencil]) == 0
    return C


def gold_bench_bands(init: np.ndarray, B, stencil: str, steps: int, threads: int,
                     loop_shape: bool = True, want_out: bool = False):
    """Wall seconds for `steps` ping-pong gold steps of ONE grid, `threads`
    threads on row bands; loop_shape selects gold's own loop shape.  With
    want_out, returns (seconds, final grid)."""
    init = np.ascontiguousarray(init, np.float32)
    Bc = _coef(B, stencil)
    out = np.empty_like(init) if want_out else None
    t = lib().oracle_gold_bench_bands(_p(init), _p(Bc), init.shape[0], init.shape[1],
                                      STENCILS[stencil], steps, threads, int(loop_shape),
                                      _p(out) if want_out else None)
    assert t >= 0, t
    return (t, out) if want_out else t


# ------------------------------------------------------- reference build --
class Ref:
    """The reference's own gold()/layout16 helpers, compiled by `make -C oracle
    ref` from the reference sources, and its GPU kernels as sm_103a cubins
    (`make -C oracle refgpu`, launched by oracle/ref_gpu.py).  Exists only where
    those sources were."""

    def __init__(self, ref_dir: str = REF_DIR):
        self.dir = ref_dir

    @staticmethod
    def build(ref_src: str | None = None) -> bool:
        env = dict(os.environ)
        src = ref_src or ref_src_dir()
        env["TCS_REF_DIR"] = src
        if not os.path.isdir(os.path.join(src, "common")):
            return False
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref", "refgpu"], check=True, env=env)
        return True

    def available(self) -> bool:
        return all(os.path.exists(os.path.join(self.dir, f"libref_gold_{s}.so")) and
                   os.path.exists(os.path.join(self.dir, f"libref_layout16_{s}.so"))
                   for s in STENCILS)

    def _gold(self, stencil):
        L = ctypes.CDLL(os.path.join(self.dir, f"libref_gold_{stencil}.so"))
        L.gold.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_int]
        return L

    def _l16(self, stencil):
        return ctypes.CDLL(os.path.join(self.dir, f"libref_layout16_{stencil}.so"))

    def gold(self, A: np.ndarray, B, stencil: str, C: np.ndarray | None = None):
        """gold(h_A, h_B, h_C, N, n): square N x N, writes [r, N-r)^2 of C."""
        N = A.shape[0]
        assert A.shape == (N, N)
        n = 2 * RADIUS[stencil] + 1
        A = np.ascontiguousarray(A, np.float32)
        Bc = np.ascontiguousarray(B, np.float32).reshape(n, n)
        C = np.zeros_like(A) if C is None else np.ascontiguousarray(C, np.float32).copy()
        self._gold(stencil).gold(_p(A), _p(Bc), _p(C), N, n)
        return C

    def padding_2d(self, a16, halo, value16, stencil="star2d1r"):
        f = self._l16(stencil)._Z10padding_2DP6__halfS0_iiS_
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                      ctypes.c_uint16]
        size = a16.shape[0]
        a16 = np.ascontiguousarray(a16, np.uint16)
        out = np.empty((size + 2 * halo,) * 2, np.uint16)
        f(_p(a16), _p(out), size, halo, value16)
        return out

    def brick_layout_2d(self, a16, block=16, stencil="star2d1r"):
        f = self._l16(stencil)._Z15brick_layout_2DP6__halfS0_ii
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        a16 = np.ascontiguousarray(a16, np.uint16)
        out = np.empty(a16.size, np.uint16)
        f(_p(a16), _p(out), a16.shape[0], block)
        return out

    def reverse_layout_2d(self, bricks, size, block=16, stencil="star2d1r"):
        f = self._l16(stencil)._Z17reverse_layout_2DP6__halfS0_ii
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        bricks = np.ascontiguousarray(bricks, np.uint16)
        out = np.empty((size, size), np.uint16)
        f(_p(bricks), _p(out), size, block)
        return out

    def init_coe(self, B16, stencil):
        f = self._l16(stencil)._Z8init_coeP6__halfS0_S0_i if stencil.startswith("star") else \
            self._l16(stencil)._Z8init_coeP6__halfS0_i
        n = 2 * RADIUS[stencil] + 1
        B16 = np.ascontiguousarray(B16, np.uint16).reshape(-1)
        if stencil.startswith("star"):
            f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int]
            a = np.empty(256, np.uint16)
            b = np.empty(256, np.uint16)
            f(_p(B16), _p(a), _p(b), n)
            return a, b
        f.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int]
        coe = np.empty(256 * n, np.uint16)
        f(_p(B16), _p(coe), n)
        return coe
