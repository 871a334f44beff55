"""Several tensor steps in one launch against one launch per step.

A plan's run(steps) with steps >= 2 on the tensor engine (FP16 or split) can be one
cooperative launch whose tiles of step j wait for the neighbouring tile rows
of step j-1 (per-row completion counters; set_multistep(1) forces it, the
default takes it from a grid size on); run(1) is one launch of one step.
Each tile does the same arithmetic either way, so the results must be
bit-identical, on grids of one tile, one tile row, many rows, more tiles than
CTAs, and with an update rectangle whose outside cells are nonzero.
"""
import os
import subprocess
import sys
import zlib

import numpy as np
import pytest

import oracle
from conftest import STENCILS
from helpers import grid, normalized_coeffs

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _plan_out(tcs, A, B, stencil, steps, one_by_one, rect=None, use_graph=True, mode=1,
              precision="f16"):
    p = tcs.Plan(A.shape[0], A.shape[1], stencil, B, engine="tensor", precision=precision, rect=rect,
                 temporal_depth=1)
    p.set_multistep(mode)
    p.upload(A)
    if one_by_one:
        for _ in range(steps):
            p.run(1)
    else:
        p.run(steps, use_graph=use_graph)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    assert tcs.device_error() == 0
    return out


@pytest.mark.parametrize("precision", ["f16", "split"])
@pytest.mark.parametrize("stencil", STENCILS)
@pytest.mark.parametrize("shape", [(20, 37), (100, 700), (257, 129), (600, 140), (140, 1100)])
@pytest.mark.parametrize("steps", [2, 3, 8])
def test_one_launch_equals_one_step_per_launch(tcs, torch_cuda, precision, stencil, shape, steps):
    rng = np.random.default_rng(zlib.crc32(repr((stencil, shape, steps)).encode()))
    A = grid(rng, *shape)
    B = normalized_coeffs(rng, stencil)
    a = _plan_out(tcs, A, B, stencil, steps, one_by_one=False, precision=precision)
    b = _plan_out(tcs, A, B, stencil, steps, one_by_one=True, precision=precision)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("stencil,precision", [("box2d2r", "f16"), ("star2d1r", "f16"),
                                               ("box2d1r", "split"), ("star2d2r", "split")])
def test_many_tiles_per_cta_and_eager_launch(tcs, torch_cuda, stencil, precision):
    # 33 x 33 tiles = 1089 > 152 CTAs per step, over 12 steps
    rng = np.random.default_rng(77)
    A = grid(rng, 4100, 4100)
    B = normalized_coeffs(rng, stencil)
    kw = dict(precision=precision)
    a = _plan_out(tcs, A, B, stencil, 12, one_by_one=False, **kw)
    b = _plan_out(tcs, A, B, stencil, 12, one_by_one=True, **kw)
    c = _plan_out(tcs, A, B, stencil, 12, one_by_one=False, use_graph=False, **kw)
    d = _plan_out(tcs, A, B, stencil, 12, one_by_one=False, mode=-1, **kw)  # by size: one launch
    e = _plan_out(tcs, A, B, stencil, 12, one_by_one=False, mode=0, **kw)
    for x in (b, c, d, e):
        np.testing.assert_array_equal(a, x)


@pytest.mark.parametrize("precision", ["f16", "split"])
@pytest.mark.parametrize("stencil", STENCILS)
def test_rectangle_outside_cells_kept(tcs, torch_cuda, stencil, precision):
    rng = np.random.default_rng(91)
    A = grid(rng, 300, 270)  # nonzero everywhere, also outside the rectangle
    B = normalized_coeffs(rng, stencil)
    rect = (9, 290, 3, 250)
    a = _plan_out(tcs, A, B, stencil, 6, one_by_one=False, rect=rect, precision=precision)
    b = _plan_out(tcs, A, B, stencil, 6, one_by_one=True, rect=rect, precision=precision)
    np.testing.assert_array_equal(a, b)
    if precision == "f16":
        inside = np.zeros(A.shape, bool)
        inside[rect[0]:rect[1], rect[2]:rect[3]] = True
        A16 = oracle.f16_to_f32(oracle.f32_to_f16(A))
        np.testing.assert_array_equal(a[~inside], A16[~inside])


_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import tcstencil_gb300 as tcs
from helpers import grid, normalized_coeffs
rng = np.random.default_rng(5)
out = []
for (ny, nx), st, prec, eng in (((700, 500), "box2d2r", "f16", "tensor"),
                                ((700, 500), "star2d1r", "f16", "tensor"),
                                ((700, 500), "box2d1r", "split", "tensor"),
                                ((2100, 1500), "box2d1r", "f16", "tensor"),
                                ((2100, 1500), "star2d2r", "f16", "tensor"),
                                ((700, 500), "star2d2r", "f16", "cudacore"),
                                ((2100, 1500), "box2d2r", "f32", "cudacore")):
    A = grid(rng, ny, nx)
    B = normalized_coeffs(rng, st)
    p = tcs.Plan(ny, nx, st, B, engine=eng, precision=prec, temporal_depth=1)
    if eng == "tensor":
        p.set_multistep(1)
    p.upload(A); p.run(9)
    o = np.empty_like(A); p.download(o); p.close()
    out.append(o.ravel())
assert tcs.device_error() == 0
np.save(sys.argv[2], np.concatenate(out))
"""


@pytest.mark.parametrize("env", [{}, {"TCS_PDL": "0"}, {"TCS_MULTI": "0"},
                                 {"TCS_PDL": "0", "TCS_MULTI": "0"}])
def test_launch_switches_change_no_bits(tmp_path, torch_cuda, env):
    """The same sweeps (tensor and CUDA-core steps) with overlapped step
    launches and multi-step launches switched off (environment switches read
    once per process)."""
    def run(e, name):
        path = tmp_path / name
        full = dict(os.environ, **e)
        full["PYTHONPATH"] = os.pathsep.join([ROOT, os.path.join(ROOT, "tests")])
        subprocess.run([sys.executable, "-c", _CHILD, ROOT, str(path)], env=full, check=True,
                       timeout=300)
        return np.load(path)
    base = run({"TCS_PDL": "1", "TCS_MULTI": "1"}, "base.npy")
    got = run(env, "got.npy")
    np.testing.assert_array_equal(base, got)


def test_launch_count_query(tcs, torch_cuda):
    """tcs_plan_launches reports what run(steps) launches: the size rule, the
    forced forms, and temporal-depth pairs."""
    B = normalized_coeffs(np.random.default_rng(1), "box2d2r")
    big = tcs.Plan(4100, 4100, "box2d2r", B, engine="tensor", precision="f16")
    assert big.launches(100) == 1 and big.launches(1) == 1
    big.set_multistep(0)
    assert big.launches(100) == 100
    big.close()
    small = tcs.Plan(300, 300, "box2d2r", B, engine="tensor", precision="f16")
    assert small.launches(10) == 10  # few tiles per SM: one launch per step
    small.set_multistep(1)
    assert small.launches(10) == 1
    small.close()
    pairs = tcs.Plan(300, 300, "box2d2r", B, engine="tensor", precision="split", temporal_depth=2)
    assert pairs.launches(7) == 4
    pairs.close()
    cc = tcs.Plan(300, 300, "box2d2r", B, engine="cudacore", precision="f16")
    assert cc.launches(5) == 5
    cc.close()
