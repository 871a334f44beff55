"""Tile shapes of the plain FP16 tensor sweep: 128 rows by 128, 96 or 64
columns (tcs_plan_set_tile_width).  Window boundaries and each window's
parity (even windows initialise the accumulator, odd ones add) do not depend
on the width, so every output sums the same products in the same order:
results must be bit-identical to 128-column tiles, one launch per step and
all steps in one launch, with and without an update rectangle, on grids whose
last tile column is partial; and one step is checked against the oracle."""
import zlib

import numpy as np
import pytest

import oracle
from conftest import STENCILS
from helpers import assert_f16tc_step, grid, normalized_coeffs

pytestmark = pytest.mark.gpu


def run(tcs, A, B, stencil, steps, tile_w, multistep, rect=None):
    p = tcs.Plan(A.shape[0], A.shape[1], stencil, B, engine="tensor", precision="f16", rect=rect)
    p.set_multistep(multistep)
    p.set_tile_width(tile_w)
    assert p.tile_width() == tile_w
    p.upload(A)
    p.run(steps)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    assert tcs.device_error() == 0
    return out


@pytest.mark.parametrize("stencil", STENCILS)
@pytest.mark.parametrize("shape", [(20, 37), (130, 300), (257, 129), (300, 1100), (1026, 1026)])
def test_narrow_tiles_give_the_same_bits(tcs, torch_cuda, stencil, shape):
    rng = np.random.default_rng(zlib.crc32(repr((stencil, shape)).encode()))
    A = grid(rng, *shape)
    B = normalized_coeffs(rng, stencil)
    for multistep in (0, 1):
        ref = run(tcs, A, B, stencil, 3, 128, multistep)
        for w in (96, 64):
            np.testing.assert_array_equal(run(tcs, A, B, stencil, 3, w, multistep), ref,
                                          err_msg=f"width {w}, multistep {multistep}")
    one = run(tcs, A, B, stencil, 1, 64, 0)
    assert_f16tc_step(one, oracle.f32_to_f16(A), B, stencil, f"{stencil} {shape} width 64")


@pytest.mark.parametrize("stencil", ["box2d2r", "star2d1r"])
def test_narrow_tiles_with_an_update_rectangle(tcs, torch_cuda, stencil):
    rng = np.random.default_rng(5)
    A = grid(rng, 300, 270)
    B = normalized_coeffs(rng, stencil)
    rect = (7, 281, 37, 203)  # edges inside 64- and 96-column tiles
    ref = run(tcs, A, B, stencil, 4, 128, 0, rect)
    for w in (96, 64):
        for m in (0, 1):
            np.testing.assert_array_equal(run(tcs, A, B, stencil, 4, w, m, rect), ref)


def test_tile_width_arguments(tcs, torch_cuda):
    B = normalized_coeffs(np.random.default_rng(0), "box2d1r")
    p = tcs.Plan(100, 100, "box2d1r", B, engine="tensor", precision="f16")
    with pytest.raises(tcs.TcsError) as e:
        p.set_tile_width(80)
    assert e.value.status == tcs.TCS_ERR_INVALID
    p.close()
    for engine, precision in (("tensor", "split"), ("cudacore", "f16")):
        p = tcs.Plan(100, 100, "box2d1r", B, engine=engine, precision=precision)
        with pytest.raises(tcs.TcsError) as e:
            p.set_tile_width(64)
        assert e.value.status == tcs.TCS_ERR_UNSUPPORTED
        p.set_tile_width(128)
        p.close()
