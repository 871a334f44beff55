"""Sweep kernels against the oracle, through the C-ABI.

Bars (per arithmetic contract, see oracle/oracle.c):
  CUDA-core FP16   bit-exact with oracle_step_f16cc (fmaf chain in gold's order)
  CUDA-core FP32   bit-exact with gold (oracle_gold_step_f32 = common/gold_*.cpp)
  tensor FP16      |d| <= 1 FP16 step of the value per step vs oracle_step_f16tc
  tensor split     |d| <= 4e-7 * max|x| per step vs oracle_step_split, and
                   relative L2 error vs FP64 <= 1e-6
"""
import numpy as np
import pytest

import oracle
from conftest import STENCILS
from helpers import f16_ulp, grid, normalized_coeffs

pytestmark = pytest.mark.gpu

SHAPES = [(20, 37), (64, 64), (130, 300), (257, 129)]


def run_plan(tcs, A, B, stencil, steps, engine, precision, rect=None, use_graph=True):
    p = tcs.Plan(A.shape[0], A.shape[1], stencil, B, engine=engine, precision=precision, rect=rect)
    p.upload(A)
    p.run(steps, use_graph=use_graph)
    out = np.empty_like(A)
    p.download(out)
    p.close()
    assert tcs.device_error() == 0
    return out


@pytest.mark.parametrize("stencil", STENCILS)
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("steps", [1, 4])
def test_cudacore_f16_bit_exact(tcs, torch_cuda, stencil, shape, steps):
    rng = np.random.default_rng(hash((stencil, shape, steps)) % 2**32)
    A = grid(rng, *shape)
    B = normalized_coeffs(rng, stencil)
    got = oracle.f32_to_f16(run_plan(tcs, A, B, stencil, steps, "cudacore", "f16"))
    expect = oracle.sweep_f16cc(oracle.f32_to_f16(A), B, stencil, steps)
    np.testing.assert_array_equal(got, expect)


@pytest.mark.parametrize("stencil", STENCILS)
@pytest.mark.parametrize("shape", SHAPES[:3])
def test_cudacore_f32_bit_exact_with_gold(tcs, torch_cuda, stencil, shape):
    rng = np.random.default_rng(17)
    A = grid(rng, *shape)
    B = rng.uniform(-1, 1, (2 * oracle.RADIUS[stencil] + 1,) * 2).astype(np.float32)
    got = run_plan(tcs, A, B, stencil, 3, "cudacore", "f32")
    expect = oracle.sweep_f32(A, B, stencil, 3)
    np.testing.assert_array_equal(got.view(np.uint32), expect.view(np.uint32))


@pytest.mark.parametrize("precision", ["f16", "f32"])
@pytest.mark.parametrize("stencil", STENCILS)
def test_cudacore_interior_and_edge_warps(tcs, torch_cuda, stencil, precision):
    """An update rectangle that cuts through tiles, so that warps whose 32 rows
    and whose tile's columns all lie inside it (the interior path, no per-row
    tests) sit beside warps with rows or columns outside (the general path):
    bit-exact with the oracle, both storage types, over several steps."""
    rng = np.random.default_rng(77)
    A = grid(rng, 420, 700)
    B = normalized_coeffs(rng, stencil)
    rect = (37, 350, 140, 650)
    got = run_plan(tcs, A, B, stencil, 5, "cudacore", precision, rect=rect)
    if precision == "f16":
        expect = oracle.sweep_f16cc(oracle.f32_to_f16(A), B, stencil, 5, rect=rect)
        np.testing.assert_array_equal(oracle.f32_to_f16(got), expect)
    else:
        expect = oracle.sweep_f32(A, B, stencil, 5, rect=rect)
        np.testing.assert_array_equal(got.view(np.uint32), expect.view(np.uint32))


@pytest.mark.parametrize("stencil", ["box2d2r", "star2d2r"])
def test_tensor_single_taps(tcs, torch_cuda, stencil):
    """Each tap alone (coefficient 1.0) shifts the grid exactly; a failure names
    the tap whose row shift or K window is wrong."""
    rng = np.random.default_rng(1)
    r = oracle.RADIUS[stencil]
    n = 2 * r + 1
    A = grid(rng, 150, 170)
    A16 = oracle.f32_to_f16(A)
    bad = []
    for (dy, dx) in oracle.stencil_taps(stencil):
        B = np.zeros((n, n), np.float32)
        B[dy + r, dx + r] = 1.0
        got = oracle.f32_to_f16(run_plan(tcs, A, B, stencil, 1, "tensor", "f16"))
        expect = oracle.sweep_f16tc(A16, B, stencil, 1)
        if not np.array_equal(got, expect):
            diff = np.argwhere(got != expect)
            bad.append(((dy, dx), len(diff), diff[:3].tolist()))
    assert not bad, bad


@pytest.mark.parametrize("stencil", STENCILS)
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("steps", [1, 3])
def test_tensor_f16_within_one_step_per_sweep(tcs, torch_cuda, stencil, shape, steps):
    rng = np.random.default_rng(hash((stencil, shape, steps, "tc")) % 2**32)
    A = grid(rng, *shape)
    B = normalized_coeffs(rng, stencil)
    got = run_plan(tcs, A, B, stencil, steps, "tensor", "f16").astype(np.float64)
    expect = oracle.f16_to_f32(oracle.sweep_f16tc(oracle.f32_to_f16(A), B, stencil, steps))
    tol = steps * f16_ulp(np.abs(expect).max())
    assert np.max(np.abs(got - expect)) <= tol


def smooth_plus_noise(rng, ny, nx):
    """U[-1,1) plus sin(2 pi x) sin(2 pi y), the split-precision test field."""
    yy, xx = np.meshgrid(np.arange(ny) / ny, np.arange(nx) / nx, indexing="ij")
    return (rng.uniform(-1, 1, (ny, nx)) + np.sin(2 * np.pi * xx) * np.sin(2 * np.pi * yy)).astype(np.float32)


@pytest.mark.parametrize("stencil", STENCILS)
@pytest.mark.parametrize("shape", [(40, 70), (130, 300)])
def test_tensor_split_contract_and_fp64_error(tcs, torch_cuda, stencil, shape):
    rng = np.random.default_rng(23)
    A = smooth_plus_noise(rng, *shape)
    B = normalized_coeffs(rng, stencil)
    steps = 10
    got = run_plan(tcs, A, B, stencil, steps, "tensor", "split").astype(np.float64)
    e = oracle.split_scale_exp(A)
    hi, lo = oracle.split(A.astype(np.float64), e)
    h, l, e2 = oracle.sweep_split(hi, lo, B, stencil, steps, scale_exp=e)
    contract = oracle.join(h, l, e2)
    # FP32 (not double) combination of the two accumulators: a few 2^-24 per step
    assert np.max(np.abs(got - contract)) <= steps * 2.0 ** (e - 22)
    ref64 = oracle.sweep_f64(A.astype(np.float64), B.astype(np.float64), stencil, steps)
    rel_l2 = np.linalg.norm(got - ref64) / np.linalg.norm(ref64)
    assert rel_l2 <= 1e-6, rel_l2


@pytest.mark.parametrize("stencil", ["box2d1r", "box2d2r"])
def test_tensor_split_200_steps_within_1e6_of_fp64(tcs, torch_cuda, stencil):
    """The split-precision configuration's bar (FP32 grid as hi+lo FP16,
    200 steps, error vs FP64 <= 1e-6) on a 258^2 grid."""
    rng = np.random.default_rng(200)
    A = smooth_plus_noise(rng, 258, 258)
    B = normalized_coeffs(rng, stencil)
    got = run_plan(tcs, A, B, stencil, 200, "tensor", "split").astype(np.float64)
    ref64 = oracle.sweep_f64(A.astype(np.float64), B.astype(np.float64), stencil, 200)
    rel_l2 = np.linalg.norm(got - ref64) / np.linalg.norm(ref64)
    gold = oracle.sweep_f32(A, B, stencil, 200).astype(np.float64)
    rel_gold = np.linalg.norm(gold - ref64) / np.linalg.norm(ref64)
    assert rel_l2 <= 1e-6, (rel_l2, rel_gold)


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
@pytest.mark.parametrize("stencil", STENCILS)
def test_update_rectangle_keeps_the_rest(tcs, torch_cuda, engine, stencil):
    rng = np.random.default_rng(31)
    A = grid(rng, 90, 140)
    B = normalized_coeffs(rng, stencil)
    rect = (7, 61, 5, 133)
    got = run_plan(tcs, A, B, stencil, 2, engine, "f16", rect=rect)
    A16 = oracle.f32_to_f16(A)
    f = oracle.sweep_f16cc if engine == "cudacore" else oracle.sweep_f16tc
    expect = oracle.f16_to_f32(f(A16, B, stencil, 2, rect=rect))
    mask = np.zeros(A.shape, bool)
    mask[rect[0]:rect[1], rect[2]:rect[3]] = True
    np.testing.assert_array_equal(got[~mask], oracle.f16_to_f32(A16)[~mask])
    assert np.max(np.abs(got - expect)) <= 2 * f16_ulp(np.abs(expect).max())


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
def test_graph_replay_equals_eager(tcs, torch_cuda, engine):
    rng = np.random.default_rng(41)
    A = grid(rng, 200, 333)
    B = normalized_coeffs(rng, "box2d2r")
    a = run_plan(tcs, A, B, "box2d2r", 7, engine, "f16", use_graph=False)
    b = run_plan(tcs, A, B, "box2d2r", 7, engine, "f16", use_graph=True)
    np.testing.assert_array_equal(a, b)


def test_sweep_host_one_call_matches_plan(tcs, torch_cuda):
    rng = np.random.default_rng(43)
    A = grid(rng, 100, 120)
    B = normalized_coeffs(rng, "star2d2r")
    for prec, eng in (("f16", "tensor"), ("split", "tensor"), ("f16", "cudacore"), ("f32", "cudacore")):
        a = tcs.sweep_host(A, 5, "star2d2r", B, engine=eng, precision=prec)
        b = run_plan(tcs, A, B, "star2d2r", 5, eng, prec)
        np.testing.assert_array_equal(a, b)
        # a second call of the same shape reuses the cached plan
        c = tcs.sweep_host(A, 5, "star2d2r", B, engine=eng, precision=prec)
        np.testing.assert_array_equal(a, c)


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
@pytest.mark.parametrize("stencil", STENCILS)
def test_drop_in_host_code_matches_gold(tcs, torch_cuda, golden, capfd, engine, stencil):
    """host_code(h_A, h_B, h_C, N, n) with the reference drivers' coefficients,
    against gold on the grid padded with 1.0 (reference semantics)."""
    g = golden(f"gold_{stencil}.npz")
    n = 2 * oracle.RADIUS[stencil] + 1
    for N in (32, 48):
        A = np.ascontiguousarray(g[f"drop_A_{N}"])
        B = np.ascontiguousarray(g[f"drop_B_{N}"])
        C = np.zeros((N, N), np.float32)
        tcs.host_code(A, B, C, N, n, stencil, engine, run_times=3, skip_times=1)
        expect = g[f"drop_C_{N}"].astype(np.float64)
        absC = g[f"drop_absC_{N}"].astype(np.float64)
        bound = absC * (2.0 ** -11 + 2.0 ** -18) + np.abs(expect) * 2.0 ** -11 + 1e-6
        assert np.all(np.abs(C - expect) <= bound)
    out = capfd.readouterr().out
    assert out.count("[Time] Time used:") == 2


def test_config1_star2d1r_1024_zero_halo_10_steps(tcs, torch_cuda):
    """star2d1r, 1024^2 interior + 1-cell zero halo, U[0,1) inputs, 10 steps."""
    rng = np.random.default_rng(1000)
    A = np.zeros((1026, 1026), np.float32)
    A[1:-1, 1:-1] = rng.random((1024, 1024), dtype=np.float32)
    B = normalized_coeffs(rng, "star2d1r")
    A16 = oracle.f32_to_f16(A)
    cc = oracle.f32_to_f16(run_plan(tcs, A, B, "star2d1r", 10, "cudacore", "f16"))
    np.testing.assert_array_equal(cc, oracle.sweep_f16cc(A16, B, "star2d1r", 10))
    tc = run_plan(tcs, A, B, "star2d1r", 10, "tensor", "f16").astype(np.float64)
    ref = oracle.f16_to_f32(oracle.sweep_f16tc(A16, B, "star2d1r", 10))
    assert np.max(np.abs(tc - ref)) <= 10 * f16_ulp(1.0)
    gold = oracle.sweep_f32(A, B, "star2d1r", 10).astype(np.float64)
    assert np.max(np.abs(tc - gold)) <= 11 * f16_ulp(1.0)
