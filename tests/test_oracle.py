"""The oracle pinned against the reference's own outputs (CPU only).

The golden fixtures were produced by the reference's unchanged gold_*.cpp and
layout16 helpers (tests/golden/make_golden.py); the in-repo restatement must
reproduce them bit for bit."""
import numpy as np
import pytest

import oracle
from conftest import STENCILS


@pytest.mark.parametrize("stencil", STENCILS)
def test_gold_step_matches_reference_fixtures(golden, stencil):
    g = golden(f"gold_{stencil}.npz")
    for N in (16, 37, 64):
        for tag in ("refB", "normB"):
            A, B = g[f"A_{N}_{tag}"], g[f"B_{N}_{tag}"]
            out = oracle.gold_step(A, B, stencil, g[f"Cin_{N}_{tag}"])
            np.testing.assert_array_equal(out.view(np.uint32), g[f"Cout_{N}_{tag}"].view(np.uint32))


@pytest.mark.parametrize("stencil", STENCILS)
def test_gold_sweep_matches_reference_fixtures(golden, stencil):
    g = golden(f"gold_{stencil}.npz")
    for N in (16, 37, 64):
        out = oracle.sweep_f32(g[f"A_{N}_normB"], g[f"B_{N}_normB"], stencil, 5)
        np.testing.assert_array_equal(out.view(np.uint32), g[f"sweep5_{N}"].view(np.uint32))


@pytest.mark.parametrize("stencil", STENCILS)
def test_gold_loop_shape_port_matches_reference_fixtures(golden, stencil):
    """The port in gold's own loop shape (timed as the CPU baseline) gives the
    reference's bits, alone and as the threaded row-band ping-pong."""
    g = golden(f"gold_{stencil}.npz")
    for N in (16, 37, 64):
        for tag in ("refB", "normB"):
            A, B = g[f"A_{N}_{tag}"], g[f"B_{N}_{tag}"]
            out = oracle.gold_loop_step(A, B, stencil, g[f"Cin_{N}_{tag}"])
            np.testing.assert_array_equal(out.view(np.uint32), g[f"Cout_{N}_{tag}"].view(np.uint32))
        for threads in (1, 3, 8):
            for shape in (True, False):
                _, out = oracle.gold_bench_bands(g[f"A_{N}_normB"], g[f"B_{N}_normB"], stencil, 5,
                                                 threads, loop_shape=shape, want_out=True)
                np.testing.assert_array_equal(out.view(np.uint32), g[f"sweep5_{N}"].view(np.uint32))


def test_layout_helpers_match_reference_fixtures(golden):
    g = golden("layout16.npz")
    one = int(np.float16(1.0).view(np.uint16))
    for N in (16, 48):
        p = oracle.pad_2d(g[f"in_{N}"], 16, one)
        np.testing.assert_array_equal(p, g[f"padded_{N}"])
        b = oracle.brick_2d(p)
        np.testing.assert_array_equal(b, g[f"bricks_{N}"])
        np.testing.assert_array_equal(oracle.unbrick_2d(b, N + 32, N + 32), g[f"reversed_{N}"])


@pytest.mark.parametrize("stencil", STENCILS)
def test_init_coe_matches_reference_fixtures(golden, stencil):
    g = golden("init_coe.npz")
    n = 2 * oracle.RADIUS[stencil] + 1
    for tag in ("refB", "randB"):
        B16 = g[f"{stencil}_{tag}_B16"]
        if stencil.startswith("star"):
            a, b = oracle.init_coe_star(B16, n)
            np.testing.assert_array_equal(a, g[f"{stencil}_{tag}_a"])
            np.testing.assert_array_equal(b, g[f"{stencil}_{tag}_b"])
        else:
            np.testing.assert_array_equal(oracle.init_coe_box(B16, n), g[f"{stencil}_{tag}_coe"])


def test_f16_conversion_is_ieee_rne():
    rng = np.random.default_rng(7)
    x = np.concatenate([
        (rng.standard_normal(200000) * 300).astype(np.float32),
        (rng.standard_normal(20000) * 1e-5).astype(np.float32),
        np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e9, 2.0 ** -24, 2.0 ** -25,
                  3 * 2.0 ** -26, 6.1035156e-05, 6.0975552e-05], np.float32)])
    with np.errstate(over="ignore"):
        expect = x.astype(np.float16).view(np.uint16)
    np.testing.assert_array_equal(oracle.f32_to_f16(x), expect)
    h = expect
    np.testing.assert_array_equal(oracle.f16_to_f32(h), h.view(np.float16).astype(np.float32))


def test_split_round_trip_precision():
    """Fixed-point hi (multiples of 2^-11) + FP16 lo: absolute error <= 2^-23
    of the scaled value, i.e. FP32-level for the largest values."""
    rng = np.random.default_rng(3)
    for scale in (1.0, 37.5, 1e-3):
        x = rng.uniform(-1, 1, 100000) * scale
        e = oracle.split_scale_exp(x)
        assert np.max(np.abs(x)) * 2.0 ** -e <= 1.0
        hi, lo = oracle.split(x, e)
        h = oracle.f16_to_f32(hi).astype(np.float64)
        assert np.all(np.round(h * 2048) == h * 2048)  # hi is fixed point
        back = oracle.join(hi, lo, e)
        assert np.max(np.abs(back - x)) <= 2.0 ** (e - 23)


@pytest.mark.parametrize("stencil", STENCILS)
def test_arithmetic_contracts_agree(stencil):
    """The FP16 contracts differ from each other by at most one FP16 step."""
    rng = np.random.default_rng(11)
    n = 2 * oracle.RADIUS[stencil] + 1
    B = rng.random((n, n)).astype(np.float32)
    B /= B.sum()
    A = rng.uniform(-1, 1, (40, 53)).astype(np.float32)
    A16 = oracle.f32_to_f16(A)
    cc = oracle.f16_to_f32(oracle.sweep_f16cc(A16, B, stencil, 1)).astype(np.float64)
    tc = oracle.f16_to_f32(oracle.sweep_f16tc(A16, B, stencil, 1)).astype(np.float64)
    gold = oracle.sweep_f32(A, B, stencil, 1).astype(np.float64)
    assert np.max(np.abs(cc - tc)) <= 2.0 ** -9
    assert np.max(np.abs(cc - gold)) <= 2.0 ** -9


def test_reference_build_matches_restatement_on_random_cases():
    """Direct comparison with the compiled reference, where it was built."""
    R = oracle.Ref()
    if not R.available():
        pytest.skip("reference not compiled here (oracle/_ref)")
    rng = np.random.default_rng(5)
    for st in STENCILS:
        n = 2 * oracle.RADIUS[st] + 1
        for N in (5, 17, 100):
            A = rng.uniform(-3, 3, (N, N)).astype(np.float32)
            B = rng.uniform(-2, 2, (n, n)).astype(np.float32)
            C = rng.random((N, N)).astype(np.float32)
            np.testing.assert_array_equal(R.gold(A, B, st, C).view(np.uint32),
                                          oracle.gold_step(A, B, st, C).view(np.uint32))


def test_error_metrics_match_the_reference(golden):
    """checkError2D / checkRelativeError2D (common/common.hpp:38-92), run from
    the reference header by tests/golden/make_golden.py: the same RMS results
    bit for bit, the same reported cells in the same order, the same final
    maximum (as the reference prints it, %e) and its cell."""
    g = golden("check_error.npz")
    cases = sorted({k.split("_")[0] for k in g.files})
    assert len(cases) == 5
    for c in cases:
        N, region = int(g[f"{c}_N"]), [int(v) for v in g[f"{c}_region"]]
        for part, relative, key in (("abs", False, "rms"), ("rel", True, "rel")):
            r = oracle.check_error_2d(N, g[f"{c}_out"], g[f"{c}_ref"], *region, relative=relative)
            assert r["rms"] == float(g[f"{c}_{key}"]), (c, part)
            assert r["reported"] == [tuple(x) for x in g[f"{c}_{part}_reported"].tolist()], (c, part)
            line = g[f"{c}_{part}_max_line"]
            if line.size:  # printed only when the maximum's cell is not (0, 0)
                assert "%e" % r["max_error"] == str(line[0]), (c, part)
                assert r["max_at"] == tuple(g[f"{c}_{part}_max_at"].tolist()), (c, part)
            else:
                assert r["max_at"] == (0, 0), (c, part)
    # the fixtures cover messages, none, both signs and the MIN_NUMBER branch
    assert any(g[f"{c}_rel_reported"].size for c in cases)
    assert any(not g[f"{c}_abs_reported"].size for c in cases)
    assert any(not g[f"{c}_abs_max_line"].size and g[f"{c}_abs_reported"].size for c in cases)


def test_split_scale_rule_follows_the_field_and_its_fixed_border():
    """The oracle's per-step split scale: E_t follows the largest value of
    the update rectangle, or of the fixed border where that is larger (the
    border keeps its values, so it pins E).  A decaying zero-border field's
    exponent comes down and the run stays within 1e-6 of FP64; with a 0.75
    border around the same field it stays at the input's."""
    from helpers import normalized_coeffs
    rng = np.random.default_rng(5)
    B = normalized_coeffs(rng, "box2d2r")
    noise = rng.uniform(-1, 1, (76, 86))
    for border, expect_drop in ((0.0, True), (0.75, False)):
        A = np.full((80, 90), border, np.float32)
        A[2:-2, 2:-2] = noise
        e0 = oracle.split_scale_exp(A)
        hi, lo = oracle.split(A.astype(np.float64), e0)
        h, l, e = oracle.sweep_split(hi, lo, B, "box2d2r", 60, scale_exp=e0)
        assert (e < e0) == expect_drop, (border, e0, e)
        got = oracle.join(h, l, e)
        f64 = oracle.sweep_f64(A.astype(np.float64), B.astype(np.float64), "box2d2r", 60)
        assert np.linalg.norm(got - f64) / np.linalg.norm(f64) <= 1e-6
        # the border keeps its values
        np.testing.assert_allclose(got[:2], A[:2], rtol=0, atol=2.0 ** (e0 - 23))
