"""FP64 drift check (tcs_drift_*): the device FP64 shadow is the oracle's
FP64 restatement of gold bit for bit, its comparison is right, and the split
form stays within 1e-6 of it over the split configuration's 200 steps."""
import numpy as np
import pytest

import oracle
from helpers import RADIUS, normalized_coeffs

pytestmark = pytest.mark.gpu


def _field(rng, ny, nx):
    """U[-1,1) plus sin(2 pi x) sin(2 pi y) (the split configuration's input)."""
    yy, xx = np.meshgrid(np.arange(ny) / ny, np.arange(nx) / nx, indexing="ij")
    return (rng.uniform(-1, 1, (ny, nx)) + np.sin(2 * np.pi * xx) * np.sin(2 * np.pi * yy)).astype(np.float32)


@pytest.mark.parametrize("stencil", list(RADIUS))
def test_shadow_is_the_fp64_oracle_bit_for_bit(tcs, torch_cuda, stencil):
    rng = np.random.default_rng(81)
    ny, nx = 67, 130
    A = _field(rng, ny, nx)
    B = normalized_coeffs(rng, stencil)
    rect = (3, 60, 2, 127)
    d = tcs.Drift(ny, nx, stencil, B, rect=rect)
    d.upload(A)
    d.run(7)
    got = d.download()
    expect = oracle.sweep_f64(A.astype(np.float64), B.astype(np.float64), stencil, 7, rect)
    np.testing.assert_array_equal(got, expect)
    d.close()


def test_compare_measures_the_difference(tcs, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(82)
    A = _field(rng, 90, 70)
    d = tcs.Drift(90, 70, "box2d1r", normalized_coeffs(rng, "box2d1r"))
    d.upload(A)
    a = torch.from_numpy(A).cuda()
    rel, mx = d.compare(a)
    assert rel == 0.0 and mx == 0.0
    b = a.clone()
    b[10, 11] += 0.25
    rel, mx = d.compare(b)
    assert mx == 0.25
    assert abs(rel - 0.25 / np.linalg.norm(A.astype(np.float64))) < 1e-12
    d.close()


@pytest.mark.parametrize("stencil", ["box2d1r", "star2d2r"])
def test_split_stays_within_1e6_of_the_shadow_for_200_steps(tcs, torch_cuda, stencil):
    """The split configuration's error bar with the drift check every 50 steps,
    at 1026^2 (1024^2 interior + 1 halo)."""
    torch = torch_cuda
    rng = np.random.default_rng(83)
    n = 1026 if RADIUS[stencil] == 1 else 1028
    A = np.zeros((n, n), np.float32)
    r = RADIUS[stencil]
    A[r:-r, r:-r] = _field(rng, n - 2 * r, n - 2 * r)
    B = normalized_coeffs(rng, stencil)
    p = tcs.Plan(n, n, stencil, B, engine="tensor", precision="split")
    d = tcs.Drift(n, n, stencil, B)
    p.upload(A)
    d.upload(A)
    out = torch.empty((n, n), dtype=torch.float32, device="cuda")
    errs = []
    for _ in range(4):
        p.run(50)
        d.run(50)
        p.download(out)
        errs.append(d.compare(out)[0])
    p.close()
    d.close()
    assert max(errs) <= 1e-6, errs
    assert tcs.device_error() == 0
