"""Device layout transforms against the oracle's restatement of the reference's
helpers (bit-exact), through the C-ABI."""
import numpy as np
import pytest

import oracle
from helpers import to_plane

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("size,halo", [(16, 16), (48, 16), (37, 3), (100, 0)])
def test_padding_2d(tcs, torch_cuda, size, halo):
    torch = torch_cuda
    rng = np.random.default_rng(size)
    a16 = oracle.f32_to_f16(rng.random((size, size)).astype(np.float32))
    one = int(np.float16(1.0).view(np.uint16))
    d_in = _dev(torch, a16.view(np.int16))
    d_out = torch.empty((size + 2 * halo) ** 2, dtype=torch.int16, device="cuda")
    assert tcs.lib().tcs_padding_2d(d_in.data_ptr(), d_out.data_ptr(), size, halo, one, None) == 0
    got = d_out.cpu().numpy().view(np.uint16).reshape(size + 2 * halo, -1)
    np.testing.assert_array_equal(got, oracle.pad_2d(a16, halo, one))


@pytest.mark.parametrize("ny,nx", [(48, 48), (80, 80), (37, 61), (1, 300)])
def test_brick_and_reverse_layout(tcs, torch_cuda, ny, nx):
    torch = torch_cuda
    rng = np.random.default_rng(ny * 1000 + nx)
    a16 = rng.integers(0, 65535, (ny, nx), dtype=np.uint16)
    d_in = _dev(torch, a16.view(np.int16))
    d_b = torch.empty(tcs.brick_elems(ny, nx), dtype=torch.int16, device="cuda")
    d_r = torch.empty(ny * nx, dtype=torch.int16, device="cuda")
    L = tcs.lib()
    assert L.tcs_brick_layout_2d(d_in.data_ptr(), d_b.data_ptr(), ny, nx, None) == 0
    assert L.tcs_reverse_layout_2d(d_b.data_ptr(), d_r.data_ptr(), ny, nx, None) == 0
    np.testing.assert_array_equal(d_b.cpu().numpy().view(np.uint16), oracle.brick_2d(a16))
    np.testing.assert_array_equal(d_r.cpu().numpy().view(np.uint16).reshape(ny, nx), a16)


@pytest.mark.parametrize("ny,nx,pad", [(32, 32, 16), (45, 70, 2), (64, 17, 0)])
def test_pack_unpack_f16_is_float2half_pad_layout(tcs, torch_cuda, ny, nx, pad):
    """tcs_pack_f16 = array_float2half + padding_2D + the panel layout, with
    every padding cell of the plane written (0)."""
    torch = torch_cuda
    rng = np.random.default_rng(pad + ny)
    A = (rng.standard_normal((ny, nx)) * 10).astype(np.float32)
    d_A = _dev(torch, A)
    nyo, nxo = ny + 2 * pad, nx + 2 * pad
    n = tcs.plane_elems(nyo, nxo)
    assert n == len(to_plane(np.zeros((nyo, nxo), np.uint16)))
    d_b = torch.full((n,), 12345, dtype=torch.int16, device="cuda")
    L = tcs.lib()
    assert L.tcs_pack_f16(d_A.data_ptr(), ny, nx, pad, 1.0, d_b.data_ptr(), None) == 0
    padded = np.ones((nyo, nxo), np.float32)
    padded[pad:pad + ny, pad:pad + nx] = A
    expect = to_plane(oracle.f32_to_f16(padded))
    np.testing.assert_array_equal(d_b.cpu().numpy().view(np.uint16), expect)
    d_out = torch.empty((ny, nx), dtype=torch.float32, device="cuda")
    assert L.tcs_unpack_f16(d_b.data_ptr(), ny, nx, pad, d_out.data_ptr(), None) == 0
    np.testing.assert_array_equal(d_out.cpu().numpy(), oracle.f16_to_f32(oracle.f32_to_f16(A)))


def test_pack_unpack_f32_and_split(tcs, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(9)
    ny, nx, pad = 50, 77, 1
    A = rng.uniform(-1, 1, (ny, nx)).astype(np.float32)
    d_A = _dev(torch, A)
    L = tcs.lib()
    n = tcs.plane_elems(ny + 2, nx + 2, "f32")
    d_f = torch.empty(n, dtype=torch.float32, device="cuda")
    assert L.tcs_pack_f32(d_A.data_ptr(), ny, nx, pad, 0.0, d_f.data_ptr(), None) == 0
    d_o = torch.empty((ny, nx), dtype=torch.float32, device="cuda")
    assert L.tcs_unpack_f32(d_f.data_ptr(), ny, nx, pad, d_o.data_ptr(), None) == 0
    np.testing.assert_array_equal(d_o.cpu().numpy(), A)
    padded32 = np.zeros((ny + 2, nx + 2), np.float32)
    padded32[1:-1, 1:-1] = A
    np.testing.assert_array_equal(d_f.cpu().numpy(), to_plane(padded32, cpp=4))
    n = tcs.plane_elems(ny + 2, nx + 2, "split")
    d_h = torch.empty(n, dtype=torch.int16, device="cuda")
    d_l = torch.empty(n, dtype=torch.int16, device="cuda")
    import ctypes
    mx = ctypes.c_float(0.0)
    assert L.tcs_max_abs_f32(d_A.data_ptr(), ny * nx, ctypes.byref(mx), None) == 0
    assert mx.value == np.max(np.abs(A))
    e = L.tcs_split_scale_exp(mx.value)
    assert e == oracle.split_scale_exp(A)
    assert L.tcs_pack_split(d_A.data_ptr(), ny, nx, pad, 0.0, e, d_h.data_ptr(), d_l.data_ptr(), None) == 0
    padded = np.zeros((ny + 2, nx + 2), np.float64)
    padded[1:-1, 1:-1] = A
    hi, lo = oracle.split(padded, e)
    np.testing.assert_array_equal(d_h.cpu().numpy().view(np.uint16), to_plane(hi))
    np.testing.assert_array_equal(d_l.cpu().numpy().view(np.uint16), to_plane(lo))
    assert L.tcs_unpack_split(d_h.data_ptr(), d_l.data_ptr(), ny, nx, pad, e, d_o.data_ptr(), None) == 0
    back = d_o.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(back - A)) <= 2.0 ** (e - 23)
