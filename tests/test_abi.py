"""The C-ABI library: builds, loads without a GPU, exports every declared
symbol, and its host-only entry points behave (CPU only)."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT, STENCILS


def declared_functions():
    src = open(os.path.join(ROOT, "include", "tcs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?!typedef)[a-z_ ]+[\s\*]+(\w+)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "return")))


def test_header_declares_the_drop_in_and_extended_api():
    names = declared_functions()
    for must in ["host_star2d1r", "host_box2d2r", "host_cc_star2d2r", "tcs_host_code",
                 "tcs_sweep_step", "tcs_plan_create", "tcs_plan_run", "tcs_sweep_host",
                 "tcs_pack_f16", "tcs_brick_layout_2d", "tcs_init_coe_box"]:
        assert must in names


def test_library_exports_every_declared_symbol(tcs):
    L = ctypes.CDLL(tcs.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the Python mirror binds every one of them
    assert set(declared_functions()) <= set(tcs.SIGNATURES)


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
@pytest.mark.parametrize("stencil", STENCILS)
def test_variant_shims_export_host_code(tcs, engine, stencil):
    path = os.path.join(os.path.dirname(tcs.LIB_PATH), f"libtcs_host_{engine}_{stencil}.so")
    L = ctypes.CDLL(path)
    assert hasattr(L, "host_code")


def test_status_and_geometry_helpers(tcs):
    L = tcs.lib()
    assert L.tcs_status_string(0) == b"ok"
    assert [L.tcs_stencil_radius(i) for i in range(4)] == [1, 2, 1, 2]
    assert L.tcs_stencil_radius(9) == -1
    assert L.tcs_brick_elems(8196, 8196) == 513 * 513 * 256
    assert L.tcs_brick_elems(16, 17) == 2 * 256


def test_invalid_arguments_are_rejected_before_any_device_work(tcs):
    B = np.ones((5, 5), np.float32)
    with pytest.raises(tcs.TcsError) as e:
        tcs.sweep_step(1 << 20, 2 << 20, 100, 100, "box2d2r", B, rect=(0, 100, 0, 100))
    assert e.value.status == tcs.TCS_ERR_INVALID
    with pytest.raises(tcs.TcsError) as e:
        tcs.sweep_step(1 << 20, 2 << 20, 100, 100, "box2d2r", B, precision="f32")
    assert e.value.status == tcs.TCS_ERR_UNSUPPORTED
    with pytest.raises(tcs.TcsError) as e:
        tcs.sweep_step(1 << 20, 1 << 20, 100, 100, "box2d2r", B)
    assert e.value.status == tcs.TCS_ERR_INVALID
    with pytest.raises(tcs.TcsError):
        tcs.host_code(np.zeros((20, 20), np.float32), np.zeros((3, 3), np.float32),
                      np.zeros((20, 20), np.float32), 20, 3, "star2d1r")
    with pytest.raises(tcs.TcsError):  # n does not match the stencil
        tcs.host_code(np.zeros((32, 32), np.float32), np.zeros((3, 3), np.float32),
                      np.zeros((32, 32), np.float32), 32, 3, "box2d2r")
    assert tcs.lib().tcs_plan_set_multistep(None, 1) == tcs.TCS_ERR_INVALID


@pytest.mark.parametrize("stencil", STENCILS)
def test_band_builders_bit_exact(tcs, golden, stencil):
    """tcs_init_coe_* (host) against the reference's init_coe outputs."""
    g = golden("init_coe.npz")
    L = tcs.lib()
    n = 2 * oracle.RADIUS[stencil] + 1
    for tag in ("refB", "randB"):
        B16 = np.ascontiguousarray(g[f"{stencil}_{tag}_B16"])
        if stencil.startswith("star"):
            a = np.zeros(256, np.uint16)
            b = np.zeros(256, np.uint16)
            assert L.tcs_init_coe_star(B16.ctypes.data, n, a.ctypes.data, b.ctypes.data) == 0
            np.testing.assert_array_equal(a, g[f"{stencil}_{tag}_a"])
            np.testing.assert_array_equal(b, g[f"{stencil}_{tag}_b"])
        else:
            coe = np.zeros(256 * n, np.uint16)
            assert L.tcs_init_coe_box(B16.ctypes.data, n, coe.ctypes.data) == 0
            np.testing.assert_array_equal(coe, g[f"{stencil}_{tag}_coe"])


def test_reference_driver_links_against_the_shim(tcs, tmp_path):
    """common/main_1r.cu and main_2r.cu of the reference, unchanged, link with the
    per-variant host_code libraries (where the reference sources exist)."""
    ref = oracle.ref_src_dir()
    if not os.path.isdir(os.path.join(ref, "common")):
        pytest.skip("reference sources not present")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    libdir = os.path.dirname(tcs.LIB_PATH)
    for main, st in (("main_1r.cu", "star2d1r"), ("main_2r.cu", "box2d2r")):
        exe = tmp_path / f"drv_{st}"
        cmd = [nvcc, "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-DMESH_SIZE=64",
               "-o", str(exe), os.path.join(ref, "common", main),
               os.path.join(ref, "common", f"gold_{st}.cpp"), "-L", libdir,
               f"-ltcs_host_tensor_{st}", f"-Xlinker", f"-rpath,{libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert exe.exists()


def test_split_rejects_expanding_stencils(tcs):
    """Split storage needs sum |c| <= 1; the check runs before any device work."""
    B = np.full((3, 3), 0.2, np.float32)  # sum 1.8
    with pytest.raises(tcs.TcsError) as e:
        tcs.sweep_step(1 << 20, 2 << 20, 64, 64, "box2d1r", B, precision="split",
                       d_in_lo=3 << 20, d_out_lo=4 << 20)
    assert e.value.status == tcs.TCS_ERR_UNSUPPORTED


def test_batch_add_validates_before_any_device_work(tcs):
    """Batches take tensor-engine FP16/split grids; every check runs in
    tcs_batch_add, before the batch touches the device."""
    b = tcs.Batch()
    c = np.full((3, 3), 1.0 / 9.0, np.float32)
    assert b.add(64, 64, "box2d1r", c, 3) == 0
    assert b.add(200, 31, "box2d1r", c, 0, "split") == 1
    with pytest.raises(tcs.TcsError) as e:
        b.add(64, 64, "box2d1r", np.full((3, 3), 0.2, np.float32), 1, "split")
    assert e.value.status == tcs.TCS_ERR_UNSUPPORTED
    with pytest.raises(tcs.TcsError) as e:
        b.add(64, 64, "box2d1r", c, 1, "f32")
    assert e.value.status == tcs.TCS_ERR_UNSUPPORTED
    with pytest.raises(tcs.TcsError) as e:
        b.add(2, 64, "box2d1r", c, 1)
    assert e.value.status == tcs.TCS_ERR_INVALID
    with pytest.raises(tcs.TcsError):
        b.add(64, 64, "box2d1r", c, -1)
    for bad in [lambda: b.set_gate(2, 0x1000, 1), lambda: b.set_gate(-1, 0x1000, 1),
                lambda: b.set_wait_limit(0.0), lambda: b.set_wait_limit(-1.0),
                lambda: b.set_wait_limit(float("nan"))]:
        with pytest.raises(tcs.TcsError) as e:
            bad()
        assert e.value.status == tcs.TCS_ERR_INVALID
    b.set_gate(0, 0x1000, 1)
    b.set_gate(0, None, 0)
    b.set_wait_limit(0.25)
    b.close()


def test_server_config_is_validated_before_any_device_work(tcs):
    import ctypes

    h = ctypes.c_void_p()
    for cfg in [tcs.ServerConfig(0, 0, 0), tcs.ServerConfig(1 << 20, -1, 0),
                tcs.ServerConfig(1 << 20, 0, -2)]:
        assert tcs.lib().tcs_server_create(ctypes.byref(cfg), ctypes.byref(h)) == tcs.TCS_ERR_INVALID


def test_pipe_arguments_are_checked_before_device_work(tcs):
    import ctypes

    L = tcs.lib()
    assert L.tcs_pipe_submit(None, None, None, 1) == tcs.TCS_ERR_INVALID
    assert L.tcs_pipe_wait(None) == tcs.TCS_ERR_INVALID
    assert L.tcs_pipe_destroy(None) == tcs.TCS_OK
    h = ctypes.c_void_p()
    assert L.tcs_pipe_create(None, ctypes.byref(h)) == tcs.TCS_ERR_INVALID
