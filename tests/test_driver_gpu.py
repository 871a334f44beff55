"""The per-variant host_code libraries run under a driver shaped like the
reference's common/main_1r.cu / main_2r.cu (tests/driver/host_code_main.cpp:
host_code declared as common/main_1r.cu:7 declares it, init_B's coefficients,
one call on a MESH_SIZE^2 grid).  Each run prints the reference's
"[Time] Time used: %f ms" line and its h_C matches gold on the grid padded by
16 cells of 1.0 (the reference's semantics), for both engines and all four
stencils."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT, STENCILS

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(ROOT, "tests", "driver", "host_code_main.cpp")


@pytest.mark.parametrize("engine", ["tensor", "cudacore"])
@pytest.mark.parametrize("stencil", STENCILS)
def test_reference_shaped_driver_calls_host_code(tcs, torch_cuda, golden, tmp_path, engine,
                                                 stencil):
    cxx = shutil.which("g++") or shutil.which("c++")
    assert cxx, "a C++ compiler is needed to build the driver"
    libdir = os.path.dirname(tcs.LIB_PATH)
    n = 2 * oracle.RADIUS[stencil] + 1
    g = golden(f"gold_{stencil}.npz")
    for N in (32, 48):
        exe = tmp_path / f"main_{engine}_{stencil}_{N}"
        r = subprocess.run([cxx, "-O2", f"-DMESH_SIZE={N}", f"-DSTENCIL_SIZE={n}", "-o", str(exe),
                            DRIVER, "-L", libdir, f"-ltcs_host_{engine}_{stencil}",
                            f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        A = np.ascontiguousarray(g[f"drop_A_{N}"], np.float32)
        np.testing.assert_array_equal(g[f"drop_B_{N}"].reshape(-1),
                                      np.where(np.arange(n * n) == n * n // 2,
                                               -40.0 if n == 3 else -290.0, np.arange(n * n)))
        a_path, c_path = tmp_path / "A.f32", tmp_path / "C.f32"
        A.tofile(a_path)
        r = subprocess.run([str(exe), str(a_path), str(c_path)], capture_output=True, text=True,
                           timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        times = re.findall(r"\[Time\] Time used: ([0-9.]+) ms", r.stdout)
        assert len(times) == 1 and float(times[0]) > 0, r.stdout
        C = np.fromfile(c_path, np.float32).reshape(N, N).astype(np.float64)
        expect = g[f"drop_C_{N}"].astype(np.float64)
        absC = g[f"drop_absC_{N}"].astype(np.float64)
        # FP16 storage of the inputs and the result, FP32 accumulation
        bound = absC * (2.0 ** -11 + 2.0 ** -18) + np.abs(expect) * 2.0 ** -11 + 1e-6
        assert np.all(np.abs(C - expect) <= bound), (N, float(np.max(np.abs(C - expect) - bound)))
