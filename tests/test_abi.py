"""The C-ABI library: it builds for sm_103a, exports every function include/sphgpu.h declares,
and returns clean status codes on the error paths that need no GPU."""
import ctypes
import subprocess

import pytest


@pytest.fixture(scope="module")
def lib():
    from sphcode_gb300 import build, sphgpu
    build.build_library()
    return sphgpu.library()


def test_exports_every_declared_function(lib):
    from sphcode_gb300 import build, sphgpu
    declared = sphgpu.header_functions()
    assert len(declared) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    for f in declared:
        getattr(lib, f)


def test_binding_covers_header():
    from sphcode_gb300 import sphgpu
    assert set(sphgpu.header_functions()) == set(sphgpu._SIGS)


def test_invalid_arguments_rejected(lib):
    from sphcode_gb300 import sphgpu
    from sphcode_gb300.params import CParams, SPHParameters
    p = SPHParameters(dim=1, kernel="wendland", gamma=1.4)
    h = ctypes.c_void_p()
    # Wendland C4 is undefined in 1D (include/kernel/wendland_kernel.hpp:15-27)
    rc = lib.sphgpu_create(ctypes.byref(p.to_c(CParams)), 1, 100, 0, ctypes.byref(h))
    assert rc == 1 and not h.value
    assert b"Wendland" in lib.sphgpu_last_error(None)
    p = SPHParameters(dim=3, gamma=1.4)
    assert lib.sphgpu_create(ctypes.byref(p.to_c(CParams)), 3, 0, 0, ctypes.byref(h)) == 1
    assert lib.sphgpu_create(ctypes.byref(p.to_c(CParams)), 4, 10, 0, ctypes.byref(h)) == 1
    assert lib.sphgpu_create(ctypes.byref(p.to_c(CParams)), 3, 10, 7, ctypes.byref(h)) == 1
    p = SPHParameters(dim=3, gamma=1.4, max_level=30)   # 90 key bits
    assert lib.sphgpu_create(ctypes.byref(p.to_c(CParams)), 3, 10, 0, ctypes.byref(h)) == 1
    # NULL context
    assert lib.sphgpu_step(None, 1) == 1
    assert lib.sphgpu_destroy(None) == 0


def test_no_device_is_reported(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sphcode_gb300 import sphgpu
    from sphcode_gb300.params import SPHParameters
    from sphcode_gb300 import ics
    p, f = ics.sod(20, 5)
    with pytest.raises(sphgpu.SphGpuError) as e:
        sphgpu.GpuSimulation(p, f)
    assert e.value.code == 7
