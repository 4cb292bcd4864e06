"""The reference-layout particle transfer (sphgpu_upload_aos / sphgpu_download_aos) on the
SPHParticle record (include/particle.hpp:8-33), from pageable and from page-locked host memory:
same fields as the SoA accessors, caller order, and the record members outside the layout left
untouched."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

NAMES = ("pos", "vel", "vel_p", "acc", "mass", "dens", "pres", "ene", "ene_p", "dene", "sml", "sound",
         "balsara", "alpha", "gradh", "phi")


def particle_dtype(D):
    fields = [("pos", "f8", (D,)), ("vel", "f8", (D,)), ("vel_p", "f8", (D,)), ("acc", "f8", (D,))]
    fields += [(n, "f8") for n in NAMES[4:]]
    fields += [("id", "i4"), ("neighbor", "i4"), ("next", "u8")]
    return np.dtype(fields, align=True)


def layout(dt):
    from sphcode_gb300 import sphgpu
    lay = sphgpu.AosLayout()
    lay.stride = dt.itemsize
    for name in NAMES + ("neighbor",):
        setattr(lay, name, dt.fields[name][1])
    return lay


def host_buffer(dt, n, pinned):
    if not pinned:
        return None, np.zeros(n, dtype=dt)
    import torch
    t = torch.zeros(n * dt.itemsize, dtype=torch.uint8, pin_memory=True)
    return t, t.numpy().view(dt)


@pytest.mark.parametrize("pinned", [False, True])
def test_aos_round_trip(gpu_lib, pinned):
    import ctypes
    from sphcode_gb300 import ics, sphgpu
    p, f = ics.gresho(32)
    n = f["mass"].size
    dt = particle_dtype(2)
    lay = layout(dt)
    keep, rec = host_buffer(dt, n, pinned)
    rec["id"] = np.arange(n)
    rec["next"] = 0xABCDEF0123456789   # outside the layout: must survive both directions
    with sphgpu.GpuSimulation(p, f, precision="fp64") as sim:
        sim.initialize()
        sim.step(2)
        lib = sim.lib
        assert lib.sphgpu_download_aos(sim._h, rec.ctypes.data, ctypes.byref(lay)) == 0
        for name in ("pos", "vel", "acc", "dens", "pres", "ene", "sml", "dene", "alpha", "balsara"):
            got = rec[name]
            assert np.array_equal(got.reshape(sim.get(name).shape), sim.get(name)), name
        assert np.array_equal(rec["neighbor"], sim.get("neighbor").astype(np.int32))
        assert np.all(rec["next"] == 0xABCDEF0123456789)
        # modify on the host, upload, read back through the SoA accessors
        rec["vel"] *= 0.5
        rec["ene"] += 1.0
        assert lib.sphgpu_upload_aos(sim._h, rec.ctypes.data, ctypes.byref(lay)) == 0
        assert rel_err(sim.get("vel"), rec["vel"]) == 0.0
        assert rel_err(sim.get("ene"), rec["ene"]) == 0.0
        assert np.all(rec["next"] == 0xABCDEF0123456789)
        sim.step(1)
    del keep


def test_download_reuses_uploaded_records(gpu_lib):
    """Knob 19: the download takes the members outside the layout from the last upload."""
    import ctypes
    from sphcode_gb300 import ics, sphgpu
    p, f = ics.gresho(32)
    n = f["mass"].size
    dt = particle_dtype(2)
    lay = layout(dt)
    rec = np.zeros(n, dtype=dt)
    rec["id"] = np.arange(n)
    rec["next"] = 7
    with sphgpu.GpuSimulation(p, f, precision="fp64") as sim:
        sim.set_tuning("aos_reuse", 1)
        sim.initialize()
        assert sim.lib.sphgpu_download_aos(sim._h, rec.ctypes.data, ctypes.byref(lay)) == 0
        assert sim.lib.sphgpu_upload_aos(sim._h, rec.ctypes.data, ctypes.byref(lay)) == 0
        sim.step(1)
        out = np.zeros(n, dtype=dt)      # a different buffer: its own members are not read
        assert sim.lib.sphgpu_download_aos(sim._h, out.ctypes.data, ctypes.byref(lay)) == 0
        assert np.all(out["next"] == 7) and np.array_equal(out["id"], np.arange(n))
        assert np.array_equal(out["dens"], sim.get("dens"))
