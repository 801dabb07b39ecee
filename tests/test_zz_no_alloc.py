"""fluid_gb300_step_noalloc: one timestep that allocates no device memory.

It exists for callers that cannot allocate device memory where they step the
fluid (an application that owns every device allocation through its own pool,
a frame-time loop where an allocation would stall, a plugin that must not grow
the process's footprint). Its scratch is a fixed array inside the library, so
what needs proving is that it computes the same step as the ordinary entry
point and as the oracle, and that it refuses work beyond its fixed limits
cleanly: two calls in a row are compared bit for bit with
fluid_gb300_cuda_step and with the oracle on the same input (the tolerance
every parity test here uses); a call over any of the three limits (particles,
list entries, grid cells) returns FLUID_ERR_CAPACITY with the caller's arrays
and time untouched, and the next normal call is still exact. This file is
collected last so a failure here cannot hide earlier results.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLUID_ERR_CAPACITY = 3
MAX_PARTICLES = 8192
MAX_NEIGHBOR_SLOTS = 1 << 20
MAX_CELLS = 1 << 18


def _ptrs(t):
    base = t.data_ptr()
    return [ctypes.c_void_p(base + k * t.stride(0) * 4) for k in range(3)]


def _device_arrays(sc):
    import torch

    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(np.ascontiguousarray(sc.pos)).to(dev)
    vel = torch.from_numpy(np.ascontiguousarray(sc.vel)).to(dev)
    torch.cuda.synchronize(dev)
    return dev, pos, vel


def _call(cuda_lib, params, count, pos, vel, t):
    return cuda_lib.fluid_gb300_step_noalloc(ctypes.byref(params), count, *_ptrs(pos), *_ptrs(vel),
                                             ctypes.byref(t), None)


def _normal_call_is_exact(cuda_lib, oracle_lib):
    """One call on the 4,096-particle dam break (all three flags) against
    fluid_gb300_cuda_step and the oracle, bit for bit."""
    import torch

    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import cuda_step

    sc = scenes.dam_break(16, seed=0, flags=True)
    dev, pos, vel = _device_arrays(sc)
    t = ctypes.c_float(0.0)
    assert _call(cuda_lib, sc.params, sc.count, pos, vel, t) == 0
    torch.cuda.synchronize(dev)
    hp, hv = sc.pos.copy(), sc.vel.copy()
    cuda_step(sc.params, hp, hv, 0.0)
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1)
    np.testing.assert_array_equal(pos.cpu().numpy(), hp)
    np.testing.assert_array_equal(vel.cpu().numpy(), hv)
    np.testing.assert_array_equal(pos.cpu().numpy(), ref["pos"])
    np.testing.assert_array_equal(vel.cpu().numpy(), ref["vel"])
    assert t.value == np.float32(ref["time"])


def test_noalloc_step_matches_stateless_step_and_oracle_twice(cuda_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import cuda_step

    sc = scenes.dam_break(16, seed=0, flags=True)  # 4,096 particles, all three flags
    assert sc.count <= MAX_PARTICLES
    dev, pos, vel = _device_arrays(sc)
    host_pos, host_vel = sc.pos.copy(), sc.vel.copy()
    ref = oracle_lib.Oracle()
    ox, ov, ot = sc.pos.copy(), sc.vel.copy(), 0.0
    t_dev = ctypes.c_float(0.0)
    t_host = 0.0
    for call in range(2):
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = _call(cuda_lib, sc.params, sc.count, pos, vel, t_dev)
        torch.cuda.synchronize(dev)
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert rc == 0, rc
        if call == 1:
            assert free_after == free_before  # the call itself took no device memory
        t_host = cuda_step(sc.params, host_pos, host_vel, t_host)
        r = ref.run(sc.params, ox, ov, ot, 1)
        ox, ov, ot = r["pos"], r["vel"], r["time"]
        got_p, got_v = pos.cpu().numpy(), vel.cpu().numpy()
        np.testing.assert_array_equal(got_p, host_pos)
        np.testing.assert_array_equal(got_v, host_vel)
        np.testing.assert_array_equal(got_p, ox)
        np.testing.assert_array_equal(got_v, ov)
        assert t_dev.value == np.float32(t_host) == np.float32(ot)


def test_noalloc_step_refuses_oversized_input(cuda_lib):
    torch = pytest.importorskip("torch")
    from fluidsimulator_gb300 import scenes

    sc = scenes.dam_break(21, seed=1)  # 9,261 particles > the 8,192 limit
    assert sc.count > MAX_PARTICLES
    dev, pos, vel = _device_arrays(sc)
    t = ctypes.c_float(0.0)
    rc = _call(cuda_lib, sc.params, sc.count, pos, vel, t)
    torch.cuda.synchronize(dev)
    assert rc == FLUID_ERR_CAPACITY
    np.testing.assert_array_equal(pos.cpu().numpy(), sc.pos)
    assert t.value == 0.0


def _compact_cluster():
    """8,000 particles at a quarter of h apart: ~200-270 neighbours each, so
    the lists need about twice the 2^20 entries of the fixed scratch."""
    from fluidsimulator_gb300 import scenes

    sc = scenes.dam_break(20, seed=2, flags=True)
    h = np.float32(sc.params.h)
    lo = sc.pos.min(axis=1, keepdims=True)
    sc.pos[:] = (lo + (sc.pos - lo) * (np.float32(0.25) * h / np.float32(0.05))).astype(np.float32)
    return sc


def _spread_scene():
    """2,197 particles on a 13^3 lattice spread 6 h apart: a 73^3-cell
    bounding grid (389,017 cells > 2^18), one particle per occupied cell."""
    from fluidsimulator_gb300 import scenes

    sc = scenes.dam_break(13, seed=3)
    h = np.float32(sc.params.h)
    lo = sc.pos.min(axis=1, keepdims=True)
    sc.pos[:] = (lo + (sc.pos - lo) * (np.float32(6.0) * h / np.float32(0.05))).astype(np.float32)
    return sc


@pytest.mark.parametrize("make, what", [(_compact_cluster, "list entries"), (_spread_scene, "grid cells")])
def test_noalloc_step_refuses_work_over_the_scratch_limits(cuda_lib, oracle_lib, make, what):
    """The two limits found on the device (list entries, grid cells): the call
    returns FLUID_ERR_CAPACITY and leaves the arrays and time as they were,
    although the refused step had already written part of the scratch; the
    next call on a scene within the limits is exact."""
    torch = pytest.importorskip("torch")

    sc = make()
    assert sc.count <= MAX_PARTICLES
    if what == "list entries":
        counts = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)["neighbor_counts"]
        assert int(counts.sum()) > MAX_NEIGHBOR_SLOTS
    else:
        h = np.float32(sc.params.h)
        span = np.floor(sc.pos.max(axis=1) / h) - np.floor(sc.pos.min(axis=1) / h) + 1
        assert float(np.prod(span)) > MAX_CELLS
    dev, pos, vel = _device_arrays(sc)
    t = ctypes.c_float(0.25)
    for _ in range(2):
        rc = _call(cuda_lib, sc.params, sc.count, pos, vel, t)
        torch.cuda.synchronize(dev)
        assert rc == FLUID_ERR_CAPACITY, (what, rc)
        np.testing.assert_array_equal(pos.cpu().numpy(), sc.pos)
        np.testing.assert_array_equal(vel.cpu().numpy(), sc.vel)
        assert t.value == 0.25
    _normal_call_is_exact(cuda_lib, oracle_lib)
