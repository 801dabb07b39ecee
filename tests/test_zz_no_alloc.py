"""fluid_gb300_step_noalloc: one timestep that allocates no device memory.

It exists for callers that cannot allocate device memory where they step the
fluid (an application that owns every device allocation through its own pool,
a frame-time loop where an allocation would stall, a plugin that must not grow
the process's footprint). Its scratch is a fixed array inside the library, so
the only thing to prove is that it computes the same step as the ordinary
entry point: two calls in a row are compared bit for bit with
fluid_gb300_cuda_step on the same input (the tolerance every parity test here
uses), and a call over the size limit is refused without touching the arrays.
This file is collected last so a failure here cannot hide earlier results.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLUID_ERR_CAPACITY = 3
MAX_PARTICLES = 8192


def _ptrs(t):
    base = t.data_ptr()
    return [ctypes.c_void_p(base + k * t.stride(0) * 4) for k in range(3)]


def test_noalloc_step_matches_stateless_step_twice(cuda_lib):
    torch = pytest.importorskip("torch")
    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import cuda_step

    sc = scenes.dam_break(16, seed=0, flags=True)  # 4,096 particles, all three flags
    assert sc.count <= MAX_PARTICLES
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(sc.pos.copy()).to(dev)
    vel = torch.from_numpy(sc.vel.copy()).to(dev)
    torch.cuda.synchronize(dev)
    host_pos, host_vel = sc.pos.copy(), sc.vel.copy()
    t_dev = ctypes.c_float(0.0)
    t_host = 0.0
    for call in range(2):
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = cuda_lib.fluid_gb300_step_noalloc(ctypes.byref(sc.params), sc.count, *_ptrs(pos), *_ptrs(vel),
                                               ctypes.byref(t_dev), None)
        torch.cuda.synchronize(dev)
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert rc == 0, rc
        if call == 1:
            assert free_after == free_before  # the call itself took no device memory
        t_host = cuda_step(sc.params, host_pos, host_vel, t_host)
        np.testing.assert_array_equal(pos.cpu().numpy(), host_pos)
        np.testing.assert_array_equal(vel.cpu().numpy(), host_vel)
        assert t_dev.value == np.float32(t_host)


def test_noalloc_step_refuses_oversized_input(cuda_lib):
    torch = pytest.importorskip("torch")
    from fluidsimulator_gb300 import scenes

    sc = scenes.dam_break(21, seed=1)  # 9,261 particles > the 8,192 limit
    assert sc.count > MAX_PARTICLES
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(sc.pos.copy()).to(dev)
    vel = torch.from_numpy(sc.vel.copy()).to(dev)
    t = ctypes.c_float(0.0)
    rc = cuda_lib.fluid_gb300_step_noalloc(ctypes.byref(sc.params), sc.count, *_ptrs(pos), *_ptrs(vel),
                                           ctypes.byref(t), None)
    torch.cuda.synchronize(dev)
    assert rc == FLUID_ERR_CAPACITY
    np.testing.assert_array_equal(pos.cpu().numpy(), sc.pos)
    assert t.value == 0.0
