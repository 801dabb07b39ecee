"""Scene fills generated on the device (fluid_fill_block / fluid_fill_shape)
against the host fills: the lattice block of core/src/init.cpp:72-106 with the
benchmark scenes' seeded jitter, and a scene file's cube and sphere shapes
(core/src/init.cpp:285-345, which the host loader reproduces bit for bit from
the reference's loader). Bit for bit."""

import json

import numpy as np
import pytest

from fluidsimulator_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_block_fill_matches_host_1m(cuda_lib):
    sc = scenes.falling_block(100, seed=0)  # 100^3 at (3, 1, 1), spacing 0.02, jitter 1e-4
    got = scenes.fill_block_device(100, 100, 100, (3.0, 1.0, 1.0), 0.02, 1e-4, seed=0).cpu().numpy()
    np.testing.assert_array_equal(got, sc.pos)


def test_block_fill_continues_the_draws_across_blocks(cuda_lib):
    """The double dam break jitters its two blocks as one sequence: the second
    block's first particle takes the draws after the first block's last."""
    sc = scenes.double_dam_break(20, seed=3)
    sp, n = 0.025, 20
    span = (n - 1) * sp
    z0 = 0.5 * (2.0 - span)
    a = scenes.fill_block_device(n, n, n, (sp, sp, z0), sp, 1e-4, seed=3, first=0)
    b = scenes.fill_block_device(n, n, n, (4.0 - sp - span, sp, z0), sp, 1e-4, seed=3, first=n ** 3)
    got = np.concatenate([a.cpu().numpy(), b.cpu().numpy()], axis=1)
    np.testing.assert_array_equal(got, sc.pos)


def test_block_fill_without_jitter_is_init_block(cuda_lib):
    got = scenes.fill_block_device(7, 5, 3, (0.125, -2.5, 1e3), 0.037).cpu().numpy()
    np.testing.assert_array_equal(got, scenes.init_block(7, 5, 3, (0.125, -2.5, 1e3), 0.037))


def test_shape_fills_match_the_scene_loader(cuda_lib, tmp_path):
    shapes = [
        {"type": "cube", "origin": [0.1, 1.0, 0.0], "size": [2.7, 2.9, 2.45], "velocity": [0.5, 0, -1]},
        {"type": "sphere", "origin": [1.3, 0.7, 0.41], "radius": 1.13, "velocity": [0, -2, 0]},
        {"type": "cube", "origin": [-0.3, 0.2, 2.0], "size": [0.05, 0.61, 1.3]},
    ]
    scene = {"fluid": {"particle_mass": 1, "density": 6000, "h": 0.1, "shape": shapes},
             "collisions": [{"type": "plane", "point": [0, 0, 0], "normal": [0, 1, 0]}]}
    path = tmp_path / "shapes.json"
    path.write_text(json.dumps(scene))
    ref = scenes.load_scene_json(str(path))
    spacing = scenes._cbrtf(np.float32(1.0) / np.float32(6000.0))
    pos, vel = [], []
    for sh in shapes:
        ext = sh["size"] if sh["type"] == "cube" else [sh["radius"]]
        p, v = scenes.fill_shape_device(sh["type"], sh["origin"], ext, float(spacing), sh.get("velocity", (0, 0, 0)))
        pos.append(p.cpu().numpy())
        vel.append(v.cpu().numpy())
    np.testing.assert_array_equal(np.concatenate(pos, axis=1), ref.pos)
    np.testing.assert_array_equal(np.concatenate(vel, axis=1), ref.vel)
    assert ref.count > 100_000  # the sphere's compaction spans many blocks


def test_shape_fill_reports_its_size_beyond_capacity(cuda_lib):
    import ctypes

    lib = cuda_lib
    o = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
    e = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
    count = ctypes.c_int64(-1)
    rc = lib.fluid_fill_shape(0, o, e, ctypes.c_float(0.1), None, None, None, None, None, None, None, 10,
                              ctypes.byref(count), None)
    assert rc == 3 and count.value == 1000  # FLUID_ERR_CAPACITY, 10^3 points needed
