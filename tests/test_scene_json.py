"""Scene JSON loader against the reference's own loader
(core/src/init.cpp:158-418) on the reference's scene files, plus the
additional keys."""

import glob
import json
import os

import numpy as np
import pytest

from fluidsimulator_gb300 import scenes

from oracle.pyoracle import REF_TREE  # noqa: E402  (FLUIDSIM_REFERENCE_TREE)

REF_SCENES = sorted(glob.glob(os.path.join(REF_TREE, "scene", "*.json")))


@pytest.mark.parametrize("path", REF_SCENES, ids=[os.path.basename(p) for p in REF_SCENES])
def test_loader_matches_reference_loader(oracle_lib, path):
    if not oracle_lib.ref_available():
        pytest.skip("reference tree not present")
    p, pos, vel = oracle_lib.ref_load_scene(path)
    sc = scenes.load_scene_json(path)
    assert bytes(sc.params) == bytes(p)
    np.testing.assert_array_equal(sc.pos, pos)
    np.testing.assert_array_equal(sc.vel, vel)


def test_additional_keys(tmp_path):
    scene = {
        "fluid": {"particle_mass": 0.125, "density": 1000, "h": 0.1, "epsilon": 100, "n": 4, "k": 0.1, "c": 0.01,
                  "shape": [{"type": "cube", "origin": [0.025, 0.025, 0.025], "size": [0.8, 0.8, 0.8]},
                            {"type": "sphere", "origin": [0.5, 0.7, 0.5], "radius": 0.15, "velocity": [0, -1, 0]}]},
        "external_forces": [0, -9.8, 0],
        "collisions": [{"type": "plane", "point": [0, 0, 0], "normal": [0, 2, 0]},
                       {"type": "plane", "point": [1, 1, 1], "normal": [0, -1, 0]}],
        "solver": {"dt": 0.008333333, "iterations": 3, "scorr_dq_coeff": 0.2, "vort_epsilon": 0.0005,
                   "enable_scorr": True, "enable_xsph": True, "enable_vorticity": True,
                   "plane_restitution": 0.05, "plane_friction": 0.1},
        "jitter": {"amplitude": 5e-4, "seed": 3},
    }
    path = tmp_path / "s.json"
    path.write_text(json.dumps(scene))
    sc = scenes.load_scene_json(str(path))
    assert sc.params.solver_iterations == 3 and sc.params.enable_vorticity == 1
    assert sc.params.plane_count == 2 and sc.params.plane_ny[0] == 1.0 and sc.params.plane_d[1] == -1.0
    assert np.float32(sc.params.scorr_dq_coeff) == np.float32(0.2)
    assert sc.count > 1000 and np.all(sc.vel[1, -10:] == -1.0)
    plain = dict(scene)
    plain.pop("jitter")
    path.write_text(json.dumps(plain))
    base = scenes.load_scene_json(str(path))
    assert 0 < np.max(np.abs(sc.pos - base.pos)) <= 5e-4 * 1.0001


def test_per_plane_friction_key(tmp_path):
    """Per-collision "friction" is read only under "per_plane_friction";
    a collision without one takes the scene's plane_friction."""
    scene = {
        "fluid": {"particle_mass": 0.125, "density": 1000, "h": 0.1, "epsilon": 100,
                  "shape": [{"type": "cube", "origin": [0.1, 0.1, 0.1], "size": [0.2, 0.2, 0.2]}]},
        "collisions": [{"type": "plane", "point": [0, 0, 0], "normal": [0, 1, 0], "friction": 0.5},
                       {"type": "plane", "point": [0, 0, 0], "normal": [1, 0, 0]},
                       {"type": "plane", "point": [1, 1, 1], "normal": [0, -1, 0], "friction": 0.0}],
        "solver": {"plane_restitution": 0.05, "plane_friction": 0.1},
    }
    path = tmp_path / "s.json"
    path.write_text(json.dumps(scene))
    off = scenes.load_scene_json(str(path))
    assert off.params.plane_friction_per_plane == 0
    assert list(off.params.plane_friction_each[:3]) == [0.0, 0.0, 0.0]
    scene["solver"]["per_plane_friction"] = True
    path.write_text(json.dumps(scene))
    on = scenes.load_scene_json(str(path))
    assert on.params.plane_friction_per_plane == 1
    mu = [np.float32(x) for x in on.params.plane_friction_each[:3]]
    assert mu == [np.float32(0.5), np.float32(0.1), np.float32(0.0)]
    np.testing.assert_array_equal(on.pos, off.pos)


def test_set_plane_friction_needs_one_value_per_plane():
    p = scenes.dam_break(2).params
    with pytest.raises(ValueError):
        scenes.set_plane_friction(p, [0.1] * (p.plane_count - 1))
    scenes.set_plane_friction(p, [0.1] * p.plane_count)
    assert p.plane_friction_per_plane == 1
