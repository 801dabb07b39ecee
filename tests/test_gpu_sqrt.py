"""The per-pair square root of the list passes (rn_sqrt / rn_sqrt2 in
fluidsimulator_gb300/csrc/pbf_sqrt.cuh) against the IEEE square root for
every float of its checked range. (Which scenes the range covers is checked
on the CPU, tests/test_capi.py.)"""

import json
import os
import subprocess

import pytest

from fluidsimulator_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_rn_sqrt_matches_ieee_over_its_range(cuda_lib, tmp_path):
    exe = str(tmp_path / "rn_sqrt_check")
    subprocess.run([build.nvcc(), "-std=c++20", *build.ARCH, "-O3", "-fmad=false", "-I", build.CSRC, "-I",
                    build.INCLUDE, os.path.join(HERE, "cpp", "rn_sqrt_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout)
    assert r["values"] == int(r["hi"], 16) - int(r["lo"], 16) > 1_800_000_000
    assert r["scalar_mismatches"] == 0, r
    assert r["paired_mismatches"] == 0, r


def test_scene_outside_the_checked_range_takes_sqrtf(cuda_lib, oracle_lib):
    """A dam break scaled to h = 1e-14, gravity off (so the predicted
    positions stay within a few cells): (0.01 h)^2 is below rn_sqrt's
    checked range, so the step's passes take their sqrtf forms. The kernel
    constants of such a scene overflow (h^6 and h^9 flush to zero), so its
    values need not be finite; the step must still give the oracle's values,
    infinities and NaNs in the same places."""
    import numpy as np

    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import Solver

    sc = scenes.dam_break(6, seed=2, flags=True)
    scale = np.float32(1e-13)
    p = sc.params
    p.h = float(np.float32(p.h) * scale)
    for k in range(3):
        p.external_force[k] = 0.0
    for q in range(p.plane_count):
        p.plane_d[q] = float(np.float32(p.plane_d[q]) * scale)
    pos = (sc.pos * scale).astype(np.float32)
    vel = np.zeros_like(pos)
    ref = oracle_lib.Oracle().run(p, pos, vel, 0.0, 1)
    s = Solver(0)
    s.configure([p], [sc.count])
    s.upload(pos, vel)
    s.step(1)
    gpos, gvel = s.download()
    pairs = s.stats()["neighbor_pairs"]
    s.close()
    assert pairs > 0
    np.testing.assert_array_equal(gpos, ref["pos"])
    np.testing.assert_array_equal(gvel, ref["vel"])
