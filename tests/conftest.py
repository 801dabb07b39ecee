import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_lib():
    """Builds the oracle restatement (and the reference pin where the
    reference tree exists)."""
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def cuda_lib():
    """Builds the CUDA library in-tree and loads it (no fallback)."""
    from fluidsimulator_gb300 import _capi, build

    build.build()
    return _capi.load()


def golden_files():
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    import numpy as np

    from fluidsimulator_gb300._capi import FluidParams

    d = dict(np.load(os.path.join(GOLDEN, name)))
    p = FluidParams.from_buffer_copy(d["params"].tobytes())
    return p, d


def golden_scene(name):
    """Rebuilds the fixture's initial state with the scene builders."""
    from fluidsimulator_gb300 import scenes

    if name.startswith("dam_break_flags"):
        return scenes.dam_break(16, seed=0, flags=True)
    if name.startswith("dam_break"):
        return scenes.dam_break(16, seed=0)
    if name.startswith("double_dam_break"):
        return scenes.double_dam_break(12, seed=0)
    if name.startswith("differentiable"):
        return scenes.differentiable_block(16, seed=0)
    if name.startswith("no_iterations"):
        sc = scenes.dam_break(8, seed=3, flags=True)
        sc.params.solver_iterations = 0
        return sc
    if name.startswith("batch"):
        k = int(name[5])
        return scenes.batched_scenes(count=3, seed=1, n_min=300, n_max=3000)[k]
    raise KeyError(name)
