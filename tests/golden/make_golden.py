"""Writes the golden fixtures of tests/golden/ from the reference's own CPU
step (core/src/core.cpp of CTKnight/FluidSimulator, compiled from its sources
by `make -C oracle ref`). Run from the repository root where the reference
tree exists:

    python tests/golden/make_golden.py

Each fixture holds the scene's parameters (raw struct bytes), a SHA-256 of
its initial state (which the scene builder must reproduce), and the
reference's outputs: step-1 records (cell keys, sorted order, neighbour
counts, rho, lambda, positions, velocities), later snapshots, and per-step
statistics (neighbour pairs / max, mean / max of rho/rho0 - 1).
"""

from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fluidsimulator_gb300 import scenes  # noqa: E402
from oracle import pyoracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def state_sha(pos: np.ndarray, vel: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(pos, np.float32).tobytes())
    h.update(np.ascontiguousarray(vel, np.float32).tobytes())
    return h.hexdigest()


def fixture(name: str, sc: scenes.Scene, snapshots: list[int], stats_steps: int) -> None:
    ref = pyoracle.Reference()
    data = {
        "params": np.frombuffer(bytes(sc.params), np.uint8),
        "init_sha256": np.array(state_sha(sc.pos, sc.vel)),
    }
    s1 = ref.run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)
    for k in ("pos", "vel", "cell_keys", "sorted_order", "neighbor_counts", "rho", "lambda"):
        data[f"s1_{k}"] = s1[k]
    data["s1_time"] = np.float32(s1["time"])
    for snap in snapshots:
        r = pyoracle.Reference().run(sc.params, sc.pos, sc.vel, 0.0, snap)
        data[f"s{snap}_pos"] = r["pos"]
        data[f"s{snap}_vel"] = r["vel"]
        data[f"s{snap}_time"] = np.float32(r["time"])
    if stats_steps:
        r = pyoracle.Reference().run(sc.params, sc.pos, sc.vel, 0.0, stats_steps, records=True)
        for k in ("neighbor_pairs", "neighbor_max", "density_mean", "density_max"):
            data[f"stats_{k}"] = r[k]
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **data)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


def main() -> None:
    pyoracle.build(ref=True)
    fixture("dam_break_4096", scenes.dam_break(16, seed=0), [10, 240], 240)
    fixture("dam_break_flags_4096", scenes.dam_break(16, seed=0, flags=True), [20], 60)
    fixture("double_dam_break_3456", scenes.double_dam_break(12, seed=0), [20], 0)
    fixture("differentiable_4096", scenes.differentiable_block(16, seed=0), [10], 0)
    sc = scenes.dam_break(8, seed=3, flags=True)
    sc.params.solver_iterations = 0
    fixture("no_iterations_512", sc, [5], 0)
    for k, b in enumerate(scenes.batched_scenes(count=3, seed=1, n_min=300, n_max=3000)):
        fixture(f"batch{k}_{b.count}", b, [10], 0)


if __name__ == "__main__":
    main()
