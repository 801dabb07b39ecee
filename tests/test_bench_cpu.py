"""The benchmark's CPU-side pieces: the reference arm's JSON line (it times
the oracle restatement on the host cores, so it runs here) and the binning of
the trajectory's neighbour-count histograms."""

import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-budget", "0.2"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    assert out["metric"] == "particle-steps/s @1M" and out["unit"] == "particle-steps/s"
    assert out["higher_is_better"] is True and out["n_gpus"] == 1 and out["steps"] == 1
    assert out["value"] > 0
    cpu = out["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == out["value"]
    assert "oracle/pbf_oracle.cpp" in cpu["sample"]
    assert out["e2e"] == {"value": out["value"], "unit": out["unit"], "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}


def test_neighbor_histogram_bins():
    sys.path.insert(0, ROOT)
    import bench

    edges = bench.HIST_EDGES
    assert edges[:4] == [0, 8, 16, 32] and edges[-1] == 32768
    assert all(b == 2 * a for a, b in zip(edges[1:], edges[2:]))
    counts = np.array([0, 7, 8, 15, 16, 28, 31, 32, 8191, 8192, 32767, 32768, 40000], np.int32)
    h = bench.neighbor_histogram(counts)
    assert len(h) == len(edges) and sum(h) == counts.size
    want = [0] * len(edges)
    for c in counts:
        want[max(k for k, e in enumerate(edges) if c >= e)] += 1
    assert h == want
    assert bench.neighbor_histogram(np.zeros(0, np.int32)) == [0] * len(edges)
