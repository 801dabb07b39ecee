"""Frame output: ASCII .vtp/.pvd identical to the reference's writers,
binary .vtp round trip, and asynchronous frame capture on the GPU."""

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from fluidsimulator_gb300 import scenes
from fluidsimulator_gb300.solver import read_vtp, write_pvd, write_vtp

from oracle.pyoracle import REF_TREE as REF  # noqa: E402  (FLUIDSIM_REFERENCE_TREE)


def _positions(n=777, seed=3):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((3, n)) * 3.0).astype(np.float32)


def test_ascii_output_matches_reference_writer(cuda_lib, tmp_path):
    if not os.path.isdir(REF):
        pytest.skip("reference tree not present")
    pos = _positions()
    exe = str(tmp_path / "ref_vtk")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", f"{REF}/io/include",
                    os.path.join(ROOT, "tests", "cpp", "ref_vtk_main.cpp"), f"{REF}/io/src/vtk_writer.cpp", "-o", exe],
                   check=True)
    binf = tmp_path / "p.bin"
    with open(binf, "wb") as f:
        f.write(np.int64(pos.shape[1]).tobytes())
        f.write(pos.tobytes())
    ref_dir = tmp_path / "ref"
    subprocess.run([exe, str(binf), str(ref_dir)], check=True)
    ours = tmp_path / "ours.vtp"
    write_vtp(str(ours), pos, binary=False)
    assert ours.read_bytes() == (ref_dir / "frame_000000.vtp").read_bytes()
    pvd = tmp_path / "ours.pvd"
    write_pvd(str(pvd), [0.008333333, 1.25], ["frame_000000.vtp", "frame_000001.vtp"])
    assert pvd.read_bytes() == (ref_dir / "series.pvd").read_bytes()


def test_binary_output_round_trip(cuda_lib, tmp_path):
    pos = _positions(5000, 4)
    path = tmp_path / "b.vtp"
    write_vtp(str(path), pos, binary=True)
    np.testing.assert_array_equal(read_vtp(str(path)), pos)
    assert path.stat().st_size < 21 * pos.shape[1] + 1024
    write_vtp(str(tmp_path / "a.vtp"), pos, binary=False)
    # the reference's ASCII format keeps 9 fixed decimals: lossy near zero
    np.testing.assert_allclose(read_vtp(str(tmp_path / "a.vtp")), pos, rtol=1e-6, atol=6e-10)


@pytest.mark.gpu
def test_async_frames_match_synchronous_downloads(cuda_lib):
    torch = pytest.importorskip("torch")
    from fluidsimulator_gb300.solver import Solver

    sc = scenes.dam_break(12, seed=5, flags=True)
    n = sc.count
    bufs = [torch.empty((3, n), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    vbuf = torch.empty((3, n), dtype=torch.float32, pin_memory=True).numpy()
    s = Solver(0)
    s.configure([sc.params], [n])
    s.upload(sc.pos, sc.vel)
    frames = []
    for k in range(4):
        s.step(3)
        ref = s.download()
        slot = k % 2
        s.frame_begin(slot, bufs[slot], vbuf if slot == 0 else None)
        s.step_async(2)  # overlaps the copy
        s.frame_wait(slot)
        np.testing.assert_array_equal(bufs[slot], ref[0])
        if slot == 0:
            np.testing.assert_array_equal(vbuf, ref[1])
        s.synchronize()
        frames.append(bufs[slot].copy())
        ref_after = s.download()
        s.upload(*ref)  # rewind the two overlapped steps so k advances by 3
        s.set_time(s.time())
    s.close()
    assert not np.array_equal(frames[0], frames[1])
