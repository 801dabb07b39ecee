"""The C++ side of the boundary: the drop-in shim linked into the reference's
own application, and the C++ host interface driving the GPU step."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_scene, load_golden

REF = "/root/reference"
LIB_DIR = os.path.join(ROOT, "fluidsimulator_gb300", "_lib")
HOST = os.path.join(ROOT, "fluidsimulator_gb300", "csrc", "host")


def _build_driver(tmp_path):
    exe = str(tmp_path / "host_mirror_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", HOST,
                    os.path.join(ROOT, "tests", "cpp", "host_mirror_main.cpp"), "-L", LIB_DIR, "-lfluid_gb300",
                    f"-Wl,-rpath,{LIB_DIR}", "-o", exe], check=True)
    return exe


def test_reference_app_runs_with_the_drop_in(cuda_lib, tmp_path):
    """app/src/main.cpp of the reference, unchanged, linked against the shim
    instead of cuda/src/cuda_stub.cu."""
    if not os.path.isdir(REF):
        pytest.skip("reference tree not present")
    exe = str(tmp_path / "fluidsim")
    srcs = [f"{REF}/app/src/main.cpp", f"{REF}/cli/src/cli.cpp", f"{REF}/io/src/vtk_writer.cpp",
            f"{REF}/core/src/core.cpp", f"{REF}/core/src/init.cpp", os.path.join(HOST, "cuda_step_shim.cpp")]
    inc = []
    for d in ("core/include", "cli/include", "io/include", "cuda/include"):
        inc += ["-I", f"{REF}/{d}"]
    subprocess.run(["g++", "-std=c++17", "-O2", "-fopenmp", "-w", *inc, "-I", os.path.join(ROOT, "include"), *srcs,
                    "-L", LIB_DIR, "-lfluid_gb300", f"-Wl,-rpath,{LIB_DIR}", "-o", exe], check=True)
    r = subprocess.run([exe, "--backend=cpu", "--steps", "1", "--no-output"], capture_output=True, text=True)
    assert r.returncode == 0 and "particle_count=" in r.stdout
    r = subprocess.run([exe, "--backend=cuda", "--steps", "2", "--no-output"], capture_output=True, text=True)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        assert r.returncode == 0 and "backend=cuda" in r.stdout
    else:
        assert r.returncode == 1 and "CUDA backend unavailable" in r.stderr


def test_host_interface_builds(cuda_lib, tmp_path):
    assert shutil.which("g++")
    exe = _build_driver(tmp_path)
    assert os.path.exists(exe)


def test_params_per_plane_friction_to_c(cuda_lib, tmp_path):
    """Params::plane_friction_each maps to the C struct's per-plane fields;
    a list that does not match the planes is rejected."""
    exe = str(tmp_path / "params_to_c_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", HOST,
                    os.path.join(ROOT, "tests", "cpp", "params_to_c_main.cpp"), "-L", LIB_DIR, "-lfluid_gb300",
                    f"-Wl,-rpath,{LIB_DIR}", "-o", exe], check=True)
    assert subprocess.run([exe]).returncode == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["cuda_step", "solver"])
def test_host_interface_matches_golden(cuda_lib, tmp_path, mode):
    exe = _build_driver(tmp_path)
    p, d = load_golden("dam_break_flags_4096.npz")
    sc = golden_scene("dam_break_flags_4096.npz")
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(bytes(p))
        f.write(np.int64(sc.count).tobytes())
        f.write(sc.pos.tobytes())
        f.write(sc.vel.tobytes())
    subprocess.run([exe, str(inp), str(out), "20", mode], check=True)
    raw = np.fromfile(out, np.float32)
    n = sc.count
    pos = raw[: 3 * n].reshape(3, n)
    vel = raw[3 * n: 6 * n].reshape(3, n)
    np.testing.assert_array_equal(pos, d["s20_pos"])
    np.testing.assert_array_equal(vel, d["s20_vel"])
    assert np.float32(raw[6 * n]) == d["s20_time"]
