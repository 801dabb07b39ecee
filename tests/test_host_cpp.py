"""The C++ side of the boundary: the drop-in shim linked into the reference's
own application, and the C++ host interface driving the GPU step."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_scene, load_golden

from oracle.pyoracle import REF_TREE as REF  # noqa: E402  (FLUIDSIM_REFERENCE_TREE)
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


def _build_shim_app(tmp_path):
    """The shim compiled against the reference-interface stand-in
    (tests/cpp/ref_iface) and driven as the reference's app drives it."""
    exe = str(tmp_path / "shim_app_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "tests", "cpp", "ref_iface"), "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "shim_app_main.cpp"),
                    os.path.join(HOST, "cuda_step_shim.cpp"), "-L", LIB_DIR, "-lfluid_gb300",
                    f"-Wl,-rpath,{LIB_DIR}", "-o", exe], check=True)
    return exe


def _write_scene(path, p, pos, vel):
    with open(path, "wb") as f:
        f.write(bytes(p))
        f.write(np.int64(pos.shape[1]).tobytes())
        f.write(np.ascontiguousarray(pos, np.float32).tobytes())
        f.write(np.ascontiguousarray(vel, np.float32).tobytes())


def test_shim_app_builds_and_checks_the_device(cuda_lib, tmp_path):
    exe = _build_shim_app(tmp_path)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if not has_gpu:  # the reference app's own exit path without a device
        r = subprocess.run([exe, "in.bin", "out.bin", "1"], capture_output=True, text=True)
        assert r.returncode == 1 and "CUDA backend unavailable" in r.stderr


@pytest.mark.gpu
def test_shim_drives_the_gpu_step_like_the_reference_app(cuda_lib, tmp_path):
    """fluid::cuda_step of the drop-in shim, called once per step as
    app/src/main.cpp:250-251 calls it, gives the reference's 20-step result
    (golden fixture) bit for bit."""
    exe = _build_shim_app(tmp_path)
    p, d = load_golden("dam_break_flags_4096.npz")
    sc = golden_scene("dam_break_flags_4096.npz")
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    _write_scene(inp, p, sc.pos, sc.vel)
    r = subprocess.run([exe, str(inp), str(out), "20"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "backend=cuda" in r.stdout and f"particle_count={sc.count}" in r.stdout
    raw = np.fromfile(out, np.float32)
    n = sc.count
    np.testing.assert_array_equal(raw[: 3 * n].reshape(3, n), d["s20_pos"])
    np.testing.assert_array_equal(raw[3 * n: 6 * n].reshape(3, n), d["s20_vel"])
    assert np.float32(raw[6 * n]) == d["s20_time"]


@pytest.mark.gpu
def test_shim_failure_stops_an_app_without_try(cuda_lib, tmp_path):
    """A failed step (a non-finite input position, which the step's own key
    kernel reports as FLUID_ERR_NONFINITE) throws from fluid::cuda_step; in
    an application that, like the reference's, calls it outside any try
    block, the run ends through std::terminate with the status on stderr and
    no output written."""
    exe = _build_shim_app(tmp_path)
    p, _ = load_golden("dam_break_flags_4096.npz")
    sc = golden_scene("dam_break_flags_4096.npz")
    pos = sc.pos.copy()
    pos[1, 17] = np.nan
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    _write_scene(inp, p, pos, sc.vel)
    r = subprocess.run([exe, str(inp), str(out), "3"], capture_output=True, text=True)
    assert r.returncode != 0
    assert "cuda_step: " in r.stderr and "non-finite" in r.stderr.lower(), r.stderr
    assert not out.exists()
