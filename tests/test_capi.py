"""The C-ABI library without a GPU: it builds, loads, exports every entry
point include/*.h declares, its struct layout matches the ctypes mirror, and
its defaults match fluid::Params (core/include/fluid/core.h:11-43)."""

import ctypes
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT
from fluidsimulator_gb300 import _capi
from fluidsimulator_gb300._capi import FluidParams, FluidStats, default_params


def _declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fluid_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(cuda_lib):
    names = _declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_params_default_matches_mirror(cuda_lib):
    p = FluidParams()
    cuda_lib.fluid_params_default(ctypes.byref(p))
    assert bytes(p) == bytes(default_params())


def test_version(cuda_lib):
    assert cuda_lib.fluid_gb300_version() == 3


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    fields = [f for f, _ in FluidParams._fields_]
    sfields = [f for f, _ in FluidStats._fields_]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "fluid_gb300.h"', "int main(void) {",
             'printf("%zu\\n", sizeof(fluid_params));', 'printf("%zu\\n", sizeof(fluid_stats));']
    lines += [f'printf("%zu\\n", offsetof(fluid_params, {f}));' for f in fields]
    lines += [f'printf("%zu\\n", offsetof(fluid_stats, {f}));' for f in sfields]
    lines += ["return 0; }"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(FluidParams)
    assert out[1] == ctypes.sizeof(FluidStats)
    assert out[2:2 + len(fields)] == [getattr(FluidParams, f).offset for f in fields]
    assert out[2 + len(fields):] == [getattr(FluidStats, f).offset for f in sfields]


def test_rn_sqrt_range_covers_every_scene_with_finite_kernels(tmp_path):
    """A scene's list passes take the fast per-pair square root (rn_sqrt,
    compared with the IEEE square root over its whole checked range on the
    GPU) when the clamped r^2 range [(0.01 h)^2, h^2) lies in that range.
    That holds for every h from 1e-12 to 1e18, far wider than the h for which
    the kernels' float constants are finite (h^9 and h^6 neither overflow nor
    flush to zero: about 1e-4 to 1e4); h = 1e-14 and 1e19 take sqrtf."""
    src = tmp_path / "covers.cpp"
    src.write_text("\n".join([
        '#include <cstdio>', '#include <cstdlib>', '#include "pbf_sqrt.cuh"',
        "int main(int argc, char** argv) {",
        "  for (int k = 1; k < argc; ++k) {",
        "    const float h = std::strtof(argv[k], nullptr);",
        "    const float min_r = 0.01f * h;",  # as the solver's scene constants
        '    std::printf("%d\\n", fgb::rn_sqrt_covers(min_r * min_r, h * h) ? 1 : 0);',
        "  }",
        "  return 0; }"]))
    exe = tmp_path / "covers"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "fluidsimulator_gb300", "csrc"), "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    hs = [f"{10.0 ** e:g}" for e in range(-12, 19)]
    out = subprocess.run([str(exe), *hs, "1e-14", "1e19"], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["1"] * len(hs) + ["0", "0"]


def test_default_lanes_by_particle_count(tmp_path):
    """StepPlan::size_for, the untuned solver's lanes per particle: 8 in
    lambda and delta up to 16,384 particles in all, 4 up to 32,768, 1 above;
    1 in every other pass."""
    src = tmp_path / "lanes.cpp"
    src.write_text("\n".join([
        '#include <cstdio>', '#include <cstdlib>', '#include "pbf_launch.h"',
        "int main(int argc, char** argv) {",
        "  for (int k = 1; k < argc; ++k) {",
        "    fgb::StepPlan p;",
        "    p.size_for(std::atoll(argv[k]));",
        '    std::printf("%d %d %d %d %d\\n", p.lanes[FLUID_KERNEL_LAMBDA], p.lanes[FLUID_KERNEL_DELTA],',
        "                p.lanes[FLUID_KERNEL_XSPH], p.lanes[FLUID_KERNEL_OMEGA], p.lanes[FLUID_KERNEL_ETA]);",
        "  }",
        "  return 0; }"]))
    exe = tmp_path / "lanes"
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "fluidsimulator_gb300", "csrc"), "-I",
                    os.path.join(ROOT, "include"), "-I", cuda_inc, str(src), "-o", str(exe)], check=True)
    counts = [1, 4096, 16384, 16385, 32768, 32769, 1_000_000]
    out = subprocess.run([str(exe), *map(str, counts)], capture_output=True, text=True, check=True).stdout.split("\n")
    want = {1: 8, 4096: 8, 16384: 8, 16385: 4, 32768: 4, 32769: 1, 1_000_000: 1}
    for n, line in zip(counts, out):
        assert [int(x) for x in line.split()] == [want[n], want[n], 1, 1, 1], (n, line)


def test_status_strings(cuda_lib):
    for code in range(10):
        assert cuda_lib.fluid_status_string(code)


def test_device_query_without_gpu(cuda_lib):
    torch = pytest.importorskip("torch")
    n = ctypes.c_int(-1)
    err = ctypes.c_char_p()
    ok = cuda_lib.fluid_gb300_device_available(ctypes.byref(n), ctypes.byref(err))
    assert bool(ok) == torch.cuda.is_available()
    if not torch.cuda.is_available():
        assert n.value == 0
        h = ctypes.c_void_p()
        assert cuda_lib.fluid_solver_create(ctypes.byref(h), 0) == 6  # FLUID_ERR_NO_DEVICE
        assert not h.value


def test_stateless_step_empty_state_advances_time(cuda_lib):
    # count == 0 only advances time (cuda/src/cuda_stub.cu:766-769); no device needed.
    p = default_params()
    p.h = 0.1
    t = ctypes.c_float(1.0)
    assert cuda_lib.fluid_gb300_cuda_step(ctypes.byref(p), 0, None, None, None, None, None, None, ctypes.byref(t)) == 0
    assert t.value == ctypes.c_float(1.0 + ctypes.c_float(p.dt).value).value


def test_null_arguments_rejected(cuda_lib):
    assert cuda_lib.fluid_solver_step(None, 1) == 1
    assert cuda_lib.fluid_solver_configure(None, 1, None, None) == 1
    assert cuda_lib.fluid_gb300_cuda_step(None, 0, None, None, None, None, None, None, None) == 1
