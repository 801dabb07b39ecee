"""ctypes binding of the C ABI in include/fluid_gb300.h.

The library is built in-tree (fluidsimulator_gb300/_lib/libfluid_gb300.so) by
fluidsimulator_gb300.build. Loading it never touches a GPU; compute calls fail
with FLUID_ERR_NO_DEVICE / FLUID_ERR_CUDA when no device is present. There is
no CPU fallback: if the library is missing, load() raises.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_uint64, c_void_p

MAX_PLANES = 32

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
# FLUID_GB300_LIB selects another build of the same library (e.g. a tuning variant).
LIB_PATH = os.environ.get("FLUID_GB300_LIB") or os.path.join(LIB_DIR, "libfluid_gb300.so")

FLUID_OK = 0
STATUS_NAMES = {
    0: "FLUID_OK",
    1: "FLUID_ERR_INVALID_ARGUMENT",
    2: "FLUID_ERR_CUDA",
    3: "FLUID_ERR_CAPACITY",
    4: "FLUID_ERR_DOMAIN",
    5: "FLUID_ERR_NONFINITE",
    6: "FLUID_ERR_NO_DEVICE",
    7: "FLUID_ERR_OUT_OF_MEMORY",
    8: "FLUID_ERR_NOT_SUPPORTED",
    9: "FLUID_ERR_STATE",
}

MEMORY_HOST = 0
MEMORY_DEVICE = 1

DEBUG_CELL_KEYS = 0
DEBUG_SORTED_ORDER = 1
DEBUG_NEIGHBOR_COUNTS = 2
DEBUG_RHO = 3
DEBUG_LAMBDA = 4

KERNEL_NAMES = ["k_bounds", "k_grid_setup", "k_keys", "k_radix_digits", "k_radix_starts", "k_radix_onesweep",
                "k_reorder", "k_nbr_build", "k_nbr_overflow", "k_lambda", "k_delta", "k_commit",
                "k_xsph", "k_omega", "k_eta"]
TUNABLE = ("k_nbr_build", "k_lambda", "k_delta", "k_xsph", "k_omega", "k_eta")
LIST_PASSES = ("k_lambda", "k_delta", "k_xsph", "k_omega", "k_eta")  # may take several lanes per particle


class FluidParams(ctypes.Structure):
    """Mirror of struct fluid_params (include/fluid_gb300.h)."""

    _fields_ = [
        ("dt", c_float),
        ("density", c_float),
        ("particle_mass", c_float),
        ("h", c_float),
        ("particle_radius", c_float),
        ("epsilon", c_float),
        ("solver_iterations", c_int32),
        ("neighbor_reserve_factor", c_float),
        ("use_uniform_grid", c_int32),
        ("enable_scorr", c_int32),
        ("enable_xsph", c_int32),
        ("enable_vorticity", c_int32),
        ("scorr_k", c_float),
        ("scorr_n", c_int32),
        ("scorr_dq_coeff", c_float),
        ("visc_c", c_float),
        ("plane_restitution", c_float),
        ("plane_friction", c_float),
        ("vort_epsilon", c_float),
        ("vort_norm_eps", c_float),
        ("external_force", c_float * 3),
        ("plane_count", c_int32),
        ("plane_nx", c_float * MAX_PLANES),
        ("plane_ny", c_float * MAX_PLANES),
        ("plane_nz", c_float * MAX_PLANES),
        ("plane_d", c_float * MAX_PLANES),
        ("plane_friction_per_plane", c_int32),
        ("plane_friction_each", c_float * MAX_PLANES),
    ]

    def planes(self):
        n = self.plane_count
        return [(self.plane_nx[i], self.plane_ny[i], self.plane_nz[i], self.plane_d[i]) for i in range(n)]

    def copy(self) -> "FluidParams":
        out = FluidParams()
        ctypes.memmove(ctypes.byref(out), ctypes.byref(self), ctypes.sizeof(FluidParams))
        return out


class FluidStats(ctypes.Structure):
    _fields_ = [
        ("particles", c_int64),
        ("steps", c_int64),
        ("neighbor_pairs", c_int64),
        ("neighbor_max", c_int32),
        ("grid_cells", c_int32),
        ("neighbor_capacity", c_int64),
        ("grid_capacity", c_int64),
        ("regrows", c_int64),
        ("kernel_launches", c_int64),
    ]


def default_params() -> FluidParams:
    """The defaults of fluid::Params (core/include/fluid/core.h:12-43), no planes.

    Kept in Python so that scene construction needs no GPU library; a CPU test
    checks it against fluid_params_default() and the reference's own defaults.
    """
    p = FluidParams()
    p.dt = 1.0 / 60.0
    p.density = 6000.0
    p.particle_mass = 0.0
    p.h = 0.0
    p.particle_radius = 0.01
    p.epsilon = 600.0
    p.solver_iterations = 4
    p.neighbor_reserve_factor = 1.5
    p.use_uniform_grid = 1
    p.enable_scorr = 0
    p.enable_xsph = 0
    p.enable_vorticity = 0
    p.scorr_k = 0.00005
    p.scorr_n = 4
    p.scorr_dq_coeff = 0.3
    p.visc_c = 0.0002
    p.plane_restitution = 0.0
    p.plane_friction = 0.0
    p.vort_epsilon = 0.5
    p.vort_norm_eps = 1e-6
    p.external_force[0] = 0.0
    p.external_force[1] = -9.8
    p.external_force[2] = 0.0
    p.plane_count = 0
    return p


_LIB = None


def _declare(lib):
    f = POINTER(c_float)
    lib.fluid_params_default.argtypes = [POINTER(FluidParams)]
    lib.fluid_params_default.restype = None
    lib.fluid_gb300_version.restype = c_int
    lib.fluid_gb300_device_available.argtypes = [POINTER(c_int), POINTER(c_char_p)]
    lib.fluid_gb300_device_available.restype = c_int
    lib.fluid_gb300_cuda_step.argtypes = [POINTER(FluidParams), c_int64, f, f, f, f, f, f, f]
    lib.fluid_gb300_cuda_step.restype = c_int
    lib.fluid_gb300_step_noalloc.argtypes = [POINTER(FluidParams), c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                             c_void_p, c_void_p, POINTER(c_float), c_void_p]
    lib.fluid_gb300_step_noalloc.restype = c_int
    lib.fluid_solver_create.argtypes = [POINTER(c_void_p), c_int]
    lib.fluid_solver_create.restype = c_int
    lib.fluid_solver_destroy.argtypes = [c_void_p]
    lib.fluid_solver_destroy.restype = None
    lib.fluid_solver_set_stream.argtypes = [c_void_p, c_void_p]
    lib.fluid_solver_set_stream.restype = c_int
    lib.fluid_solver_configure.argtypes = [c_void_p, c_int32, POINTER(FluidParams), POINTER(c_int64)]
    lib.fluid_solver_configure.restype = c_int
    lib.fluid_solver_set_params.argtypes = [c_void_p, POINTER(FluidParams)]
    lib.fluid_solver_set_params.restype = c_int
    lib.fluid_solver_upload.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32]
    lib.fluid_solver_upload.restype = c_int
    lib.fluid_solver_download.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32]
    lib.fluid_solver_download.restype = c_int
    lib.fluid_solver_step.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_step.restype = c_int
    lib.fluid_solver_step_async.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_step_async.restype = c_int
    lib.fluid_solver_synchronize.argtypes = [c_void_p]
    lib.fluid_solver_synchronize.restype = c_int
    lib.fluid_solver_set_graphs.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_set_graphs.restype = c_int
    lib.fluid_solver_set_profiling.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_set_profiling.restype = c_int
    lib.fluid_solver_kernel_times.argtypes = [c_void_p, POINTER(c_double), POINTER(c_int64), c_int32, c_int32]
    lib.fluid_solver_kernel_times.restype = c_int
    lib.fluid_solver_autotune.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_autotune.restype = c_int
    lib.fluid_solver_get_tuning.argtypes = [c_void_p, POINTER(c_int32), POINTER(c_int32), c_int32]
    lib.fluid_solver_get_tuning.restype = c_int
    lib.fluid_solver_set_tuning.argtypes = [c_void_p, POINTER(c_int32), POINTER(c_int32), c_int32]
    lib.fluid_solver_set_tuning.restype = c_int
    lib.fluid_fill_block.argtypes = [c_int64, c_int64, c_int64, c_float, c_float, c_float, c_float, c_double,
                                     c_uint64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]
    lib.fluid_fill_block.restype = c_int
    lib.fluid_fill_shape.argtypes = [c_int32, POINTER(c_float), POINTER(c_float), c_float, POINTER(c_float),
                                     c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64,
                                     POINTER(c_int64), c_void_p]
    lib.fluid_fill_shape.restype = c_int
    lib.fluid_solver_get_lanes.argtypes = [c_void_p, POINTER(c_int32), c_int32]
    lib.fluid_solver_get_lanes.restype = c_int
    lib.fluid_solver_set_lanes.argtypes = [c_void_p, POINTER(c_int32), c_int32]
    lib.fluid_solver_set_lanes.restype = c_int
    lib.fluid_solver_get_sort_bits.argtypes = [c_void_p, POINTER(c_int32)]
    lib.fluid_solver_get_sort_bits.restype = c_int
    lib.fluid_solver_set_sort_bits.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_set_sort_bits.restype = c_int
    lib.fluid_solver_step_backward.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32]
    lib.fluid_solver_step_backward.restype = c_int
    lib.fluid_solver_record.argtypes = [c_void_p, c_int32, c_int32]
    lib.fluid_solver_record.restype = c_int
    lib.fluid_solver_backward.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32]
    lib.fluid_solver_backward.restype = c_int
    lib.fluid_solver_frame_begin.argtypes = [c_void_p, c_int32, c_void_p, c_void_p]
    lib.fluid_solver_frame_begin.restype = c_int
    lib.fluid_solver_frame_wait.argtypes = [c_void_p, c_int32]
    lib.fluid_solver_frame_wait.restype = c_int
    lib.fluid_write_vtp.argtypes = [c_char_p, c_void_p, c_void_p, c_void_p, c_int64, c_int32]
    lib.fluid_write_vtp.restype = c_int
    lib.fluid_write_pvd.argtypes = [c_char_p, POINTER(c_double), POINTER(c_char_p), c_int64]
    lib.fluid_write_pvd.restype = c_int
    lib.fluid_kernel_name.argtypes = [c_int]
    lib.fluid_kernel_name.restype = c_char_p
    lib.fluid_solver_get_time.argtypes = [c_void_p, c_int32, POINTER(c_float)]
    lib.fluid_solver_get_time.restype = c_int
    lib.fluid_solver_set_time.argtypes = [c_void_p, c_int32, c_float]
    lib.fluid_solver_set_time.restype = c_int
    lib.fluid_solver_get_stats.argtypes = [c_void_p, POINTER(FluidStats)]
    lib.fluid_solver_get_stats.restype = c_int
    lib.fluid_solver_read_debug.argtypes = [c_void_p, c_int32, c_void_p, c_int64]
    lib.fluid_solver_read_debug.restype = c_int
    lib.fluid_solver_last_error.argtypes = [c_void_p]
    lib.fluid_solver_last_error.restype = c_char_p
    lib.fluid_status_string.argtypes = [c_int]
    lib.fluid_status_string.restype = c_char_p


def load():
    """Loads the in-tree C-ABI library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no CPU fallback)"
            )
        lib = ctypes.CDLL(LIB_PATH)
        _declare(lib)
        _LIB = lib
    return _LIB
