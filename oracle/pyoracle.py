"""ORACLE — test infrastructure, not product code.

ctypes access to the CPU restatement (oracle/_build/libpbf_oracle.so, built by
oracle/Makefile) and, where the reference tree exists, to the reference's own
CPU step (oracle/_ref/libfluid_ref.so). Only the tests, the smoke check and the
bench's CPU-baseline leg import this module.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_void_p

import numpy as np

from fluidsimulator_gb300._capi import FluidParams

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libpbf_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfluid_ref.so")
# The reference source tree (only the pin and a few tests read it): the
# FLUIDSIM_REFERENCE_TREE environment variable, else the default location of
# the read-only checkout. The GPU host has no such tree; the pin is then skipped.
REF_TREE = os.environ.get("FLUIDSIM_REFERENCE_TREE", "/root/reference")


class _Dump(ctypes.Structure):
    _fields_ = [
        ("cell_keys", c_void_p),
        ("sorted_order", c_void_p),
        ("neighbor_counts", c_void_p),
        ("rho", c_void_p),
        ("lambda_", c_void_p),
    ]


def build(ref: bool | None = None) -> None:
    """Compiles the restatement, and the reference pin when its tree exists."""
    if ref is None:
        ref = os.path.isdir(REF_TREE)
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, f"REF={REF_TREE}"] + targets, check=True)


_LIBS: dict[str, ctypes.CDLL] = {}


def _lib(path: str) -> ctypes.CDLL:
    if path not in _LIBS:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} not built (run oracle.pyoracle.build())")
        _LIBS[path] = ctypes.CDLL(path)
    return _LIBS[path]


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


class _Runner:
    """Common driver for the oracle (f32 / f64) and the reference pin."""

    dtype = np.float32

    def __init__(self):
        self.handle = None

    def _run(self, params, pos, vel, time, nsteps, dump, pairs, nmax, dmean, dmax):
        raise NotImplementedError

    def run(self, params: FluidParams, pos: np.ndarray, vel: np.ndarray, time: float = 0.0,
            nsteps: int = 1, dump: bool = False, records: bool = False):
        """Advances copies of (pos, vel) by nsteps; returns a dict with pos,
        vel, time and, on request, the last step's dump and per-step records."""
        n = pos.shape[1]
        pos = np.ascontiguousarray(pos, dtype=self.dtype).copy()
        vel = np.ascontiguousarray(vel, dtype=self.dtype).copy()
        t = np.array([time], dtype=self.dtype)
        out = {}
        d = None
        if dump:
            out["cell_keys"] = np.zeros((n, 3), np.int32)
            out["sorted_order"] = np.zeros(n, np.int32)
            out["neighbor_counts"] = np.zeros(n, np.int32)
            out["rho"] = np.zeros(n, self.dtype)
            out["lambda"] = np.zeros(n, self.dtype)
            d = _Dump(_ptr(out["cell_keys"]), _ptr(out["sorted_order"]), _ptr(out["neighbor_counts"]),
                      _ptr(out["rho"]), _ptr(out["lambda"]))
        rec = None
        if records:
            rec = {
                "neighbor_pairs": np.zeros(nsteps, np.int64),
                "neighbor_max": np.zeros(nsteps, np.int32),
                "density_mean": np.zeros(nsteps, np.float64),
                "density_max": np.zeros(nsteps, np.float64),
            }
        rc = self._run(params, n, pos, vel, t, nsteps, d,
                       *(_ptr(rec[k]) if rec else None for k in ("neighbor_pairs", "neighbor_max", "density_mean", "density_max")))
        if rc != 0:
            raise RuntimeError(f"oracle step failed with status {rc}")
        out["pos"], out["vel"], out["time"] = pos, vel, t[0]
        if rec:
            out.update(rec)
        return out


class Oracle(_Runner):
    """The CPU restatement, float32 (default) or float64 arithmetic."""

    def __init__(self, dtype=np.float32):
        super().__init__()
        self.dtype = np.dtype(dtype).type
        self.suffix = "f32" if self.dtype == np.float32 else "f64"
        lib = _lib(ORACLE_SO)
        create = getattr(lib, f"pbf_oracle_create_{self.suffix}")
        create.restype = c_void_p
        self._destroy = getattr(lib, f"pbf_oracle_destroy_{self.suffix}")
        self._destroy.argtypes = [c_void_p]
        self._step = getattr(lib, f"pbf_oracle_run_{self.suffix}")
        fp = c_void_p
        self._step.argtypes = [c_void_p, POINTER(FluidParams), c_int64, fp, fp, fp, fp, fp, fp, fp, c_int32,
                               POINTER(_Dump), fp, fp, fp, fp]
        self._step.restype = c_int
        self.handle = create()

    def __del__(self):
        if getattr(self, "handle", None):
            self._destroy(self.handle)
            self.handle = None

    def _run(self, params, n, pos, vel, t, nsteps, d, pairs, nmax, dmean, dmax):
        return self._step(self.handle, ctypes.byref(params), n, _ptr(pos[0]), _ptr(pos[1]), _ptr(pos[2]),
                          _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), _ptr(t), nsteps,
                          ctypes.byref(d) if d is not None else None, pairs, nmax, dmean, dmax)


def set_threads(n: int) -> int:
    lib = _lib(ORACLE_SO)
    lib.pbf_oracle_threads.argtypes = [c_int]
    lib.pbf_oracle_threads.restype = c_int
    return lib.pbf_oracle_threads(n)


class Reference(_Runner):
    """The reference's own fluid::step, compiled from its sources (float32)."""

    def __init__(self):
        super().__init__()
        lib = _lib(REF_SO)
        lib.ref_create.restype = c_void_p
        lib.ref_destroy.argtypes = [c_void_p]
        fp = c_void_p
        lib.ref_run.argtypes = [c_void_p, POINTER(FluidParams), c_int64, fp, fp, fp, fp, fp, fp, fp, c_int32,
                                POINTER(_Dump), fp, fp, fp, fp]
        lib.ref_run.restype = c_int
        self.lib = lib
        self.handle = lib.ref_create()

    def __del__(self):
        if getattr(self, "handle", None):
            self.lib.ref_destroy(self.handle)
            self.handle = None

    def _run(self, params, n, pos, vel, t, nsteps, d, pairs, nmax, dmean, dmax):
        return self.lib.ref_run(self.handle, ctypes.byref(params), n, _ptr(pos[0]), _ptr(pos[1]), _ptr(pos[2]),
                                _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), _ptr(t), nsteps,
                                ctypes.byref(d) if d is not None else None, pairs, nmax, dmean, dmax)


def ref_default_params() -> FluidParams:
    lib = _lib(REF_SO)
    lib.ref_default_params.argtypes = [POINTER(FluidParams)]
    p = FluidParams()
    lib.ref_default_params(ctypes.byref(p))
    return p


def ref_init_block(params: FluidParams, nx, ny, nz, origin, spacing) -> np.ndarray:
    lib = _lib(REF_SO)
    n = nx * ny * nz
    out = np.zeros((3, n), np.float32)
    lib.ref_init_block.argtypes = [POINTER(FluidParams), c_int64, c_int64, c_int64, c_float, c_float, c_float,
                                   c_float, c_void_p, c_void_p, c_void_p]
    lib.ref_init_block(ctypes.byref(params), nx, ny, nz, origin[0], origin[1], origin[2], spacing,
                       _ptr(out[0]), _ptr(out[1]), _ptr(out[2]))
    return out


def ref_init_planes(params: FluidParams, bx, by, bz) -> FluidParams:
    lib = _lib(REF_SO)
    lib.ref_init_planes.argtypes = [POINTER(FluidParams), c_float, c_float, c_float]
    p = params.copy()
    lib.ref_init_planes(ctypes.byref(p), bx, by, bz)
    return p


def ref_init_test_scene(params: FluidParams):
    lib = _lib(REF_SO)
    lib.ref_init_test_scene.argtypes = [POINTER(FluidParams), c_int64, c_void_p, c_void_p, c_void_p, POINTER(c_int64)]
    p = params.copy()
    cnt = c_int64(0)
    lib.ref_init_test_scene(ctypes.byref(p), 0, None, None, None, ctypes.byref(cnt))
    pos = np.zeros((3, cnt.value), np.float32)
    lib.ref_init_test_scene(ctypes.byref(p), cnt.value, _ptr(pos[0]), _ptr(pos[1]), _ptr(pos[2]), ctypes.byref(cnt))
    return p, pos


def ref_load_scene(path: str):
    lib = _lib(REF_SO)
    fp = c_void_p
    lib.ref_load_scene.argtypes = [c_char_p, POINTER(FluidParams), c_int64, fp, fp, fp, fp, fp, fp,
                                   POINTER(c_int64), c_char_p, c_int64]
    p = FluidParams()
    cnt = c_int64(0)
    err = ctypes.create_string_buffer(512)
    rc = lib.ref_load_scene(path.encode(), ctypes.byref(p), 0, None, None, None, None, None, None,
                            ctypes.byref(cnt), err, 512)
    if rc == 1:
        raise ValueError(err.value.decode())
    pos = np.zeros((3, cnt.value), np.float32)
    vel = np.zeros((3, cnt.value), np.float32)
    rc = lib.ref_load_scene(path.encode(), ctypes.byref(p), cnt.value, _ptr(pos[0]), _ptr(pos[1]), _ptr(pos[2]),
                            _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), ctypes.byref(cnt), err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return p, pos, vel


def vjp(params: FluidParams, pos, vel, gx_out, gv_out, fwd32: bool = False):
    """One step's vector-Jacobian product by the oracle (double arithmetic).

    Runs the forward step from (pos, vel) in float32 (fwd32) or float64,
    then back-propagates the output cotangents. Returns (gx_in, gv_in, gc,
    pos_out, vel_out)."""
    lib = _lib(ORACLE_SO)
    fp = c_void_p
    lib.pbf_oracle_vjp.argtypes = [POINTER(FluidParams), c_int64, c_int32, fp, fp, fp, fp, fp, fp, fp, fp, fp]
    lib.pbf_oracle_vjp.restype = c_int
    dt = np.float32 if fwd32 else np.float64
    n = pos.shape[1]
    x = np.ascontiguousarray(pos, dt)
    v = np.ascontiguousarray(vel, dt)
    xo = np.zeros_like(x)
    vo = np.zeros_like(v)
    gxo = np.ascontiguousarray(gx_out, np.float64)
    gvo = np.ascontiguousarray(gv_out, np.float64)
    gxi = np.zeros((3, n))
    gvi = np.zeros((3, n))
    gc = np.zeros(1)
    rc = lib.pbf_oracle_vjp(ctypes.byref(params), n, int(fwd32), _ptr(x), _ptr(v), _ptr(xo), _ptr(vo), _ptr(gxo),
                            _ptr(gvo), _ptr(gxi), _ptr(gvi), _ptr(gc))
    if rc != 0:
        raise RuntimeError(f"oracle vjp failed with status {rc}")
    return gxi, gvi, float(gc[0]), xo, vo
