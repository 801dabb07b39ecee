"""Python access to the device-resident solver of include/fluid_gb300.h.

Thin ctypes plumbing over the C ABI, used by the tests and the benchmark:
every step runs in the CUDA library; nothing here computes physics.
"""

from __future__ import annotations

import ctypes
from ctypes import byref, c_char_p, c_double, c_float, c_int, c_int64, c_void_p

import numpy as np

from . import _capi
from ._capi import FluidParams, FluidStats


class FluidError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_capi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def device_available() -> tuple[bool, int, str | None]:
    lib = _capi.load()
    n = c_int(0)
    err = c_char_p()
    ok = lib.fluid_gb300_device_available(byref(n), byref(err))
    return bool(ok), n.value, (err.value.decode() if err.value else None)


def _rows(a):
    """Row pointers of a (3, N) float32 array: numpy (host) or torch (host/device)."""
    if isinstance(a, np.ndarray):
        if a.dtype != np.float32 or a.ndim != 2 or a.shape[0] != 3 or not a.flags.c_contiguous:
            raise ValueError("expected a C-contiguous (3, N) float32 array")
        base = a.ctypes.data
        stride = a.strides[0]
        return [base + k * stride for k in range(3)], _capi.MEMORY_HOST
    # torch.Tensor
    if str(a.dtype) != "torch.float32" or a.dim() != 2 or a.shape[0] != 3 or not a.is_contiguous():
        raise ValueError("expected a contiguous (3, N) float32 tensor")
    base = a.data_ptr()
    stride = a.stride(0) * 4
    return [base + k * stride for k in range(3)], (_capi.MEMORY_DEVICE if a.is_cuda else _capi.MEMORY_HOST)


class Solver:
    """One device-resident solver for one or more independent scenes."""

    def __init__(self, device: int = 0):
        self.lib = _capi.load()
        h = c_void_p()
        self._check(self.lib.fluid_solver_create(byref(h), device), None)
        self.h = h
        self.n = 0
        self.counts: list[int] = []

    def _check(self, rc: int, h=...):
        if rc != 0:
            handle = self.h if h is ... else h
            msg = self.lib.fluid_solver_last_error(handle).decode() if handle else ""
            raise FluidError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fluid_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- configuration -----------------------------------------------------
    def configure(self, params: list[FluidParams], counts: list[int]) -> None:
        arr = (FluidParams * len(params))(*params)
        cnt = (c_int64 * len(counts))(*counts)
        self._check(self.lib.fluid_solver_configure(self.h, len(params), arr, cnt))
        self.n = int(sum(counts))
        self.counts = list(counts)

    def set_params(self, params: list[FluidParams]) -> None:
        arr = (FluidParams * len(params))(*params)
        self._check(self.lib.fluid_solver_set_params(self.h, arr))

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(self.lib.fluid_solver_set_stream(self.h, c_void_p(stream_ptr or 0)))

    def set_graphs(self, on: bool) -> None:
        self._check(self.lib.fluid_solver_set_graphs(self.h, int(on)))

    def set_profiling(self, on: bool) -> None:
        self._check(self.lib.fluid_solver_set_profiling(self.h, int(on)))

    # -- state ---------------------------------------------------------------
    def upload(self, pos, vel) -> None:
        pr, pm = _rows(pos)
        vr, vm = _rows(vel)
        if pm != vm:
            raise ValueError("pos and vel must live in the same memory")
        self._check(self.lib.fluid_solver_upload(self.h, *[c_void_p(p) for p in pr + vr], pm))

    def download(self, pos=None, vel=None):
        if pos is None:
            pos = np.empty((3, self.n), np.float32)
        if vel is None:
            vel = np.empty((3, self.n), np.float32)
        pr, pm = _rows(pos)
        vr, vm = _rows(vel)
        if pm != vm:
            raise ValueError("pos and vel must live in the same memory")
        self._check(self.lib.fluid_solver_download(self.h, *[c_void_p(p) for p in pr + vr], pm))
        return pos, vel

    def step(self, n: int = 1) -> None:
        self._check(self.lib.fluid_solver_step(self.h, n))

    def step_async(self, n: int = 1) -> None:
        self._check(self.lib.fluid_solver_step_async(self.h, n))

    def synchronize(self) -> None:
        self._check(self.lib.fluid_solver_synchronize(self.h))

    def time(self, scene: int = 0) -> float:
        t = c_float()
        self._check(self.lib.fluid_solver_get_time(self.h, scene, byref(t)))
        return t.value

    def set_time(self, t: float, scene: int = 0) -> None:
        self._check(self.lib.fluid_solver_set_time(self.h, scene, c_float(t)))

    def stats(self) -> dict:
        s = FluidStats()
        self._check(self.lib.fluid_solver_get_stats(self.h, byref(s)))
        return {k: getattr(s, k) for k, _ in FluidStats._fields_}

    def kernel_times(self, reset: bool = False) -> dict:
        """{kernel name: (total ms, launches)} since the last reset."""
        n = len(_capi.KERNEL_NAMES)
        ms = (c_double * n)()
        la = (c_int64 * n)()
        self._check(self.lib.fluid_solver_kernel_times(self.h, ms, la, n, int(reset)))
        return {name: (ms[k], la[k]) for k, name in enumerate(_capi.KERNEL_NAMES)}

    def autotune(self, trials: int = 2) -> dict:
        """Picks the fastest launch shape per kernel and the faster sort
        digit width on the current state (state not advanced); returns the
        chosen shapes (`sort_bits()` gives the width)."""
        self._check(self.lib.fluid_solver_autotune(self.h, trials))
        return self.tuning()

    def tuning(self) -> dict:
        """{kernel: {"unroll", "block", "lanes"}} of the tunable kernels (lanes:
        lanes per particle of a list pass, 1 elsewhere)."""
        n = len(_capi.KERNEL_NAMES)
        u = (ctypes.c_int32 * n)()
        b = (ctypes.c_int32 * n)()
        g = (ctypes.c_int32 * n)()
        self._check(self.lib.fluid_solver_get_tuning(self.h, u, b, n))
        self._check(self.lib.fluid_solver_get_lanes(self.h, g, n))
        return {name: {"unroll": u[k], "block": b[k], "lanes": g[k]} for k, name in enumerate(_capi.KERNEL_NAMES)
                if name in _capi.TUNABLE}

    def set_tuning(self, shapes: dict) -> None:
        """Sets launch shapes ({kernel: {"unroll", "block"[, "lanes"]}}); kernels
        not named keep theirs."""
        n = len(_capi.KERNEL_NAMES)
        cur = self.tuning()
        u = (ctypes.c_int32 * n)(*([4] * n))
        b = (ctypes.c_int32 * n)(*([256] * n))
        g = (ctypes.c_int32 * n)(*([1] * n))
        for k, name in enumerate(_capi.KERNEL_NAMES):
            shape = shapes.get(name, cur.get(name))
            if shape:
                u[k], b[k] = shape["unroll"], shape["block"]
                g[k] = shape.get("lanes", 1)
        self._check(self.lib.fluid_solver_set_tuning(self.h, u, b, n))
        self._check(self.lib.fluid_solver_set_lanes(self.h, g, n))

    def sort_bits(self) -> int:
        """Digit width of the cell-key radix sort (8, 9 or 11)."""
        b = ctypes.c_int32(0)
        self._check(self.lib.fluid_solver_get_sort_bits(self.h, ctypes.byref(b)))
        return b.value

    def set_sort_bits(self, bits: int) -> None:
        self._check(self.lib.fluid_solver_set_sort_bits(self.h, int(bits)))

    def _cot(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(3, self.n)
        return a

    def step_backward(self, g_pos_out, g_vel_out):
        """VJP of the step the current state would take (state unchanged).
        Returns (g_pos_in, g_vel_in, g_visc_c per scene)."""
        gpo, gvo = self._cot(g_pos_out), self._cot(g_vel_out)
        gpi = np.zeros((3, self.n), np.float32)
        gvi = np.zeros((3, self.n), np.float32)
        gc = np.zeros(max(1, len(self.counts)), np.float32)
        self._check(self.lib.fluid_solver_step_backward(self.h, gpo.ctypes.data_as(c_void_p),
                                                        gvo.ctypes.data_as(c_void_p), gpi.ctypes.data_as(c_void_p),
                                                        gvi.ctypes.data_as(c_void_p), gc.ctypes.data_as(c_void_p),
                                                        _capi.MEMORY_HOST))
        return gpi, gvi, gc

    def record(self, nsteps: int, checkpoint_every: int) -> None:
        self._check(self.lib.fluid_solver_record(self.h, nsteps, checkpoint_every))

    def backward(self, g_pos_final, g_vel_final):
        """dL/d(initial state) and dL/d(visc_c) of the last record()."""
        gpf, gvf = self._cot(g_pos_final), self._cot(g_vel_final)
        gpi = np.zeros((3, self.n), np.float32)
        gvi = np.zeros((3, self.n), np.float32)
        gc = np.zeros(max(1, len(self.counts)), np.float32)
        self._check(self.lib.fluid_solver_backward(self.h, gpf.ctypes.data_as(c_void_p), gvf.ctypes.data_as(c_void_p),
                                                   gpi.ctypes.data_as(c_void_p), gvi.ctypes.data_as(c_void_p),
                                                   gc.ctypes.data_as(c_void_p), _capi.MEMORY_HOST))
        return gpi, gvi, gc

    def frame_begin(self, slot: int, host_pos, host_vel=None) -> None:
        """Starts an asynchronous copy of the current state into host
        buffers of shape (3, N) (pinned memory for overlap)."""
        pr, _ = _rows(host_pos)
        vr = _rows(host_vel)[0][0] if host_vel is not None else None
        self._check(self.lib.fluid_solver_frame_begin(self.h, slot, c_void_p(pr[0]),
                                                      c_void_p(vr) if vr is not None else None))

    def frame_wait(self, slot: int) -> None:
        self._check(self.lib.fluid_solver_frame_wait(self.h, slot))

    def read_debug(self, what: int) -> np.ndarray:
        if what == _capi.DEBUG_CELL_KEYS:
            out = np.empty((self.n, 3), np.int32)
        elif what in (_capi.DEBUG_RHO, _capi.DEBUG_LAMBDA):
            out = np.empty(self.n, np.float32)
        else:
            out = np.empty(self.n, np.int32)
        self._check(self.lib.fluid_solver_read_debug(self.h, what, out.ctypes.data_as(c_void_p), out.size))
        return out


def cuda_step(params: FluidParams, pos: np.ndarray, vel: np.ndarray, time: float) -> float:
    """fluid::cuda_step semantics on host arrays: advances (pos, vel) in place
    by one step and returns the new time."""
    lib = _capi.load()
    pr, _ = _rows(pos)
    vr, _ = _rows(vel)
    t = c_float(time)
    f = ctypes.POINTER(c_float)
    rc = lib.fluid_gb300_cuda_step(byref(params), pos.shape[1], *[ctypes.cast(p, f) for p in pr + vr], byref(t))
    if rc != 0:
        raise FluidError(rc, "fluid_gb300_cuda_step")
    return t.value


def write_vtp(path: str, pos: np.ndarray, binary: bool = True) -> None:
    """One frame of positions (3, N) as VTK PolyData (.vtp)."""
    lib = _capi.load()
    pos = np.ascontiguousarray(pos, np.float32)
    rc = lib.fluid_write_vtp(path.encode(), pos[0].ctypes.data_as(c_void_p), pos[1].ctypes.data_as(c_void_p),
                             pos[2].ctypes.data_as(c_void_p), pos.shape[1], int(binary))
    if rc != 0:
        raise FluidError(rc, f"write_vtp {path}")


def write_pvd(path: str, times, files) -> None:
    lib = _capi.load()
    t = (c_double * len(times))(*times)
    f = (c_char_p * len(files))(*[x.encode() for x in files])
    rc = lib.fluid_write_pvd(path.encode(), t, f, len(files))
    if rc != 0:
        raise FluidError(rc, f"write_pvd {path}")


def read_vtp(path: str) -> np.ndarray:
    """Positions (3, N) from a .vtp written by write_vtp (either encoding)."""
    import re

    data = open(path, "rb").read()
    n = int(re.search(rb'NumberOfPoints="(\d+)"', data).group(1))
    if b'format="appended"' in data:
        start = data.index(b"<AppendedData encoding=\"raw\">") + len(b"<AppendedData encoding=\"raw\">")
        start = data.index(b"_", start) + 1
        nbytes = int(np.frombuffer(data[start:start + 8], np.uint64)[0])
        xyz = np.frombuffer(data[start + 8:start + 8 + nbytes], np.float32).reshape(n, 3)
        return np.ascontiguousarray(xyz.T)
    body = data.split(b'format="ascii">')[1].split(b"</DataArray>")[0]
    return np.array(body.split(), dtype=np.float32).reshape(n, 3).T.copy()
