"""Scene construction for the PBF step: lattice blocks, box planes and the
seeded benchmark scenes.

`init_block` and `init_planes` restate the reference's scene helpers
(core/src/init.cpp:72-107 and :109-117) in float32 arithmetic, so a scene built
here is bit-identical to one built by the reference (checked by a CPU test
against the reference compiled from source).

Randomness (lattice jitter, scene sizes, initial velocities) comes from
SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014) keyed by an explicit seed, so every run on every
machine builds the same scene. The reference publishes no dataset; all scenes
are synthetic.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from ._capi import MAX_PLANES, FluidParams, default_params

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Draws `count` 64-bit outputs of SplitMix64 seeded with `seed`,
    starting after `offset` earlier draws."""
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Float64 uniforms in [0, 1) with 53 random bits."""
    return (splitmix64(seed, count, offset) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Standard normals by the Box-Muller transform of paired uniforms."""
    m = (count + 1) // 2
    u = uniform01(seed, 2 * m, offset)
    u1 = 1.0 - u[0::2]  # (0, 1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2.0 * np.pi * u2), r * np.sin(2.0 * np.pi * u2)])
    out = np.empty(2 * m)
    out[0::2] = z[:m]
    out[1::2] = z[m:]
    return out[:count]


@dataclass
class Scene:
    """One scene: parameters plus SoA float32 state in caller order."""

    name: str
    params: FluidParams
    pos: np.ndarray  # (3, N) float32
    vel: np.ndarray  # (3, N) float32
    steps: int = 1
    info: dict = field(default_factory=dict)

    def __post_init__(self):
        self.pos = np.ascontiguousarray(self.pos, dtype=np.float32)
        self.vel = np.ascontiguousarray(self.vel, dtype=np.float32)

    @property
    def count(self) -> int:
        return int(self.pos.shape[1])

    def copy(self) -> "Scene":
        return Scene(self.name, self.params.copy(), self.pos.copy(), self.vel.copy(), self.steps, dict(self.info))


def init_block(nx: int, ny: int, nz: int, origin, spacing: float) -> np.ndarray:
    """Lattice of nx*ny*nz particles, z outermost and x innermost, each
    coordinate origin + float(index) * spacing in float32
    (core/src/init.cpp:96-106). Returns (3, N) float32."""
    f32 = np.float32
    step = f32(spacing)
    ix = np.arange(nx, dtype=np.float32)
    iy = np.arange(ny, dtype=np.float32)
    iz = np.arange(nz, dtype=np.float32)
    x = f32(origin[0]) + ix * step
    y = f32(origin[1]) + iy * step
    z = f32(origin[2]) + iz * step
    zz, yy, xx = np.meshgrid(z, y, x, indexing="ij")
    return np.stack([xx.ravel(), yy.ravel(), zz.ravel()]).astype(np.float32)


def add_plane_normalized(p: FluidParams, nx: float, ny: float, nz: float, d: float) -> None:
    """PlaneSoA::add_normalized (core/include/fluid/core.h:69-77) in float32."""
    if p.plane_count >= MAX_PLANES:
        raise ValueError("too many planes")
    f32 = np.float32
    nx, ny, nz, d = f32(nx), f32(ny), f32(nz), f32(d)
    len_sq = nx * nx + ny * ny + nz * nz
    if len_sq > f32(0):
        inv = f32(1) / np.sqrt(len_sq, dtype=np.float32)
        nx, ny, nz = nx * inv, ny * inv, nz * inv
    i = p.plane_count
    p.plane_nx[i], p.plane_ny[i], p.plane_nz[i], p.plane_d[i] = float(nx), float(ny), float(nz), float(d)
    p.plane_count = i + 1


def init_planes(p: FluidParams, bx: float, by: float, bz: float) -> None:
    """Six inward planes of the box [0,bx]x[0,by]x[0,bz] (core/src/init.cpp:109-117)."""
    p.plane_count = 0
    add_plane_normalized(p, 1.0, 0.0, 0.0, 0.0)
    add_plane_normalized(p, -1.0, 0.0, 0.0, -bx)
    add_plane_normalized(p, 0.0, 1.0, 0.0, 0.0)
    add_plane_normalized(p, 0.0, -1.0, 0.0, -by)
    add_plane_normalized(p, 0.0, 0.0, 1.0, 0.0)
    add_plane_normalized(p, 0.0, 0.0, -1.0, -bz)


def set_plane_friction(p: FluidParams, frictions) -> None:
    """Gives each plane its own friction, in plane order (an extension: the
    reference applies one plane_friction to all planes, core/src/core.cpp:575)."""
    if len(frictions) != p.plane_count:
        raise ValueError(f"{len(frictions)} frictions for {p.plane_count} planes")
    p.plane_friction_per_plane = 1
    for q, mu in enumerate(frictions):
        p.plane_friction_each[q] = float(np.float32(mu))


def jitter(pos: np.ndarray, amplitude: float, seed: int, offset: int = 0) -> np.ndarray:
    """pos + U(-a, a) per coordinate; draw k = 3*i + axis, added in float32."""
    n = pos.shape[1]
    u = uniform01(seed, 3 * n, offset).reshape(n, 3).T
    j = (amplitude * (2.0 * u - 1.0)).astype(np.float32)
    return (pos + j).astype(np.float32)


def base_params(spacing: float, h: float) -> FluidParams:
    """Physics shared by the benchmark scenes: rho0 = 1000, m = rho0 * sp^3,
    relaxation 100, dt = 1/120, 4 iterations, restitution 0.05, friction 0.1."""
    p = default_params()
    p.density = 1000.0
    p.particle_mass = float(np.float32(1000.0) * np.float32(spacing) ** 3)
    p.h = h
    p.epsilon = 100.0
    p.dt = 1.0 / 120.0
    p.solver_iterations = 4
    p.plane_restitution = 0.05
    p.plane_friction = 0.1
    return p


def all_flags(p: FluidParams, h: float) -> None:
    """s_corr k = 0.1, n = 4, dq = 0.2 h; XSPH c = 0.01; vorticity eps = 5e-4."""
    p.enable_scorr = 1
    p.scorr_k = 0.1
    p.scorr_n = 4
    p.scorr_dq_coeff = 0.2
    p.enable_xsph = 1
    p.visc_c = 0.01
    p.enable_vorticity = 1
    p.vort_epsilon = 0.0005


def dam_break(n_side: int = 16, seed: int = 0, flags: bool = False) -> Scene:
    """Plain dam break: n^3 lattice, spacing 0.05, corner (0.05,0.05,0.05),
    jitter U(+-5e-4), box [0,1]^3, h = 0.1, flags off; 240 steps (n = 16:
    4,096 particles)."""
    sp, h = 0.05, 0.1
    p = base_params(sp, h)
    init_planes(p, 1.0, 1.0, 1.0)
    if flags:
        all_flags(p, h)
    pos = jitter(init_block(n_side, n_side, n_side, (0.05, 0.05, 0.05), sp), 5e-4, seed)
    vel = np.zeros_like(pos)
    return Scene(f"dam_break_{n_side ** 3}", p, pos, vel, steps=240,
                 info={"spacing": sp, "box": (1.0, 1.0, 1.0), "seed": seed})


def double_dam_break(n_side: int = 50, seed: int = 0) -> Scene:
    """Two n^3 blocks (2 x 125,000 at n = 50), spacing 0.025, h = 0.05, at the
    two x-ends of a 4x2x2 box floor, centred in z; all three flags on; jitter
    U(+-1e-4); 480 steps. Block placement is this builder's choice (the
    benchmark leaves it open)."""
    sp, h = 0.025, 0.05
    bx, by, bz = 4.0, 2.0, 2.0
    p = base_params(sp, h)
    init_planes(p, bx, by, bz)
    all_flags(p, h)
    span = (n_side - 1) * sp
    z0 = 0.5 * (bz - span)
    a = init_block(n_side, n_side, n_side, (sp, sp, z0), sp)
    b = init_block(n_side, n_side, n_side, (bx - sp - span, sp, z0), sp)
    pos = jitter(np.concatenate([a, b], axis=1), 1e-4, seed)
    vel = np.zeros_like(pos)
    return Scene(f"double_dam_break_{2 * n_side ** 3}", p, pos, vel, steps=480,
                 info={"spacing": sp, "box": (bx, by, bz), "seed": seed})


def falling_block(n_side: int = 100, seed: int = 0) -> Scene:
    """1M-particle throughput scene: an n^3 block (n = 100), spacing 0.02,
    h = 0.04, in an 8x4x4 box, lower corner at (3, 1, 1) so it falls under
    gravity; all three flags on; jitter U(+-1e-4); 600 steps. The corner is
    this builder's choice (the benchmark leaves it open)."""
    sp, h = 0.02, 0.04
    bx, by, bz = 8.0, 4.0, 4.0
    p = base_params(sp, h)
    init_planes(p, bx, by, bz)
    all_flags(p, h)
    pos = jitter(init_block(n_side, n_side, n_side, (3.0, 1.0, 1.0), sp), 1e-4, seed)
    vel = np.zeros_like(pos)
    return Scene(f"falling_block_{n_side ** 3}", p, pos, vel, steps=600,
                 info={"spacing": sp, "box": (bx, by, bz), "seed": seed, "origin": (3.0, 1.0, 1.0)})


def batched_scenes(count: int = 64, seed: int = 0, n_min: int = 2000, n_max: int = 64000) -> list[Scene]:
    """Batched dam breaks: `count` scenes, particle targets U[n_min, n_max]
    and lattice aspect ratios x:y and z:y in U[0.5, 2] from the seed; spacing
    0.05, h = 0.1, each in its own [0,2]x[0,1]x[0,1] box with the block's
    corner at (0.05, 0.05, 0.05); flags on; jitter U(+-5e-4); 240 steps.
    Blocks above ~16k particles do not fit the box at this spacing: the first
    plane projection moves the overhang onto the walls, as the reference would."""
    sp, h = 0.05, 0.1
    u = uniform01(seed ^ 0xB47C4, 3 * count).reshape(count, 3)
    scenes = []
    off = 0
    for s in range(count):
        target = n_min + int(u[s, 0] * (n_max - n_min + 1))
        rx = 0.5 + 1.5 * u[s, 1]
        rz = 0.5 + 1.5 * u[s, 2]
        base = (target / (rx * rz)) ** (1.0 / 3.0)
        nx = max(1, int(round(rx * base)))
        nz = max(1, int(round(rz * base)))
        ny = max(1, int(round(target / (nx * nz))))
        p = base_params(sp, h)
        init_planes(p, 2.0, 1.0, 1.0)
        all_flags(p, h)
        pos = jitter(init_block(nx, ny, nz, (0.05, 0.05, 0.05), sp), 5e-4, seed, offset=off)
        off += 3 * pos.shape[1]
        scenes.append(Scene(f"batch_{s}", p, pos, np.zeros_like(pos), steps=240,
                            info={"lattice": (nx, ny, nz), "target": target}))
    return scenes


def differentiable_block(n_side: int = 32, seed: int = 0, unit_mass: bool = False) -> Scene:
    """Differentiable scene: n^3 block (n = 32), spacing 0.05, h = 0.1, corner
    (0.2, 0.05, 0.2) in a [0,2]^3 box, XSPH c = 0.01 and s_corr on (k = 0.1,
    n = 4, dq = 0.2 h), vorticity off; initial velocity N(0, 0.1^2) per
    component; 60 steps.

    unit_mass: the well-conditioned variant with m = 1 and rho0 = 1/sp^3 (the
    convention of the reference's own scene files), where the Jacobi update
    is not scaled by 1/m."""
    sp, h = 0.05, 0.1
    p = base_params(sp, h)
    if unit_mass:
        p.particle_mass = 1.0
        p.density = float(np.float32(1.0) / np.float32(sp) ** 3)
    init_planes(p, 2.0, 2.0, 2.0)
    all_flags(p, h)
    p.enable_vorticity = 0
    pos = init_block(n_side, n_side, n_side, (0.2, 0.05, 0.2), sp)
    n = pos.shape[1]
    vel = (0.1 * normal(seed ^ 0x5E1, 3 * n).reshape(n, 3).T).astype(np.float32)
    return Scene(f"differentiable_{n}" + ("_unit_mass" if unit_mass else ""), p, pos, vel, steps=60,
                 info={"spacing": sp, "box": (2.0, 2.0, 2.0), "seed": seed, "target": (1.5, 0.3, 1.0)})


def _fill_axis(start: np.float32, stop: np.float32, step: np.float32) -> np.ndarray:
    """float v = start; v < stop; v += step -- accumulated in float32."""
    out = []
    v = np.float32(start)
    while v < stop:
        out.append(v)
        v = np.float32(v + step)
    return np.array(out, dtype=np.float32)


def _cbrtf(x: np.float32) -> np.float32:
    """The C library's cbrtf (what std::cbrt(float) calls), for bit-identical
    spacing; numpy's float32 cbrt may differ in the last place."""
    import ctypes
    import ctypes.util

    try:
        libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        fn = libm.cbrtf
        fn.argtypes = [ctypes.c_float]
        fn.restype = ctypes.c_float
        return np.float32(fn(float(x)))
    except (OSError, AttributeError):
        return np.cbrt(np.float32(x), dtype=np.float32)


def load_scene_json(path: str) -> Scene:
    """Scene file in the reference's legacy format (core/src/init.cpp:158-418):
    fluid {particle_mass, density, h, epsilon, n, k, c, shape[]} with cube
    (origin, size) and sphere (origin, radius) fills and an optional velocity,
    external_forces, and collisions[] of planes (point, normal). Fills
    accumulate in float32 exactly as the reference's loops do, so the
    particles are bit-identical to the reference loader's.

    Additional keys, ignored by the reference and optional here:
      "solver": {"dt", "iterations", "scorr_dq_coeff", "vort_epsilon",
                 "enable_scorr", "enable_xsph", "enable_vorticity",
                 "plane_restitution", "plane_friction", "per_plane_friction"}
      "jitter": {"amplitude", "seed"}  -- U(-a, a) per coordinate (SplitMix64)
    With "per_plane_friction": true, each collision's own "friction" (the key
    the reference scene files carry and the reference loader drops) applies
    to its plane; a collision without one takes "plane_friction". Without
    that switch the per-collision values are ignored, as in the reference.
    """
    import json

    f32 = np.float32
    with open(path) as fh:
        root = json.load(fh)
    if not isinstance(root.get("fluid"), dict):
        raise ValueError("Scene JSON missing fluid object.")
    fl = root["fluid"]
    p = default_params()
    for key, field in (("particle_mass", "particle_mass"), ("density", "density"), ("h", "h"),
                       ("epsilon", "epsilon"), ("k", "scorr_k"), ("c", "visc_c")):
        if key in fl:
            setattr(p, field, float(f32(fl[key])))
    if "n" in fl:
        p.scorr_n = int(fl["n"])
    if "external_forces" in root:
        fx, fy, fz = root["external_forces"]
        p.external_force[0], p.external_force[1], p.external_force[2] = float(f32(fx)), float(f32(fy)), float(f32(fz))
    spacing = f32(0)
    from_mass = False
    if f32(p.density) > 0 and f32(p.particle_mass) > 0:
        spacing = _cbrtf(f32(p.particle_mass) / f32(p.density))
        from_mass = True
    if spacing <= 0 and f32(p.particle_radius) > 0:
        spacing = f32(p.particle_radius) * f32(2.0)
    if spacing <= 0:
        spacing = f32(0.02)
    if from_mass or f32(p.particle_radius) <= 0:
        p.particle_radius = float(spacing * f32(0.5))
    if f32(p.h) <= 0:
        p.h = float(f32(2.5) * spacing)
    if not isinstance(fl.get("shape"), list):
        raise ValueError("Fluid shape must be an array.")
    half = spacing * f32(0.5)
    blocks_p, blocks_v = [], []
    for shape in fl["shape"]:
        kind = shape.get("type")
        vel = [f32(c) for c in shape.get("velocity", (0, 0, 0))]
        o = [f32(c) for c in shape["origin"]]
        if kind == "cube":
            size = [f32(c) for c in shape["size"]]
            ax = [_fill_axis(f32(o[d] + half), f32(o[d] + size[d]), spacing) for d in range(3)]
            xx, yy, zz = np.meshgrid(*ax, indexing="ij")  # x outermost, z innermost
            pts = np.stack([xx.ravel(), yy.ravel(), zz.ravel()])
        elif kind == "sphere":
            r = f32(shape["radius"])
            ax = [_fill_axis(f32(f32(o[d] - r) + half), f32(o[d] + r), spacing) for d in range(3)]
            xx, yy, zz = np.meshgrid(*ax, indexing="ij")
            dx, dy, dz = (xx - o[0]).astype(np.float32), (yy - o[1]).astype(np.float32), (zz - o[2]).astype(np.float32)
            keep = ((dx * dx + dy * dy) + dz * dz) < f32(r * r)
            pts = np.stack([xx[keep], yy[keep], zz[keep]])
        else:
            raise ValueError(f"Unsupported shape type: {kind}")
        blocks_p.append(pts.astype(np.float32))
        blocks_v.append(np.repeat(np.array(vel, np.float32)[:, None], pts.shape[1], axis=1))
    pos = np.concatenate(blocks_p, axis=1) if blocks_p else np.zeros((3, 0), np.float32)
    vel = np.concatenate(blocks_v, axis=1) if blocks_v else np.zeros((3, 0), np.float32)
    p.plane_count = 0
    plane_mu = []
    for entry in root.get("collisions", []):
        if entry.get("type") != "plane":
            raise ValueError(f"Unsupported collision type: {entry.get('type')}")
        px_, py_, pz_ = (f32(c) for c in entry["point"])
        nx, ny, nz = (f32(c) for c in entry["normal"])
        len_sq = (nx * nx + ny * ny) + nz * nz
        if len_sq <= 0:
            raise ValueError("Collision normal must be non-zero.")
        inv = f32(1) / np.sqrt(len_sq, dtype=np.float32)
        nx, ny, nz = nx * inv, ny * inv, nz * inv
        d = (nx * px_ + ny * py_) + nz * pz_
        i = p.plane_count
        if i >= MAX_PLANES:
            raise ValueError("too many planes")
        p.plane_nx[i], p.plane_ny[i], p.plane_nz[i], p.plane_d[i] = float(nx), float(ny), float(nz), float(d)
        p.plane_count = i + 1
        plane_mu.append(entry.get("friction"))
    solver = root.get("solver", {})
    for key, field in (("dt", "dt"), ("scorr_dq_coeff", "scorr_dq_coeff"), ("vort_epsilon", "vort_epsilon"),
                       ("plane_restitution", "plane_restitution"), ("plane_friction", "plane_friction")):
        if key in solver:
            setattr(p, field, float(f32(solver[key])))
    if "iterations" in solver:
        p.solver_iterations = int(solver["iterations"])
    for key in ("enable_scorr", "enable_xsph", "enable_vorticity"):
        if key in solver:
            setattr(p, key, int(bool(solver[key])))
    if solver.get("per_plane_friction", False):
        set_plane_friction(p, [p.plane_friction if mu is None else mu for mu in plane_mu])
    if "jitter" in root:
        pos = jitter(pos, float(root["jitter"].get("amplitude", 0.0)), int(root["jitter"].get("seed", 0)))
    import os

    return Scene(os.path.splitext(os.path.basename(path))[0], p, pos, vel, steps=1, info={"path": path})


# ---------------------------------------------------------------------------
# Fills generated on the device (fluid_fill_block / fluid_fill_shape): the
# same particles as init_block + jitter and the scene file's shapes above, bit
# for bit, written straight into device memory.

def _device_rows(count: int, device: int):
    import torch

    return torch.empty((3, count), dtype=torch.float32, device=torch.device("cuda", device))


def _row_ptrs(t):
    import ctypes

    base = t.data_ptr()
    return [ctypes.c_void_p(base + k * t.stride(0) * 4) for k in range(3)]


def fill_block_device(nx: int, ny: int, nz: int, origin, spacing: float, jitter_amplitude: float = 0.0,
                      seed: int = 0, first: int = 0, device: int = 0):
    """init_block (+ jitter with the same draws as `jitter`, the first particle
    taking draw 3 * first + 1) generated on the GPU; returns a (3, N) float32
    tensor on that device."""
    from fluidsimulator_gb300 import _capi

    lib = _capi.load()
    out = _device_rows(nx * ny * nz, device)
    rc = lib.fluid_fill_block(nx, ny, nz, float(np.float32(origin[0])), float(np.float32(origin[1])),
                              float(np.float32(origin[2])), float(np.float32(spacing)), float(jitter_amplitude),
                              int(seed) & 0xFFFFFFFFFFFFFFFF, int(first), *_row_ptrs(out), None)
    if rc != 0:
        raise RuntimeError(f"fluid_fill_block failed with status {rc}")
    return out


def fill_shape_device(kind: str, origin, extent, spacing: float, velocity=(0.0, 0.0, 0.0), device: int = 0):
    """A scene file's cube (extent = size) or sphere (extent = (radius,)) fill
    generated on the GPU; returns (pos, vel) (3, N) float32 tensors."""
    import ctypes

    from fluidsimulator_gb300 import _capi

    lib = _capi.load()
    k = {"cube": 0, "sphere": 1}[kind]
    o = (ctypes.c_float * 3)(*[float(np.float32(v)) for v in origin])
    ext = list(extent) + [0.0] * (3 - len(extent))
    e = (ctypes.c_float * 3)(*[float(np.float32(v)) for v in ext])
    v = (ctypes.c_float * 3)(*[float(np.float32(c)) for c in velocity])
    count = ctypes.c_int64(0)
    sp = float(np.float32(spacing))
    rc = lib.fluid_fill_shape(k, o, e, sp, v, None, None, None, None, None, None, 0, ctypes.byref(count), None)
    if rc not in (0, 3):
        raise RuntimeError(f"fluid_fill_shape failed with status {rc}")
    pos, vel = _device_rows(count.value, device), _device_rows(count.value, device)
    if count.value:
        rc = lib.fluid_fill_shape(k, o, e, sp, v, *_row_ptrs(pos), *_row_ptrs(vel), count.value, ctypes.byref(count),
                                  None)
        if rc != 0:
            raise RuntimeError(f"fluid_fill_shape failed with status {rc}")
    return pos, vel
