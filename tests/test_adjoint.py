"""Adjoint of the PBF step. The oracle's reverse-mode derivative (double
arithmetic, neighbour sets and branches held at the recorded forward) is
checked against central finite differences of the double-precision forward;
the GPU adjoint is checked against the oracle's (test_gpu_adjoint below)."""

import numpy as np
import pytest

from fluidsimulator_gb300 import scenes


def _scene(side=6, seed=1, floor=False):
    """floor: start just above the floor, moving down (plane contacts in
    step 1); "per_plane" also gives each plane its own friction."""
    sc = scenes.differentiable_block(side, seed=seed)
    if floor:
        sc.pos[1] -= np.float32(0.045)
        sc.vel[1] -= np.float32(3.0)
    if floor == "per_plane":
        scenes.set_plane_friction(sc.params, [0.3, 0.0, 0.6, 0.2, 0.9, 0.1])
    return sc


def _run64(oracle_lib, params, pos, vel, steps):
    r = oracle_lib.Oracle(np.float64).run(params, pos.astype(np.float64), vel.astype(np.float64), 0.0, steps)
    return r["pos"], r["vel"]


@pytest.mark.parametrize("floor", [False, True, "per_plane"])
def test_cpu_adjoint_matches_central_differences(oracle_lib, floor):
    sc = _scene(floor=floor)
    rng = np.random.default_rng(3)
    n = sc.count
    x = sc.pos.astype(np.float64)
    v = sc.vel.astype(np.float64)
    gx = rng.standard_normal((3, n))
    gv = rng.standard_normal((3, n))
    gxi, gvi, gc, _, _ = oracle_lib.vjp(sc.params, x, v, gx, gv)
    loss = lambda xo, vo: float(np.sum(gx * xo) + np.sum(gv * vo))  # noqa: E731
    # Small enough that no neighbour or contact branch flips between +eps and
    # -eps (larger steps cross kinks and converge only linearly).
    eps = 1e-8
    for k in range(4):
        dx = rng.standard_normal((3, n))
        dv = rng.standard_normal((3, n))
        lp = loss(*_run64(oracle_lib, sc.params, x + eps * dx, v + eps * dv, 1))
        lm = loss(*_run64(oracle_lib, sc.params, x - eps * dx, v - eps * dv, 1))
        fd = (lp - lm) / (2 * eps)
        ad = float(np.sum(gxi * dx) + np.sum(gvi * dv))
        assert abs(fd - ad) <= 1e-5 * max(1.0, abs(fd)), (k, fd, ad)
    # XSPH coefficient (a float32 parameter: use the representable step)
    c0 = np.float32(sc.params.visc_c)
    cp, cm = np.float32(c0 * np.float32(1.01)), np.float32(c0 * np.float32(0.99))
    pp, pm = sc.params.copy(), sc.params.copy()
    pp.visc_c, pm.visc_c = float(cp), float(cm)
    fd = (loss(*_run64(oracle_lib, pp, x, v, 1)) - loss(*_run64(oracle_lib, pm, x, v, 1))) / (float(cp) - float(cm))
    assert abs(fd - gc) <= 1e-6 * max(1.0, abs(fd)), (fd, gc)


def test_cpu_adjoint_chains_over_steps(oracle_lib):
    # Two steps: derivatives grow ~10-100x per step (the Jacobi update scales
    # by 1/m), so longer chains need steps far below any kink distance.
    sc = _scene(side=5, seed=2)
    rng = np.random.default_rng(5)
    n = sc.count
    steps = 2
    states = [(sc.pos.astype(np.float64), sc.vel.astype(np.float64))]
    for _ in range(steps):
        states.append(_run64(oracle_lib, sc.params, *states[-1], 1))
    gx = rng.standard_normal((3, n))
    gv = np.zeros((3, n))
    gc_total = 0.0
    for t in reversed(range(steps)):
        gx, gv, gc, _, _ = oracle_lib.vjp(sc.params, *states[t], gx, gv)
        gc_total += gc
    dv = rng.standard_normal((3, n))
    eps = 1e-8
    gx_final = np.random.default_rng(5).standard_normal((3, n))
    loss = lambda v0: float(np.sum(gx_final * _run64(oracle_lib, sc.params, states[0][0], v0, steps)[0]))  # noqa: E731
    fd = (loss(states[0][1] + eps * dv) - loss(states[0][1] - eps * dv)) / (2 * eps)
    ad = float(np.sum(gv * dv))
    assert abs(fd - ad) <= 1e-5 * max(1.0, abs(fd)), (fd, ad)


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("floor", [False, True, "per_plane"])
def test_gpu_vjp_matches_oracle(cuda_lib, oracle_lib, floor):
    """FP32 GPU adjoint vs the oracle's FP64 adjoint of the same FP32 forward."""
    from fluidsimulator_gb300.solver import Solver

    sc = _scene(side=8, seed=4, floor=floor)
    rng = np.random.default_rng(11)
    n = sc.count
    gx = rng.standard_normal((3, n)).astype(np.float32)
    gv = rng.standard_normal((3, n)).astype(np.float32)
    rx, rv, rc, xo, vo = oracle_lib.vjp(sc.params, sc.pos, sc.vel, gx, gv, fwd32=True)
    s = Solver(0)
    s.configure([sc.params], [n])
    s.upload(sc.pos, sc.vel)
    px, pv, pc = s.step_backward(gx, gv)
    after = s.download()
    np.testing.assert_array_equal(after[0], sc.pos)  # state not advanced
    s.step(1)
    np.testing.assert_array_equal(s.download()[0], xo)  # forward it linearised around
    s.close()
    assert _rel(px, rx) < 1e-4, _rel(px, rx)
    assert _rel(pv, rv) < 1e-4, _rel(pv, rv)
    assert abs(pc[0] - rc) <= 1e-4 * abs(rc), (pc[0], rc)


@pytest.mark.gpu
def test_gpu_trajectory_backward_with_checkpoints(cuda_lib, oracle_lib):
    from fluidsimulator_gb300.solver import Solver

    sc = _scene(side=6, seed=6)
    n = sc.count
    steps, every = 5, 2
    s = Solver(0)
    s.configure([sc.params], [n])
    s.upload(sc.pos, sc.vel)
    s.record(steps, every)
    xf, vf = s.download()
    # centre-of-mass loss |COM - target|^2
    target = np.array([1.5, 0.3, 1.0])
    com = xf.astype(np.float64).mean(axis=1)
    gxf = np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1).astype(np.float32)
    gvf = np.zeros((3, n), np.float32)
    gx0, gv0, gc = s.backward(gxf, gvf)
    np.testing.assert_array_equal(s.download()[0], xf)  # left at the final state
    # record() tapes its last segment for the first backward(); a second
    # backward(), or one after step_backward() reused the tapes, recomputes it
    for between in (None, "step_backward"):
        if between:
            s.upload(sc.pos, sc.vel)
            s.record(steps, every)
            s.step_backward(gxf, gvf)
        again = s.backward(gxf, gvf)
        np.testing.assert_array_equal(again[0], gx0)
        np.testing.assert_array_equal(again[1], gv0)
    s.close()
    # oracle: chain of single-step VJPs around the float32 trajectory
    states = [(sc.pos, sc.vel)]
    for _ in range(steps):
        r = oracle_lib.Oracle().run(sc.params, *states[-1], 0.0, 1)
        states.append((r["pos"], r["vel"]))
    np.testing.assert_array_equal(states[-1][0], xf)
    gx, gv, gct = gxf.astype(np.float64), gvf.astype(np.float64), 0.0
    for t in reversed(range(steps)):
        gx, gv, c, _, _ = oracle_lib.vjp(sc.params, *states[t], gx, gv, fwd32=True)
        gct += c
    assert _rel(gv0, gv) < 1e-3, _rel(gv0, gv)
    assert _rel(gx0, gx) < 1e-3, _rel(gx0, gx)
    assert abs(gc[0] - gct) <= 1e-3 * abs(gct), (gc[0], gct)


@pytest.mark.gpu
def test_gpu_adjoint_per_scene_in_a_batch(cuda_lib):
    from fluidsimulator_gb300.solver import Solver

    a, b = _scene(side=6, seed=7), _scene(side=5, seed=8, floor=True)
    rng = np.random.default_rng(2)
    ga = [rng.standard_normal((3, a.count)).astype(np.float32) for _ in range(2)]
    gb = [rng.standard_normal((3, b.count)).astype(np.float32) for _ in range(2)]
    single = []
    for sc, g in ((a, ga), (b, gb)):
        s = Solver(0)
        s.configure([sc.params], [sc.count])
        s.upload(sc.pos, sc.vel)
        single.append(s.step_backward(*g))
        s.close()
    s = Solver(0)
    s.configure([a.params, b.params], [a.count, b.count])
    s.upload(np.concatenate([a.pos, b.pos], 1), np.concatenate([a.vel, b.vel], 1))
    px, pv, pc = s.step_backward(np.concatenate([ga[0], gb[0]], 1), np.concatenate([ga[1], gb[1]], 1))
    s.close()
    np.testing.assert_allclose(px[:, :a.count], single[0][0], rtol=1e-5, atol=1e-5 * np.abs(single[0][0]).max())
    np.testing.assert_allclose(pv[:, a.count:], single[1][1], rtol=1e-5, atol=1e-5 * np.abs(single[1][1]).max())
    np.testing.assert_allclose(pc, [single[0][2][0], single[1][2][0]], rtol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("veps", [0.0005, 0.5])
def test_gpu_vjp_with_vorticity_matches_oracle(cuda_lib, oracle_lib, veps):
    """All three flags on (vorticity at the benchmark's 5e-4 and the
    reference default 0.5), plane contacts on the floor."""
    from fluidsimulator_gb300.solver import Solver

    sc = _scene(side=8, seed=12, floor=True)
    sc.params.enable_vorticity = 1
    sc.params.vort_epsilon = veps
    rng = np.random.default_rng(17)
    n = sc.count
    gx = rng.standard_normal((3, n)).astype(np.float32)
    gv = rng.standard_normal((3, n)).astype(np.float32)
    rx, rv, rc, _, _ = oracle_lib.vjp(sc.params, sc.pos, sc.vel, gx, gv, fwd32=True)
    s = Solver(0)
    s.configure([sc.params], [n])
    s.upload(sc.pos, sc.vel)
    px, pv, pc = s.step_backward(gx, gv)
    s.close()
    # FP32 against FP64: the normalisation N = eta/|eta| amplifies rounding
    # where |eta| is small, so the strong-confinement case gets 5e-4 on the
    # state gradients and 2e-3 on dL/dc (a sum over all particles).
    tol = 1e-4 if veps < 0.01 else 5e-4
    assert _rel(px, rx) < tol, _rel(px, rx)
    assert _rel(pv, rv) < tol, _rel(pv, rv)
    assert abs(pc[0] - rc) <= (tol if veps < 0.01 else 2e-3) * abs(rc), (pc[0], rc)


def _com_cotangent(x, target):
    n = x.shape[1]
    com = np.asarray(x, np.float64).mean(axis=1)
    return np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1)


_TARGET = np.array([1.5, 0.3, 1.0])


def _fp64_adjoint(oracle_lib, sc, horizon, fwd32):
    """dL/dx0, dL/dv0, dL/dc of the centre-of-mass loss by the oracle's FP64
    adjoint, chained over the FP32 (fwd32) or FP64 trajectory of the scene;
    also returns the trajectory."""
    dt = np.float32 if fwd32 else np.float64
    o = oracle_lib.Oracle(dt)
    states = [(sc.pos.astype(dt), sc.vel.astype(dt))]
    for _ in range(horizon):
        r = o.run(sc.params, *states[-1], 0.0, 1)
        states.append((r["pos"], r["vel"]))
    g = _com_cotangent(states[-1][0], _TARGET)
    gv = np.zeros_like(g)
    gc = 0.0
    for t in reversed(range(horizon)):
        g, gv, c, _, _ = oracle_lib.vjp(sc.params, *states[t], g, gv, fwd32=fwd32)
        gc += c
    return g, gv, gc, states


def _gpu_grad(s, scene, horizon, every=10):
    n = scene.count
    s.set_params([scene.params])
    s.upload(scene.pos, scene.vel)
    s.record(horizon, every)
    x, _ = s.download()
    gxf = _com_cotangent(x, _TARGET).astype(np.float32)
    return s.backward(gxf, np.zeros((3, n), np.float32)), x


def test_cpu_adjoint_is_the_derivative_of_each_late_step(oracle_lib):
    """The 32^3 differentiable scene, unit-mass variant, 60 steps. Going
    backwards from the centre-of-mass loss, the cotangent grows by 5-120x per
    step over steps 44-58 (the free-surface particles at the floor's edge).
    Each of the last ten steps' vector-Jacobian products, applied to the
    cotangent that actually arrives there, equals the central difference of
    that step along a random direction (step 1e-10: larger steps cross a
    neighbour cut-off or a plane contact and converge only linearly). So the
    chained adjoint is the exact derivative of the discrete map and the growth
    is the map's own sensitivity, not an instability of the adjoint; central
    differences of the whole 60-step loss cannot show it, since their linear
    regime would need a step below 1e-17."""
    sc = scenes.differentiable_block(32, seed=0, unit_mass=True)
    n = sc.count
    o = oracle_lib.Oracle(np.float64)
    horizon, window = 60, 10
    states = [(sc.pos.astype(np.float64), sc.vel.astype(np.float64))]
    for _ in range(horizon):
        r = o.run(sc.params, *states[-1], 0.0, 1)
        states.append((r["pos"], r["vel"]))
    g = _com_cotangent(states[-1][0], _TARGET)
    gv = np.zeros_like(g)
    rng = np.random.default_rng(1)
    growth = 1.0
    for t in reversed(range(horizon - window, horizon)):
        scale = np.sqrt(np.sum(g * g) + np.sum(gv * gv))
        gx1, gv1 = g / scale, gv / scale
        gx0, gv0, _, _, _ = oracle_lib.vjp(sc.params, *states[t], gx1, gv1)
        dx, dv = rng.standard_normal((3, n)), rng.standard_normal((3, n))
        eps = 1e-10
        rp = o.run(sc.params, states[t][0] + eps * dx, states[t][1] + eps * dv, 0.0, 1)
        rm = o.run(sc.params, states[t][0] - eps * dx, states[t][1] - eps * dv, 0.0, 1)
        fd = (np.sum(gx1 * (rp["pos"] - rm["pos"])) + np.sum(gv1 * (rp["vel"] - rm["vel"]))) / (2 * eps)
        ad = float(np.sum(gx0 * dx) + np.sum(gv0 * dv))
        assert abs(fd - ad) <= 1e-4 * abs(ad), (t, fd, ad)
        step_growth = float(np.sqrt(np.sum(gx0 * gx0) + np.sum(gv0 * gv0)))
        growth *= step_growth
        g, gv = gx0 * scale, gv0 * scale
    assert growth > 1e6, growth  # the sensitivity is real and large


@pytest.mark.gpu
def test_differentiable_scene_gradients_match_fp64(cuda_lib, oracle_lib):
    """The 32^3 differentiable scene as specified (m = rho0 sp^3, XSPH c =
    0.01, s_corr, loss |COM - (1.5, 0.3, 1.0)|^2), 5 steps through record /
    backward: dL/dv0, dL/dx0 and dL/dc against the oracle's FP64 adjoint of
    the same FP32 trajectory. Its gradient grows ~10^3 per step (the Jacobi
    update scales by 1/m) and leaves the FP32 range after ~10 steps; the
    unit-mass variant below carries the 60-step checks."""
    from fluidsimulator_gb300.solver import Solver

    sc = scenes.differentiable_block(32, seed=0)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    horizon = 5
    g, gv, gc_ref, _ = _fp64_adjoint(oracle_lib, sc, horizon, fwd32=True)
    (gx0, gv0, gc), _ = _gpu_grad(s, sc, horizon)
    s.close()
    rel_v, rel_x = _rel(gv0, gv), _rel(gx0, g)
    rel_c = abs(gc[0] - gc_ref) / abs(gc_ref)
    print(f"fp64 adjoint, horizon {horizon}: dL/dv0 {rel_v:.2e}, dL/dx0 {rel_x:.2e}, dL/dc {rel_c:.2e}")
    assert rel_v < 1e-4 and rel_x < 1e-4 and rel_c < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("horizon", [20, 60])
def test_unit_mass_gradients_match_fp64_adjoint(cuda_lib, oracle_lib, horizon):
    """Unit-mass variant (m = 1, rho0 = 1/sp^3) of the 32^3 differentiable
    scene over 20 steps and over the full 60 with checkpoints every 10 (the
    60-step backward pass recomputes five checkpoint segments and crosses five
    boundaries): the GPU's FP32 dL/dv0, dL/dx0 and dL/dc against the oracle's
    FP64 adjoint of the same FP32 trajectory, within 1e-3. The gradient
    reaches ~1e15 at 60 steps (the map's own sensitivity; see the CPU test
    above)."""
    from fluidsimulator_gb300.solver import Solver

    um = scenes.differentiable_block(32, seed=0, unit_mass=True)
    g, gv, gc_ref, states = _fp64_adjoint(oracle_lib, um, horizon, fwd32=True)
    s = Solver(0)
    s.configure([um.params], [um.count])
    (gx0, gv0, gc), xf = _gpu_grad(s, um, horizon, every=10)
    s.close()
    np.testing.assert_array_equal(xf, states[-1][0])  # the same FP32 trajectory, bit for bit
    rel_v, rel_x = _rel(gv0, gv), _rel(gx0, g)
    rel_c = abs(gc[0] - gc_ref) / abs(gc_ref)
    print(f"unit mass, horizon {horizon}: |dL/dv0| {np.linalg.norm(gv):.3e}; against the FP64 adjoint "
          f"dL/dv0 {rel_v:.2e}, dL/dx0 {rel_x:.2e}, dL/dc {rel_c:.2e}")
    assert rel_v < 1e-3 and rel_x < 1e-3 and rel_c < 1e-3


def test_cpu_adjoint_matches_central_differences_at_horizon_20(oracle_lib):
    """The oracle's FP64 adjoint, chained over 20 steps of the FP64 trajectory
    of the 32^3 unit-mass differentiable scene, against central differences
    of the FP64 forward (step 1e-8, 4 random directions of unit RMS) and of
    the XSPH coefficient (16 float32 ulps): the reverse mode is the derivative
    of the map it differentiates, within 1e-4."""
    um = scenes.differentiable_block(32, seed=0, unit_mass=True)
    n = um.count
    horizon = 20
    _, gv, gc, states = _fp64_adjoint(oracle_lib, um, horizon, fwd32=False)
    o = oracle_lib.Oracle(np.float64)

    def loss(v0, params=um.params):
        r = o.run(params, states[0][0], v0, 0.0, horizon)
        return float(np.sum((r["pos"].mean(axis=1) - _TARGET) ** 2))

    rng = np.random.default_rng(7)
    for _ in range(4):
        d = rng.standard_normal((3, n))
        d /= np.sqrt(np.mean(d * d))
        fd = (loss(states[0][1] + 1e-8 * d) - loss(states[0][1] - 1e-8 * d)) / 2e-8
        ad = float(np.sum(gv * d))
        assert abs(fd - ad) <= 1e-4 * abs(ad), (fd, ad)
    c0 = np.float32(um.params.visc_c)
    ulp = np.nextafter(c0, np.float32(1.0), dtype=np.float32) - c0
    pp, pm = um.params.copy(), um.params.copy()
    pp.visc_c, pm.visc_c = float(np.float32(c0 + 16 * ulp)), float(np.float32(c0 - 16 * ulp))
    fd_c = (loss(states[0][1], pp) - loss(states[0][1], pm)) / (pp.visc_c - pm.visc_c)
    assert abs(fd_c - gc) <= 1e-4 * abs(gc), (fd_c, gc)


@pytest.mark.gpu
def test_unit_mass_gradients_match_central_differences(cuda_lib, oracle_lib):
    """Unit-mass variant of the 32^3 differentiable scene: the GPU's dL/dv0
    along 16 random directions, and dL/dc, against central differences of the
    FP64 forward (velocity step 1e-8 along directions of unit RMS; XSPH step
    16 float32 ulps of c), within 1e-3, at horizon 10. A step sweep on this
    scene (1e-7, 1e-8, 1e-9) agrees with the FP64 adjoint to 1e-5 at 1e-8;
    1e-3 or 1e-4 already crosses neighbour cut-offs and plane contacts.

    The GPU linearises around the FP32 trajectory and the differences around
    the FP64 one, so each directional derivative differs by the trajectories'
    divergence as well (median ~1e-4 at horizon 10). By horizon 20 the two
    trajectories have separated enough that their gradients differ by a few
    per cent (measured: median 2.5e-2), so beyond 10 steps the GPU is held to
    the FP64 adjoint of its own trajectory (the test above) and the FP64
    adjoint to central differences of the FP64 forward (the CPU test above).
    Its error is measured against the
    gradient's RMS directional derivative |dL/dv0| (for directions of unit
    RMS, E[(g . d)^2] = |g|^2): a direction nearly orthogonal to the gradient
    has a small derivative whose own relative error says nothing about the
    gradient's. The median of the per-direction relative errors is held to
    1e-3 as well."""
    from fluidsimulator_gb300.solver import Solver

    um = scenes.differentiable_block(32, seed=0, unit_mass=True)
    n = um.count
    horizon = 10
    s = Solver(0)
    s.configure([um.params], [n])
    (_, gv0, gc), _ = _gpu_grad(s, um, horizon)
    s.close()
    o = oracle_lib.Oracle(np.float64)
    x64, v64 = um.pos.astype(np.float64), um.vel.astype(np.float64)

    def loss(v0, params=um.params):
        r = o.run(params, x64, v0, 0.0, horizon)
        return float(np.sum((r["pos"].mean(axis=1) - _TARGET) ** 2))

    rng = np.random.default_rng(7)
    g64 = gv0.astype(np.float64)
    gnorm = float(np.linalg.norm(g64))
    rels, errs = [], []
    for _ in range(16):
        d = rng.standard_normal((3, n))
        d /= np.sqrt(np.mean(d * d))
        eps = 1e-8
        fd = (loss(v64 + eps * d) - loss(v64 - eps * d)) / (2 * eps)
        ad = float(np.sum(g64 * d))
        rels.append(abs(fd - ad) / max(abs(fd), abs(ad), 1e-30))
        errs.append(abs(fd - ad) / gnorm)
    c0 = np.float32(um.params.visc_c)
    ulp = np.nextafter(c0, np.float32(1.0), dtype=np.float32) - c0
    pp, pm = um.params.copy(), um.params.copy()
    pp.visc_c, pm.visc_c = float(np.float32(c0 + 16 * ulp)), float(np.float32(c0 - 16 * ulp))
    fd_c = (loss(v64, pp) - loss(v64, pm)) / (pp.visc_c - pm.visc_c)
    rel_c = abs(fd_c - gc[0]) / abs(fd_c)
    print(f"unit mass, horizon {horizon}: dL/dv0 against FP64 central differences, 16 directions: error "
          f"/ |dL/dv0| max {max(errs):.2e}; per-direction relative max {max(rels):.2e}, median "
          f"{np.median(rels):.2e}; dL/dc rel {rel_c:.2e}")
    assert max(errs) < 1e-3
    assert np.median(rels) < 1e-3
    assert rel_c < 1e-3
