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


@pytest.mark.gpu
def test_differentiable_scene_gradients_match_fp64(cuda_lib, oracle_lib):
    """The 32^3 differentiable scene (XSPH c = 0.01, s_corr, loss |COM -
    (1.5, 0.3, 1.0)|^2): over a 5-step horizon through record / backward
    (checkpoints every 10), dL/dv0, dL/dx0 and dL/dc against the oracle's FP64
    adjoint of the same FP32 trajectory; and, on the unit-mass variant (the
    scene as specified is too ill-conditioned for any finite difference),
    dL/dv0 along 4 random directions against central differences of the FP64
    forward (step 1e-6) at horizons 1 and 5."""
    from fluidsimulator_gb300.solver import Solver

    sc = scenes.differentiable_block(32, seed=0)
    n = sc.count
    target = np.array([1.5, 0.3, 1.0])
    s = Solver(0)
    s.configure([sc.params], [n])

    def gpu_grad(scene, horizon):
        s.set_params([scene.params])
        s.upload(scene.pos, scene.vel)
        s.record(horizon, 10)
        x, _ = s.download()
        com = x.astype(np.float64).mean(axis=1)
        gxf = np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1).astype(np.float32)
        return s.backward(gxf, np.zeros((3, n), np.float32))

    horizon = 5
    states = [(sc.pos, sc.vel)]
    for _ in range(horizon):
        r = oracle_lib.Oracle().run(sc.params, *states[-1], 0.0, 1)
        states.append((r["pos"], r["vel"]))
    com = states[-1][0].astype(np.float64).mean(axis=1)
    g = np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1)
    gv = np.zeros((3, n))
    gc_ref = 0.0
    for t in reversed(range(horizon)):
        g, gv, c, _, _ = oracle_lib.vjp(sc.params, *states[t], g, gv, fwd32=True)
        gc_ref += c
    gx0, gv0, gc = gpu_grad(sc, horizon)
    rel_v = np.linalg.norm(gv0 - gv) / np.linalg.norm(gv)
    rel_x = np.linalg.norm(gx0 - g) / np.linalg.norm(g)
    rel_c = abs(gc[0] - gc_ref) / abs(gc_ref)
    print(f"fp64 adjoint, horizon {horizon}: dL/dv0 {rel_v:.2e}, dL/dx0 {rel_x:.2e}, dL/dc {rel_c:.2e}")
    assert rel_v < 1e-4 and rel_x < 1e-4 and rel_c < 1e-4

    um = scenes.differentiable_block(32, seed=0, unit_mass=True)
    rng = np.random.default_rng(7)
    for hz in (1, 5):
        _, gv_um, _ = gpu_grad(um, hz)
        rels = []
        for _ in range(4):
            d = rng.standard_normal((3, n))
            d /= np.sqrt(np.mean(d * d))

            def l64(v0):
                r = oracle_lib.Oracle(np.float64).run(um.params, um.pos.astype(np.float64), v0, 0.0, hz)
                return float(np.sum((r["pos"].mean(axis=1) - target) ** 2))

            e6 = 1e-6
            v64 = um.vel.astype(np.float64)
            fd = (l64(v64 + e6 * d) - l64(v64 - e6 * d)) / (2 * e6)
            ad = float(np.sum(gv_um.astype(np.float64) * d))
            rels.append(abs(fd - ad) / max(abs(fd), abs(ad), 1e-30))
        print(f"unit mass, horizon {hz}: FP64 central differences vs GPU adjoint, max rel {max(rels):.2e}")
        assert max(rels) < 1e-4
    s.close()
