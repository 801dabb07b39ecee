"""GPU parity: the sm_103a step through the C ABI against the golden
fixtures (written from the reference itself) and the live oracle.

The bar is bit-exact: cell keys, sort order and neighbour counts at step 1
(integer work) and, because the kernels follow the reference's float
operations in the reference's order, positions, velocities, rho and lambda
too. The stated floating-point tolerance (max |dx| <= 1e-5 h after one step)
is checked as well, so a failure report shows both."""

import numpy as np
import pytest

from conftest import golden_files, golden_scene, load_golden
from fluidsimulator_gb300 import _capi, scenes
from fluidsimulator_gb300.solver import FluidError, Solver, cuda_step

pytestmark = pytest.mark.gpu

STEP1_INT = ("cell_keys", "sorted_order", "neighbor_counts")
DEBUG = {"cell_keys": _capi.DEBUG_CELL_KEYS, "sorted_order": _capi.DEBUG_SORTED_ORDER,
         "neighbor_counts": _capi.DEBUG_NEIGHBOR_COUNTS, "rho": _capi.DEBUG_RHO, "lambda": _capi.DEBUG_LAMBDA}


def run_gpu(sc, steps, graphs=True, profiling=False, records=False, lanes=None):
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    if lanes is not None:  # else the solver's default shapes
        s.set_tuning({k: {"unroll": 4, "block": 256, "lanes": lanes if k in _capi.LIST_PASSES else 1}
                      for k in _capi.TUNABLE})
    s.set_graphs(graphs)
    s.set_profiling(profiling)
    s.upload(sc.pos, sc.vel)
    s.step(steps)
    pos, vel = s.download()
    out = {"pos": pos, "vel": vel, "time": s.time(), "stats": s.stats()}
    if records:
        for k, w in DEBUG.items():
            out[k] = s.read_debug(w)
    s.close()
    return out


def test_device_present(cuda_lib):
    from fluidsimulator_gb300.solver import device_available

    ok, n, err = device_available()
    assert ok and n >= 1, err


@pytest.mark.parametrize("name", golden_files())
def test_step1_matches_golden(cuda_lib, name):
    p, d = load_golden(name)
    sc = golden_scene(name)
    r = run_gpu(sc, 1, records=True)
    for k in STEP1_INT:
        np.testing.assert_array_equal(r[k], d[f"s1_{k}"], err_msg=k)
    h = np.float32(p.h)
    assert np.max(np.abs(r["pos"] - d["s1_pos"])) <= 1e-5 * h
    for k in ("pos", "vel", "rho", "lambda"):
        np.testing.assert_array_equal(r[k], d[f"s1_{k}"], err_msg=k)
    assert np.float32(r["time"]) == d["s1_time"]


@pytest.mark.parametrize("name", golden_files())
def test_trajectory_matches_golden(cuda_lib, name):
    p, d = load_golden(name)
    sc = golden_scene(name)
    snaps = sorted(int(k[1:].split("_")[0]) for k in d if k.startswith("s") and k.endswith("_pos") and k != "s1_pos")
    for s in snaps:
        r = run_gpu(sc, s)
        np.testing.assert_array_equal(r["pos"], d[f"s{s}_pos"], err_msg=f"pos after {s} steps")
        np.testing.assert_array_equal(r["vel"], d[f"s{s}_vel"], err_msg=f"vel after {s} steps")
        assert np.float32(r["time"]) == d[f"s{s}_time"]


def test_neighbor_statistics_match_golden(cuda_lib):
    # Per-step neighbour pairs / max and density statistics over the whole
    # 240-step plain dam break (4,096 particles) and 60 collapsing steps with
    # all flags on.
    for name in ("dam_break_4096.npz", "dam_break_flags_4096.npz"):
        p, d = load_golden(name)
        sc = golden_scene(name)
        n = len(d["stats_neighbor_pairs"])
        s = Solver(0)
        s.configure([p], [sc.count])
        s.upload(sc.pos, sc.vel)
        pairs, mx, dmean, dmax = [], [], [], []
        for _ in range(n):
            s.step(1)
            st = s.stats()
            pairs.append(st["neighbor_pairs"])
            mx.append(st["neighbor_max"])
            rho = s.read_debug(_capi.DEBUG_RHO).astype(np.float64)
            e = rho / np.float64(p.density) - 1.0
            dmean.append(e.mean())
            dmax.append(e.max())
        s.close()
        np.testing.assert_array_equal(pairs, d["stats_neighbor_pairs"])
        np.testing.assert_array_equal(mx, d["stats_neighbor_max"])
        # Same floats summed in a different order (numpy) -> tiny differences.
        np.testing.assert_allclose(dmean, d["stats_density_mean"], rtol=1e-9, atol=1e-12)
        np.testing.assert_array_equal(dmax, d["stats_density_max"])


def test_graphs_eager_and_profiling_agree(cuda_lib):
    sc = scenes.dam_break(12, seed=4, flags=True)
    a = run_gpu(sc, 15, graphs=True)
    b = run_gpu(sc, 15, graphs=False)
    c = run_gpu(sc, 15, graphs=True, profiling=True)
    for k in ("pos", "vel"):
        np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(a[k], c[k])


def test_batched_scenes_match_each_fixture(cuda_lib):
    names = [n for n in golden_files() if n.startswith("batch")]
    fixtures = [load_golden(n) for n in names]
    scs = [golden_scene(n) for n in names]
    s = Solver(0)
    s.configure([f[0] for f in fixtures], [sc.count for sc in scs])
    s.upload(np.concatenate([sc.pos for sc in scs], axis=1), np.concatenate([sc.vel for sc in scs], axis=1))
    s.step(1)
    order = s.read_debug(_capi.DEBUG_SORTED_ORDER)
    counts = s.read_debug(_capi.DEBUG_NEIGHBOR_COUNTS)
    off = 0
    for (p, d), sc in zip(fixtures, scs):
        np.testing.assert_array_equal(order[off:off + sc.count], d["s1_sorted_order"])
        np.testing.assert_array_equal(counts[off:off + sc.count], d["s1_neighbor_counts"])
        off += sc.count
    s.step(9)
    pos, vel = s.download()
    off = 0
    for k, ((p, d), sc) in enumerate(zip(fixtures, scs)):
        np.testing.assert_array_equal(pos[:, off:off + sc.count], d["s10_pos"])
        np.testing.assert_array_equal(vel[:, off:off + sc.count], d["s10_vel"])
        assert np.float32(s.time(k)) == d["s10_time"]
        off += sc.count
    s.close()


@pytest.mark.parametrize("builder,steps", [
    (lambda: scenes.double_dam_break(24, seed=7), 12),
    (lambda: scenes.falling_block(28, seed=7), 12),
    (lambda: scenes.differentiable_block(20, seed=7), 20),
])
def test_matches_live_oracle(cuda_lib, oracle_lib, builder, steps):
    sc = builder()
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, steps, dump=True)
    b = run_gpu(sc, steps, records=True)
    for k in ("pos", "vel", "neighbor_counts", "rho", "lambda", "cell_keys", "sorted_order"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)


def test_full_size_first_step_1m(cuda_lib, oracle_lib):
    """1,000,000 particles (the throughput scene) at full size: step-1 keys,
    order, counts, positions and velocities equal the oracle's."""
    sc = scenes.falling_block(100, seed=0)
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)
    b = run_gpu(sc, 1, records=True)
    for k in ("cell_keys", "sorted_order", "neighbor_counts", "pos", "vel", "rho", "lambda"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    hist_a = np.bincount(a["neighbor_counts"])
    hist_b = np.bincount(b["neighbor_counts"])
    np.testing.assert_array_equal(hist_a, hist_b)


def test_full_size_double_dam_break_two_steps(cuda_lib, oracle_lib):
    """The 250,000-particle double dam break (two 50^3 blocks, all three
    flags) at full size: after two steps (the collapse has begun: up to ~200
    neighbours) keys, order, counts, rho, lambda, positions and velocities
    equal the oracle's."""
    sc = scenes.double_dam_break(50, seed=0)
    assert sc.count == 250_000
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 2, dump=True)
    b = run_gpu(sc, 2, records=True)
    for k in ("cell_keys", "sorted_order", "neighbor_counts", "rho", "lambda", "pos", "vel"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    assert np.float32(b["time"]) == np.float32(a["time"])


def test_full_size_double_dam_break_into_the_collapse(cuda_lib, oracle_lib):
    """The 250,000-particle double dam break over its first 10 steps, by which
    it has collapsed to ~1,700 neighbours per particle (max ~6,300; the lists
    regrow several times): every step's neighbour-pair total and maximum
    equal the oracle's, the final keys, order, counts, rho, lambda, positions
    and velocities equal the oracle's, and the run's mean and maximum density
    error (rho/rho0 - 1, per step) are within 0.5 % of the CPU run's (they
    are equal here, since every rho is)."""
    sc = scenes.double_dam_break(50, seed=0)
    steps = 10
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, steps, dump=True, records=True)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.upload(sc.pos, sc.vel)
    pairs, mx, dmean, dmax = [], [], [], []
    for _ in range(steps):
        s.step(1)
        st = s.stats()
        pairs.append(st["neighbor_pairs"])
        mx.append(st["neighbor_max"])
        e = s.read_debug(_capi.DEBUG_RHO).astype(np.float64) / np.float64(sc.params.density) - 1.0
        dmean.append(e.mean())
        dmax.append(e.max())
    rec = {k: s.read_debug(w) for k, w in DEBUG.items()}
    pos, vel = s.download()
    regrows = s.stats()["regrows"]
    s.close()
    assert regrows >= 1 and mx[-1] > 1000
    np.testing.assert_array_equal(pairs, a["neighbor_pairs"])
    np.testing.assert_array_equal(mx, a["neighbor_max"])
    for k in DEBUG:
        np.testing.assert_array_equal(rec[k], a[k], err_msg=k)
    np.testing.assert_array_equal(pos, a["pos"])
    np.testing.assert_array_equal(vel, a["vel"])
    # the stated floating-point bar, asserted beside the exact equality
    np.testing.assert_allclose(dmean, a["density_mean"], rtol=5e-3)
    np.testing.assert_allclose(dmax, a["density_max"], rtol=5e-3)
    np.testing.assert_allclose(np.mean(dmean), np.mean(a["density_mean"]), rtol=5e-3)
    assert max(dmax) <= 1.005 * max(a["density_max"])


@pytest.fixture(scope="module")
def differentiable_20_oracle(oracle_lib):
    sc = scenes.differentiable_block(32, seed=0)
    return sc, oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 20, dump=True)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_full_size_differentiable_scene_20_steps(cuda_lib, differentiable_20_oracle, lanes):
    """The 32,768-particle differentiable scene (XSPH and s_corr, initial
    velocities N(0, 0.1^2)) at full size over 20 steps, by which it has
    collapsed to ~380 neighbours per particle (max ~1,700: lists regrow and
    run past the staged and live-bit heads), with 1, 2, 4 and 8 lanes per
    particle in every list pass: the last step's records and the state equal
    the oracle's."""
    sc, a = differentiable_20_oracle
    assert sc.count == 32_768
    b = run_gpu(sc, 20, records=True, lanes=lanes)
    assert b["stats"]["regrows"] >= 1 and b["stats"]["neighbor_max"] > 64
    for k in ("cell_keys", "sorted_order", "neighbor_counts", "rho", "lambda", "pos", "vel"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    assert np.float32(b["time"]) == np.float32(a["time"])


def test_full_size_batch_first_step(cuda_lib, oracle_lib):
    """The 64 batched dam breaks (particle counts U[2k, 64k] from seed 0,
    about 2.1M particles) stepped together in one solver: every scene's
    step-1 keys, order, counts, rho, lambda, positions, velocities and time
    equal the oracle run on that scene alone."""
    scs = scenes.batched_scenes(64, seed=0)
    s = Solver(0)
    s.configure([sc.params for sc in scs], [sc.count for sc in scs])
    s.upload(np.concatenate([sc.pos for sc in scs], axis=1), np.concatenate([sc.vel for sc in scs], axis=1))
    s.step(1)
    rec = {k: s.read_debug(w) for k, w in DEBUG.items()}
    pos, vel = s.download()
    times = [s.time(k) for k in range(len(scs))]
    s.close()
    off = 0
    for k, sc in enumerate(scs):
        a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)
        part = slice(off, off + sc.count)
        for name in DEBUG:
            np.testing.assert_array_equal(rec[name][part], a[name], err_msg=f"scene {k}: {name}")
        np.testing.assert_array_equal(pos[:, part], a["pos"], err_msg=f"scene {k}: pos")
        np.testing.assert_array_equal(vel[:, part], a["vel"], err_msg=f"scene {k}: vel")
        assert np.float32(times[k]) == np.float32(a["time"])
        off += sc.count
    assert off == sum(sc.count for sc in scs) > 2_000_000


def test_stateless_cuda_step_matches_golden(cuda_lib):
    p, d = load_golden("dam_break_4096.npz")
    sc = golden_scene("dam_break_4096.npz")
    pos, vel = sc.pos.copy(), sc.vel.copy()
    t = cuda_step(p, pos, vel, 0.0)
    np.testing.assert_array_equal(pos, d["s1_pos"])
    np.testing.assert_array_equal(vel, d["s1_vel"])
    assert np.float32(t) == d["s1_time"]
    # second call reuses the cached device buffers
    for _ in range(9):
        t = cuda_step(p, pos, vel, t)
    np.testing.assert_array_equal(pos, d["s10_pos"])


def _pinned_copy(a):
    """A page-locked host copy of a float32 array (numpy view of pinned memory)."""
    import torch

    t = torch.empty(a.shape, dtype=torch.float32).pin_memory()
    out = t.numpy()
    out[...] = a
    return out, t


def test_page_locked_host_arrays_are_read_in_place(cuda_lib, oracle_lib):
    """Page-locked caller arrays go straight to the upload / download kernels
    (no staging copies): same bits as pageable arrays and as the oracle,
    through the stateless step and through a solver."""
    p, d = load_golden("dam_break_4096.npz")
    sc = golden_scene("dam_break_4096.npz")
    pos, keep_p = _pinned_copy(sc.pos)
    vel, keep_v = _pinned_copy(sc.vel)
    t = 0.0
    for _ in range(10):
        t = cuda_step(p, pos, vel, t)
    np.testing.assert_array_equal(pos, d["s10_pos"])
    np.testing.assert_array_equal(vel, d["s10_vel"])
    flags = scenes.dam_break(8, seed=3, flags=True)
    ref = oracle_lib.Oracle().run(flags.params, flags.pos, flags.vel, 0.0, 12)
    ip, keep_ip = _pinned_copy(flags.pos)
    iv, keep_iv = _pinned_copy(flags.vel)
    op, keep_op = _pinned_copy(np.zeros_like(flags.pos))
    ov, keep_ov = _pinned_copy(np.zeros_like(flags.vel))
    s = Solver(0)
    s.configure([flags.params], [flags.count])
    s.upload(ip, iv)
    s.step(12)
    s.download(op, ov)
    s.close()
    np.testing.assert_array_equal(op, ref["pos"])
    np.testing.assert_array_equal(ov, ref["vel"])
    # a collapsing scene through the stateless step: the lists regrow and the
    # failed steps are re-run while the result is written out beside them
    grow = scenes.dam_break(12, seed=9, flags=True)
    ref = oracle_lib.Oracle().run(grow.params, grow.pos, grow.vel, 0.0, 30)
    gp, keep_gp = _pinned_copy(grow.pos)
    gv, keep_gv = _pinned_copy(grow.vel)
    t = 0.0
    for _ in range(30):
        t = cuda_step(grow.params, gp, gv, t)
    np.testing.assert_array_equal(gp, ref["pos"])
    np.testing.assert_array_equal(gv, ref["vel"])
    assert np.float32(t) == np.float32(ref["time"])
    del keep_p, keep_v, keep_ip, keep_iv, keep_op, keep_ov, keep_gp, keep_gv


def test_capacity_regrow_keeps_results(cuda_lib, oracle_lib):
    # The flags scene collapses from ~25 to ~500 neighbours: the lists grow
    # several times and every re-run step must still match the oracle.
    sc = scenes.dam_break(12, seed=9, flags=True)
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 50)
    b = run_gpu(sc, 50)
    assert b["stats"]["regrows"] >= 1
    np.testing.assert_array_equal(b["pos"], a["pos"])
    np.testing.assert_array_equal(b["vel"], a["vel"])


@pytest.mark.parametrize("block, lanes", [(128, 1), (256, 1), (512, 1), (256, 4)])
def test_batched_regrow_matches_oracle(cuda_lib, oracle_lib, block, lanes):
    """Several collapsing scenes in one solver: the lists outgrow their
    capacity mid-run (blocks of the list build fail while others proceed) and
    the failed steps are re-run, at every list-pass block size; each scene
    stays bit-exact with the oracle."""
    scs = [scenes.dam_break(n, seed=50 + n, flags=True) for n in (10, 12, 12)]
    refs = [oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 50) for sc in scs]
    s = Solver(0)
    s.configure([sc.params for sc in scs], [sc.count for sc in scs])
    s.set_tuning({k: {"unroll": 4, "block": block, "lanes": lanes if k in _capi.LIST_PASSES else 1}
                  for k in _capi.TUNABLE})
    s.upload(np.concatenate([sc.pos for sc in scs], axis=1), np.concatenate([sc.vel for sc in scs], axis=1))
    s.step(50)
    pos, vel = s.download()
    assert s.stats()["regrows"] >= 1
    s.close()
    off = 0
    for sc, ref in zip(scs, refs):
        np.testing.assert_array_equal(pos[:, off:off + sc.count], ref["pos"])
        np.testing.assert_array_equal(vel[:, off:off + sc.count], ref["vel"])
        off += sc.count


def test_lists_grown_ahead_of_need_match_oracle(cuda_lib, oracle_lib):
    """A collapse stepped one synchronised step at a time: after each step
    the solver reallocates the list buffer ahead of the next step's need, so
    no step outgrows it (the same 40 steps in one call, where growth waits
    for a failure, regrow and re-run three times). Both runs stay bit-exact
    with the oracle."""
    sc = scenes.dam_break(12, seed=7, flags=True)  # 1,728 particles, 25 -> 129 neighbours
    steps = 40
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, steps)
    regrows = {}
    for mode in ("per_step", "one_call"):
        s = Solver(0)
        s.configure([sc.params], [sc.count])
        s.upload(sc.pos, sc.vel)
        if mode == "per_step":
            for _ in range(steps):
                s.step(1)
        else:
            s.step(steps)
        pos, vel = s.download()
        regrows[mode] = s.stats()["regrows"]
        s.close()
        np.testing.assert_array_equal(pos, ref["pos"])
        np.testing.assert_array_equal(vel, ref["vel"])
    assert regrows["per_step"] == 0, regrows
    assert regrows["one_call"] >= 1, regrows


def test_nonfinite_input_reports_error_and_keeps_state(cuda_lib):
    sc = scenes.dam_break(6, seed=1)
    pos = sc.pos.copy()
    pos[1, 17] = np.nan
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.upload(pos, sc.vel)
    with pytest.raises(FluidError) as e:
        s.step(1)
    assert e.value.status == 5  # FLUID_ERR_NONFINITE
    p2, v2 = s.download()
    np.testing.assert_array_equal(p2, pos)
    # the solver stays usable
    s.upload(sc.pos, sc.vel)
    s.step(2)
    s.close()


def test_invalid_parameters_rejected(cuda_lib):
    s = Solver(0)
    p = scenes.dam_break(4).params
    bad = p.copy()
    bad.h = 0.0
    with pytest.raises(FluidError) as e:
        s.configure([bad], [64])
    assert e.value.status == 1
    bad = p.copy()
    bad.solver_iterations = -1
    with pytest.raises(FluidError) as e:
        s.configure([bad], [64])
    assert e.value.status == 1
    with pytest.raises(FluidError):
        s.step(1)  # nothing configured / uploaded
    s.close()


def test_empty_and_tiny_scenes(cuda_lib, oracle_lib):
    p = scenes.dam_break(2).params
    s = Solver(0)
    s.configure([p], [0])
    s.upload(np.zeros((3, 0), np.float32), np.zeros((3, 0), np.float32))
    s.step(3)
    assert s.time() > 0
    s.close()
    for n in (1, 2, 31, 33):
        sc = scenes.dam_break(4, seed=n)
        pos, vel = sc.pos[:, :n].copy(), sc.vel[:, :n].copy()
        s = Solver(0)
        s.configure([sc.params], [n])
        s.upload(pos, vel)
        s.step(5)
        got = s.download()
        s.close()
        ref = oracle_lib.Oracle().run(sc.params, pos, vel, 0.0, 5)
        np.testing.assert_array_equal(got[0], ref["pos"])
        np.testing.assert_array_equal(got[1], ref["vel"])


def test_autotune_keeps_state_and_results(cuda_lib, oracle_lib):
    sc = scenes.dam_break(12, seed=9, flags=True)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.upload(sc.pos, sc.vel)
    s.step(20)
    before = s.download()
    t0 = s.time()
    steps0 = s.stats()["steps"]
    shapes = s.autotune(1)
    after = s.download()
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])
    assert s.time() == t0 and s.stats()["steps"] == steps0
    assert set(shapes) >= {"k_delta", "k_lambda"}
    assert all(v["unroll"] in (2, 4, 8) for v in shapes.values())  # one ahead only when set
    s.step(10)
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 30)
    got = s.download()
    np.testing.assert_array_equal(got[0], ref["pos"])
    np.testing.assert_array_equal(got[1], ref["vel"])
    # extreme shapes give the same numbers
    s.upload(sc.pos, sc.vel)
    s.set_tuning({k: {"unroll": 1, "block": 512} for k in shapes})
    s.step(30)
    got = s.download()
    np.testing.assert_array_equal(got[0], ref["pos"])
    s.close()


def _two_corner_blocks():
    """Two 6^3 blocks at opposite corners of a 9^3 box, h = 0.1: ~6e5 cells
    in the bounding grid, 20-bit keys (three 8-bit passes, two 11-bit)."""
    sp, h = 0.05, 0.1
    p = scenes.base_params(sp, h)
    scenes.init_planes(p, 9.0, 9.0, 9.0)
    scenes.all_flags(p, h)
    a = scenes.init_block(6, 6, 6, (0.05, 0.05, 0.05), sp)
    b = scenes.init_block(6, 6, 6, (8.6, 8.6, 8.6), sp)
    pos = scenes.jitter(np.concatenate([a, b], axis=1), 5e-4, 3)
    return scenes.Scene("two_corner_blocks", p, pos, np.zeros_like(pos), steps=6)


@pytest.mark.parametrize("case", ["small_grid", "wide_grid"])
def test_sort_width_gives_same_permutation(cuda_lib, oracle_lib, case):
    """8-, 9- and 11-bit digits: same cell keys, stable permutation and
    trajectory (small_grid: keys of <= 11 bits, one 11-bit pass against two
    8- or 9-bit ones; wide_grid: 20-bit keys, two 11-bit passes against
    three)."""
    sc = scenes.dam_break(8, seed=5, flags=True) if case == "small_grid" else _two_corner_blocks()
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 6, dump=True)
    out = {}
    for bits in (8, 9, 11):
        s = Solver(0)
        s.configure([sc.params], [sc.count])
        s.set_sort_bits(bits)
        assert s.sort_bits() == bits
        s.upload(sc.pos, sc.vel)
        s.step(6)
        pos, vel = s.download()
        out[bits] = (pos, vel, s.read_debug(_capi.DEBUG_SORTED_ORDER), s.read_debug(_capi.DEBUG_CELL_KEYS))
        s.close()
        np.testing.assert_array_equal(pos, ref["pos"])
        np.testing.assert_array_equal(vel, ref["vel"])
        np.testing.assert_array_equal(out[bits][2], ref["sorted_order"])
        np.testing.assert_array_equal(out[bits][3], ref["cell_keys"])
    for bits in (9, 11):
        for x, y in zip(out[8], out[bits]):
            np.testing.assert_array_equal(x, y)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    for bad in (7, 10, 12):
        with pytest.raises(FluidError):
            s.set_sort_bits(bad)
    s.close()


@pytest.mark.parametrize("bits", [8, 9, 11])
def test_sort_across_many_tiles(cuda_lib, oracle_lib, bits):
    """216,000 particles (106 sort tiles, so every pass chains its look-back
    across tiles): the permutation of step 1 and the state after three steps
    (look-back words reused from step to step) equal the oracle's."""
    sc = scenes.falling_block(60, seed=2)
    one = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)
    three = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 3)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.set_sort_bits(bits)
    s.upload(sc.pos, sc.vel)
    s.step(1)
    np.testing.assert_array_equal(s.read_debug(_capi.DEBUG_SORTED_ORDER), one["sorted_order"])
    np.testing.assert_array_equal(s.read_debug(_capi.DEBUG_CELL_KEYS), one["cell_keys"])
    s.step(2)
    pos, vel = s.download()
    s.close()
    np.testing.assert_array_equal(pos, three["pos"])
    np.testing.assert_array_equal(vel, three["vel"])


@pytest.mark.parametrize("n", [2, 3, 4])
def test_scorr_exponent_variants_match_oracle(cuda_lib, oracle_lib, n):
    """s_corr with n = 2, 3, 4: the delta pass compiled for that exponent
    (every s_corr scene shares it) stays bit-exact with the oracle."""
    sc = scenes.dam_break(8, seed=31 + n, flags=True)
    sc.params.scorr_n = n
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 20)
    got = run_gpu(sc, 20)
    np.testing.assert_array_equal(got["pos"], ref["pos"])
    np.testing.assert_array_equal(got["vel"], ref["vel"])


def test_scorr_exponent_read_per_scene(cuda_lib, oracle_lib):
    """Scenes with different s_corr exponents in one solver take the delta
    pass that reads n per scene; the n = 5 scene goes through powf and is
    held to the accuracy check of _assert_within_fp32_error."""
    scs = []
    for k, n in enumerate((2, 3, 5)):
        sc = scenes.dam_break(6, seed=40 + k, flags=True)
        sc.params.scorr_n = n
        scs.append(sc)
    s = Solver(0)
    s.configure([sc.params for sc in scs], [sc.count for sc in scs])
    s.upload(np.concatenate([sc.pos for sc in scs], axis=1), np.concatenate([sc.vel for sc in scs], axis=1))
    s.step(1)
    pos, vel = s.download()
    s.close()
    off = 0
    for sc in scs:
        ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1)
        got = pos[:, off:off + sc.count]
        if sc.params.scorr_n <= 4:
            np.testing.assert_array_equal(got, ref["pos"])
            np.testing.assert_array_equal(vel[:, off:off + sc.count], ref["vel"])
        else:
            _assert_within_fp32_error(oracle_lib, sc, 1, got)
        off += sc.count


@pytest.mark.parametrize("unroll", [1, 2, 4, 8])
def test_every_unroll_matches_oracle(cuda_lib, oracle_lib, unroll):
    """Each list-pass variant (scalar at 1, two entries per step in paired
    arithmetic from 2 up, odd tails included) gives the oracle's bits, with
    s_corr, XSPH, vorticity and planes on."""
    sc = scenes.dam_break(9, seed=17, flags=True)
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 15)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.set_tuning({k: {"unroll": unroll, "block": 128} for k in _capi.TUNABLE})
    s.upload(sc.pos, sc.vel)
    s.step(15)
    pos, vel = s.download()
    s.close()
    np.testing.assert_array_equal(pos, ref["pos"])
    np.testing.assert_array_equal(vel, ref["vel"])


@pytest.mark.parametrize("lanes", [2, 4, 8])
@pytest.mark.parametrize("block", [128, 512])
def test_every_lane_count_matches_oracle(cuda_lib, oracle_lib, lanes, block):
    """Several lanes per particle in every list pass (rounds of `lanes`
    entries, terms added in list order through shuffles) give the oracle's
    bits over 15 collapsing steps with s_corr, XSPH, vorticity and planes on
    (lists grow past the 64-entry live-bit head and regrow)."""
    sc = scenes.dam_break(9, seed=17, flags=True)
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 15)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.set_tuning({k: {"unroll": 4, "block": block, "lanes": lanes if k in _capi.LIST_PASSES else 1}
                  for k in _capi.TUNABLE})
    assert all(s.tuning()[k]["lanes"] == lanes for k in _capi.LIST_PASSES)
    s.upload(sc.pos, sc.vel)
    s.step(15)
    pos, vel = s.download()
    s.close()
    np.testing.assert_array_equal(pos, ref["pos"])
    np.testing.assert_array_equal(vel, ref["vel"])


def test_mixed_lanes_on_a_one_wave_collapse(cuda_lib, oracle_lib):
    """The 32,768-particle differentiable scene (its launches fill a fifth of
    the SMs) over 20 steps into its collapse (~380 neighbours per particle,
    ~1,700 at most), with a different lane count per list pass, against the
    oracle's keys, order, counts, rho, lambda, positions and velocities."""
    sc = scenes.differentiable_block(32, seed=0)
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 20, dump=True)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    lanes = {"k_lambda": 4, "k_delta": 8, "k_xsph": 2, "k_omega": 4, "k_eta": 1}
    s.set_tuning({k: {"unroll": 2, "block": 256, "lanes": lanes.get(k, 1)} for k in _capi.TUNABLE})
    s.upload(sc.pos, sc.vel)
    s.step(20)
    rec = {k: s.read_debug(w) for k, w in DEBUG.items()}
    pos, vel = s.download()
    s.close()
    for k in DEBUG:
        np.testing.assert_array_equal(rec[k], a[k], err_msg=k)
    np.testing.assert_array_equal(pos, a["pos"])
    np.testing.assert_array_equal(vel, a["vel"])


def test_lanes_are_checked(cuda_lib):
    sc = scenes.dam_break(4, seed=1)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    with pytest.raises(FluidError):
        s.set_tuning({"k_lambda": {"unroll": 4, "block": 256, "lanes": 3}})
    with pytest.raises(FluidError):
        s.set_tuning({"k_nbr_build": {"unroll": 4, "block": 256, "lanes": 2}})
    s.close()


@pytest.mark.parametrize("side, lanes", [(16, 8), (25, 8), (26, 4), (32, 4), (33, 1)])
def test_default_lanes_follow_particle_count(cuda_lib, side, lanes):
    """Lambda and delta default to eight lanes per particle up to 16,384
    particles in all (25^3 = 15,625), four up to 32,768 (26^3 = 17,576 and
    32^3) and one above (33^3 = 35,937); the other list passes to one."""
    sc = scenes.dam_break(side, seed=1)
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    got = {k: v["lanes"] for k, v in s.tuning().items() if k in _capi.LIST_PASSES}
    s.close()
    assert got == {k: lanes if k in ("k_lambda", "k_delta") else 1 for k in _capi.LIST_PASSES}


def test_one_lane_on_a_small_scene_matches_oracle(cuda_lib, oracle_lib):
    """The 4,096-particle dam break (flags on) over 30 steps with one lane in
    every list pass, set explicitly (the default there is eight in lambda and
    delta), against the oracle."""
    sc = scenes.dam_break(16, seed=3, flags=True)
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 30)
    b = run_gpu(sc, 30, lanes=1)
    np.testing.assert_array_equal(b["pos"], ref["pos"])
    np.testing.assert_array_equal(b["vel"], ref["vel"])


def _corners():
    """The oracle's parameter corners plus every combination of the passes
    that follow the Jacobi loop (each takes its own commit path)."""
    base = scenes.dam_break(8, seed=11, flags=True)
    out = []

    def variant(name, frictions=None, **kw):
        v = base.copy()
        for k, val in kw.items():
            setattr(v.params, k, val)
        if frictions is not None:
            scenes.set_plane_friction(v.params, frictions)
        out.append((name, v))

    variant("all_flags")
    variant("scorr_n5", scorr_n=5)
    variant("friction_only", plane_restitution=0.0)
    variant("restitution_only", plane_friction=0.0)
    variant("no_planes", plane_count=0)
    variant("dq_fallback", scorr_dq_coeff=0.0)
    variant("one_iteration", solver_iterations=1)
    variant("xsph_only", enable_vorticity=0, enable_scorr=0)
    variant("vorticity_only", enable_xsph=0, enable_scorr=0)
    variant("scorr_only", enable_xsph=0, enable_vorticity=0)
    variant("no_flags", enable_xsph=0, enable_vorticity=0, enable_scorr=0)
    variant("no_iterations_flags", solver_iterations=0)
    variant("no_iterations_vorticity_only", solver_iterations=0, enable_xsph=0)
    mus = [0.0, 0.7, 0.5, 0.2, 0.05, 1.0]  # x-, x+, floor, ceiling, z-, z+ walls
    variant("per_plane_all_flags", frictions=mus)
    variant("per_plane_xsph_only", frictions=mus, enable_vorticity=0)
    variant("per_plane_no_flags", frictions=mus, enable_xsph=0, enable_vorticity=0, enable_scorr=0)
    variant("per_plane_friction_only", frictions=mus, plane_restitution=0.0, plane_friction=0.0)
    variant("per_plane_all_zero", frictions=[0.0] * 6, plane_restitution=0.0)
    return out


def _assert_within_fp32_error(oracle_lib, sc, steps, got_pos):
    """s_corr with n outside {2, 3, 4}: the reference calls the C library's
    powf, which is not correctly rounded (it differs from the correctly
    rounded power on ~0.07 % of arguments) and which CUDA's powf cannot
    reproduce bit for bit; the Jacobi update scales such an ulp by 1/m. The
    check is then accuracy: the GPU's distance from the FP64 oracle is at
    most twice the FP32 reference's own."""
    ref32 = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, steps)["pos"].astype(np.float64)
    ref64 = oracle_lib.Oracle(np.float64).run(sc.params, sc.pos, sc.vel, 0.0, steps)["pos"]
    cpu_err = np.max(np.abs(ref32 - ref64))
    gpu_err = np.max(np.abs(got_pos.astype(np.float64) - ref64))
    assert gpu_err <= 2.0 * cpu_err + 1e-7 * sc.params.h, (gpu_err, cpu_err)


@pytest.mark.parametrize("name,sc", _corners(), ids=[n for n, _ in _corners()])
def test_parameter_corners_match_oracle(cuda_lib, oracle_lib, name, sc):
    """Every corner bit-exact with the oracle over 12 steps, except
    scorr_n = 5 (the C library's powf; see _assert_within_fp32_error)."""
    steps = 12
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, steps, dump=True)
    got = run_gpu(sc, steps, records=True)
    if name == "scorr_n5":
        one = run_gpu(sc, 1, records=True)
        ref1 = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)
        np.testing.assert_array_equal(one["neighbor_counts"], ref1["neighbor_counts"])
        _assert_within_fp32_error(oracle_lib, sc, 1, one["pos"])
        _assert_within_fp32_error(oracle_lib, sc, steps, got["pos"])
        return
    for k in ("pos", "vel", "neighbor_counts", "rho"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    assert np.float32(got["time"]) == np.float32(ref["time"])


def test_per_plane_friction_read_per_scene(cuda_lib, oracle_lib):
    """Scenes with a single friction and with per-plane frictions in one
    solver: each takes its own planes' scales, bit-exact with the oracle."""
    scs = []
    for k, mus in enumerate((None, [0.9, 0.0, 0.4, 0.0, 0.1, 0.6], [0.0] * 6)):
        sc = scenes.dam_break(7, seed=50 + k, flags=k != 1)
        if mus is not None:
            scenes.set_plane_friction(sc.params, mus)
        scs.append(sc)
    s = Solver(0)
    s.configure([sc.params for sc in scs], [sc.count for sc in scs])
    s.upload(np.concatenate([sc.pos for sc in scs], axis=1), np.concatenate([sc.vel for sc in scs], axis=1))
    s.step(30)
    pos, vel = s.download()
    s.close()
    off = 0
    for sc in scs:
        ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 30)
        np.testing.assert_array_equal(pos[:, off:off + sc.count], ref["pos"])
        np.testing.assert_array_equal(vel[:, off:off + sc.count], ref["vel"])
        off += sc.count


def test_live_bits_with_mixed_scene_flags(cuda_lib, oracle_lib):
    """Scenes with XSPH and vorticity, vorticity only, and XSPH only in one
    solver: the vorticity passes skip the entries XSPH found out of range
    only where XSPH ran (the others' live bits are all set), bit-exact."""
    scs = []
    for k, (xs, vo) in enumerate(((1, 1), (0, 1), (1, 0))):
        sc = scenes.dam_break(7, seed=60 + k, flags=True)
        sc.params.enable_xsph, sc.params.enable_vorticity = xs, vo
        scs.append(sc)
    s = Solver(0)
    s.configure([sc.params for sc in scs], [sc.count for sc in scs])
    s.upload(np.concatenate([sc.pos for sc in scs], axis=1), np.concatenate([sc.vel for sc in scs], axis=1))
    s.step(25)
    pos, vel = s.download()
    s.close()
    off = 0
    for sc in scs:
        ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 25)
        np.testing.assert_array_equal(pos[:, off:off + sc.count], ref["pos"])
        np.testing.assert_array_equal(vel[:, off:off + sc.count], ref["vel"])
        off += sc.count


@pytest.mark.parametrize("unroll, lanes", [(1, 1), (2, 1), (4, 1), (8, 1), (4, 2), (4, 4), (4, 8)])
def test_lists_longer_than_the_live_bit_head(cuda_lib, oracle_lib, unroll, lanes):
    """A dense lattice (spacing 0.03 at h = 0.1, ~150 neighbours): every
    list runs past the 64 entries that carry live bits, so the XSPH and
    vorticity passes go through both halves of their walkers."""
    p = scenes.base_params(0.03, 0.1)
    scenes.init_planes(p, 1.0, 1.0, 1.0)
    scenes.all_flags(p, 0.1)
    pos = scenes.jitter(scenes.init_block(10, 10, 10, (0.2, 0.2, 0.2), 0.03), 5e-4, 8)
    sc = scenes.Scene("dense_block", p, pos, np.zeros_like(pos), steps=1)
    ref = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 1, dump=True)
    assert ref["neighbor_counts"].mean() > 100
    s = Solver(0)
    s.configure([sc.params], [sc.count])
    s.set_tuning({k: {"unroll": unroll, "block": 128, "lanes": lanes if k in _capi.LIST_PASSES else 1}
                  for k in _capi.TUNABLE})
    s.upload(sc.pos, sc.vel)
    s.step(1)
    got_pos, got_vel = s.download()
    s.close()
    np.testing.assert_array_equal(got_pos, ref["pos"])
    np.testing.assert_array_equal(got_vel, ref["vel"])


def test_all_pairs_lists_match_oracle(cuda_lib, oracle_lib):
    """use_uniform_grid = 0: lists in ascending caller index from all pairs
    (core/src/core.cpp:248-268), a different summation order than the grid's."""
    sc = scenes.dam_break(9, seed=21, flags=True)
    sc.params.use_uniform_grid = 0
    a = oracle_lib.Oracle().run(sc.params, sc.pos, sc.vel, 0.0, 12, dump=True)
    b = run_gpu(sc, 12, records=True)
    for k in ("pos", "vel", "neighbor_counts", "rho", "lambda"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    grid = run_gpu(scenes.dam_break(9, seed=21, flags=True), 12)
    assert not np.array_equal(grid["pos"], b["pos"])  # the order does change the floats
