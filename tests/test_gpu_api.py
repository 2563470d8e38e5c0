"""C ABI behaviour on the GPU: state transfer, caller-supplied forces, divergence
detection, empty marker sets, profiling counters and the 16-bit storage forms."""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpkg(built_pkg):
    return built_pkg


def _random_state(shape, seed=0):
    rng = np.random.default_rng(seed)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32)
    return (w * (1.0 + 0.05 * rng.standard_normal(shape + (19,)))).astype(np.float32)


def test_population_round_trip_is_exact(gpkg):
    s = gpkg.Solver(37, 11, 5, 1.6)
    f = _random_state(s.shape)
    s.write_populations(f)
    np.testing.assert_array_equal(s.read_populations(), f)
    s.close()


def test_steps_from_imported_state_match_oracle(gpkg, oracle_mod):
    shape = (40, 12, 6)
    f = _random_state(shape, seed=3)
    s = gpkg.Solver(*shape, 1.55, 1.1, 0.04, -0.006)
    o = oracle_mod.Oracle(*shape, 1.55, 1.1, 0.04, -0.006, [], [], [])
    s.write_populations(f)
    o.set_f(f)
    for _ in range(7):
        s.step()
        o.lbm_step()
    assert rel_l2(s.read_populations(), o.f()) < 1e-6


def test_host_forces_match_oracle(gpkg, oracle_mod):
    shape = (30, 10, 4)
    rng = np.random.default_rng(7)
    F = [(1e-3 * rng.standard_normal(shape)).astype(np.float32) for _ in range(3)]
    s = gpkg.Solver(*shape, 1.3, 1.0, 0.05, 0.0)
    o = oracle_mod.Oracle(*shape, 1.3, 1.0, 0.05, 0.0, [], [], [])
    o.set_forces(*F)
    for _ in range(3):
        s.step_host_force(*F)
        o.lbm_step()
    m = s.read_macro()
    rho, ux, uy, uz = o.macro()
    assert rel_l2(m["rho"], rho) < 1e-6
    assert rel_l2(m["ux"], ux) < 1e-5 and rel_l2(m["uy"], uy) < 1e-4 and rel_l2(m["uz"], uz) < 1e-4


@pytest.mark.parametrize("variant", ["cell", "staged"])
def test_forced_float32_steps_repeat_reference_arithmetic(gpkg, oracle_mod, monkeypatch, variant):
    """Forced float32 cells (the IBM force box; here every cell, through caller-supplied
    forces) collide with the reference's own arithmetic operation for operation --
    _macro_with_force, central moments as 19-term sums, relaxation, raw moments, the back
    transform in M_raw^-1 column order and the Guo term (clbm_moving.py:96-249) -- and the
    streaming, Zou-He inlet and outlet copy are exact or in the reference's order: steps
    from the same state give the oracle's populations and macroscopic fields bit for bit."""
    monkeypatch.setenv("CLBM_KERNEL", variant)
    shape = (37, 12, 5)
    f = _random_state(shape, seed=11)
    rng = np.random.default_rng(12)
    F = [(2e-3 * rng.standard_normal(shape)).astype(np.float32) for _ in range(3)]
    s = gpkg.Solver(*shape, 1.42, 1.0, 0.048, -0.007)
    o = oracle_mod.Oracle(*shape, 1.42, 1.0, 0.048, -0.007, [], [], [])
    s.write_populations(f)
    o.set_f(f)
    o.set_forces(*F)
    for _ in range(6):
        s.step_host_force(*F)
        o.lbm_step()
    np.testing.assert_array_equal(s.read_populations(), o.f())
    m = s.read_macro()
    for k, v in zip(("rho", "ux", "uy", "uz"), o.macro()):
        np.testing.assert_array_equal(m[k], v, err_msg=k)
    s.close()


def test_divergence_is_reported(gpkg):
    s = gpkg.Solver(20, 8, 4, 1.5)
    st = s.check()
    assert st["nonfinite"] == 0 and abs(st["rho_min"] - 1.0) < 1e-6
    f = s.read_populations()
    f[3, 2, 1, 5] = np.nan
    s.write_populations(f)
    with pytest.raises(gpkg.DivergedError):
        s.check()
    f = s.read_populations()
    f[np.isnan(f)] = 0.0
    f[5, 3, 2, :] *= 0.2           # rho = 0.2 < 0.3 at one cell
    s.write_populations(f)
    with pytest.raises(gpkg.DivergedError):
        s.check(rho_floor=0.3)
    s.close()


def test_graph_replayed_run_stops_itself_on_divergence(gpkg):
    """The device divergence monitor (every collision tests its density) inside the captured
    time loop: a NaN injected host-side makes a graph-replayed run stop on its own within
    five replays, instead of running its 400 steps, and clbm_synchronize keeps reporting it
    until a new state is written (main_moving.py:143-145)."""
    cfg = gpkg.wing_case(64, 32, 6, 10.0, re=30.0)
    sim = gpkg.Simulation(cfg)
    sim.run(24, graph=True)
    sim.solver.synchronize()                       # healthy so far: no report
    f = sim.solver.read_populations()
    good = f.copy()
    f[40, 20, 3, 7] = np.nan
    sim.solver.write_populations(f)
    before = sim.ibm.step_count()
    with pytest.raises(gpkg.DivergedError) as ei:
        sim.run(400, graph=True)
    assert "stopped after" in str(ei.value)
    ran = sim.ibm.step_count() - before
    assert 8 <= ran <= 1 + 6 * 8, ran
    with pytest.raises(gpkg.DivergedError):
        sim.solver.synchronize()
    sim.solver.write_populations(good)             # a new state clears the record
    sim.run(16, graph=True)
    sim.solver.synchronize()
    sim.close()


def test_density_floor_of_the_monitor(gpkg):
    """A density of 0.2 at one cell is caught by the default floor (0.3, as
    main_moving.py:143) in direct steps too; with a negative floor only non-finite values
    are."""
    s = gpkg.Solver(20, 8, 4, 1.5)
    f = s.read_populations()
    f[5, 3, 2, :] *= 0.2
    s.write_populations(f)
    s.step()
    with pytest.raises(gpkg.DivergedError):
        s.synchronize()
    s.set_rho_floor(-1.0)
    s.write_populations(f)
    s.step()
    s.synchronize()
    s.close()


def test_empty_marker_set_and_counters(gpkg):
    s = gpkg.Solver(24, 10, 4, 1.5)
    ibm = gpkg.IBM(s, [], [], [])
    ibm.compute_force(10.0, 5.0, 0.1, 0.0, 0.0, 0.0)
    s.profile(True)
    s.step(ibm)
    s.step(ibm)
    p = s.profile_read()
    # an IBM step is two stream-collide launches: the bulk pass and the force-box pass
    assert p["fused_launches"] == 4 and p["fused_ms"] > 0
    fx, fy, fz = ibm.read_forces()
    assert not fx.any() and not fy.any()
    assert ibm.step_count() == 1
    np.testing.assert_array_equal(ibm.force_history(1), np.zeros((1, 4)))
    s.close()


def test_solver_destroyed_before_ibm(gpkg):
    """Destroying the solver first orphans its IBM: later calls report CLBM_ERR_STATE and
    destroying the IBM is still safe (Python finalisers run in arbitrary order)."""
    s = gpkg.Solver(24, 10, 4, 1.5)
    ibm = gpkg.IBM(s, [0.0], [0.0], [1.0])
    gpkg.lib().clbm_destroy(s._h)
    s._h = None
    with pytest.raises(gpkg.CLBMError) as ei:
        ibm.compute_force(10.0, 5.0, 0.0, 0.0, 0.0, 0.0)
    assert ei.value.code == 4
    ibm.close()


def test_forces_persist_after_step_like_reference(gpkg):
    cfg = gpkg.wing_case(48, 24, 4, 8.0, re=20.0)
    sim = gpkg.Simulation(cfg)
    sim.ibm.compute_force(*cfg.motion_state(1))
    before = sim.ibm.read_forces()
    sim.solver.step(sim.ibm)
    after = sim.ibm.read_forces()
    np.testing.assert_array_equal(before[0], after[0])
    assert np.abs(before[0]).max() <= 0.05 and np.abs(before[0]).max() > 0
    sim.close()


W19 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


@pytest.fixture
def kernel_variant(request, monkeypatch):
    """Force one full-grid stream-collide kernel variant for solvers made in the test."""
    monkeypatch.setenv("CLBM_KERNEL", request.param)
    return request.param


@pytest.mark.parametrize("kernel_variant", ["cell", "pair", "staged"], indirect=True)
@pytest.mark.parametrize("storage,tol", [("f32", 5e-5), ("f16", 5e-3), ("bf16", 4e-2)])
@pytest.mark.parametrize("shape", [(37, 9, 5), (64, 6, 3), (3, 4, 2), (301, 5, 2), (258, 3, 3),
                                   (515, 3, 2)])
@pytest.mark.parametrize("forced", [False, True])
def test_kernel_variants_edges(gpkg, oracle_mod, kernel_variant, storage, tol, shape, forced):
    """Every stream-collide variant: odd and even Nx, rows shorter than a warp, segment and
    lane edges, inlet and outlet columns; deviations f - w against the FP64 oracle."""
    rng = np.random.default_rng(11)
    f = (W19 * (1.0 + 0.02 * rng.standard_normal(shape + (19,)))).astype(np.float32)
    F = [(2e-4 * rng.standard_normal(shape)).astype(np.float32) for _ in range(3)]
    s = gpkg.Solver(*shape, 1.45, 1.1, 0.04, 0.01, storage=storage)
    o = oracle_mod.Oracle(*shape, 1.45, 1.1, 0.04, 0.01, [], [], [], real="f64")
    s.write_populations(f)
    o.set_f(f.astype(np.float64))
    if forced:
        o.set_forces(*F)
    for _ in range(4):
        if forced:
            s.step_host_force(*F)
        else:
            s.step()
        o.lbm_step()
    got = s.read_populations().astype(np.float64) - W19
    want = o.f() - W19
    err = rel_l2(got, want)
    assert err < tol, err
    s.close()


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_kernel_variants_are_bitwise_equal(gpkg, monkeypatch, storage):
    """The one-cell, two-cell and staged (TMA) kernels of a storage form run the same
    arithmetic on the same values (the 16-bit forms collide on the deviations f - w in all
    three): identical bits after an IBM run."""
    cfg = gpkg.small_case(storage=storage)
    out = {}
    variants = ("cell", "staged") if storage == "f32" else ("cell", "pair", "staged")
    for v in variants:
        monkeypatch.setenv("CLBM_KERNEL", v)
        sim = gpkg.Simulation(cfg)
        sim.run(30, graph=True)
        out[v] = (sim.solver.read_populations(), sim.ibm.force_history(30))
        sim.close()
    a = out["cell"]
    for v in variants[1:]:
        np.testing.assert_array_equal(out[v][0], a[0])
        np.testing.assert_array_equal(out[v][1], a[1])


def test_bounded_wait_reports_timeout(gpkg):
    """Failure detection on the device: a staged launch whose barrier can never complete
    gives up after a bounded number of polls, sets the status word and returns; the host
    reads the error and the solver stays usable."""
    s = gpkg.Solver(200, 6, 4, 1.5)
    f0 = s.read_populations()
    err = s.selftest_wait_timeout(4096)
    assert err is not None and err.code == 4, err
    np.testing.assert_array_equal(s.read_populations(), f0)
    s.step()
    s.synchronize()
    st = s.check()
    assert st["nonfinite"] == 0
    s.close()


@pytest.mark.parametrize("storage,tol", [("f16", 2e-3), ("bf16", 2e-2)])
def test_shifted_storage_error_against_fp64_oracle(gpkg, oracle_mod, storage, tol):
    """16-bit shifted populations f - w with float32 collision: field and lift/drag error
    against the FP64 oracle of the same case (200x80x16, 300 steps)."""
    cfg = gpkg.small_case(storage=storage)
    sim = gpkg.Simulation(cfg)
    sim.run(300)
    got = sim.solver.read_macro()
    ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                            cfg.X0, cfg.Y0, cfg.Z0, real="f64")
    ref_hist = ref.run(0, 300, cfg.motion())
    rho, ux, uy, _ = ref.macro()
    e_rho = rel_l2(got["rho"] - 1.0, rho - 1.0)
    e_u = rel_l2(got["ux"], ux)
    hist = sim.ibm.force_history(300)
    e_f = rel_l2(hist, ref_hist)
    # mean C_L and C_D over the run (the precision form's target: within 1 % of FP64)
    cg, cr = gpkg.force_coefficients(hist, cfg), gpkg.force_coefficients(ref_hist, cfg)
    e_mean = {k: abs(np.mean(cg[k]) - np.mean(cr[k])) / abs(np.mean(cr[k])) for k in ("cl", "cd")}
    print(f"{storage}: rel L2 (rho-1) {e_rho:.2e}, ux {e_u:.2e}, force history {e_f:.2e}, "
          f"mean C_L {e_mean['cl']:.2e}, mean C_D {e_mean['cd']:.2e}")
    assert e_u < tol and e_f < 10 * tol
    assert e_mean["cl"] < 1e-2 and e_mean["cd"] < 1e-2
    sim.close()


def test_graph_replay_after_a_direct_step_waits_for_its_bulk_pass(gpkg):
    """An IBM step launched directly leaves its bulk pass running on the second stream
    (joined by the next call); a divergence check between runs makes the next run start
    with such a step and then replay the graph already captured. The replay must wait for
    that bulk pass: two chunks with a check between give the bits of one run (600x200x50,
    FP16, where any overlap with the pass changes the stored values)."""
    cfg = gpkg.full_case(storage="f16")
    runs = []
    for chunks in ((400,), (200, 200)):
        sim = gpkg.Simulation(cfg)
        for k in chunks:
            sim.run(k, graph=True)
            sim.solver.synchronize()
            sim.solver.check()
        runs.append((sim.ibm.force_history(400), sim.solver.read_populations()))
        sim.close()
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])


def test_float32_long_run_against_fp64_oracle(gpkg, oracle_mod):
    """The plain float32 path over 1,000 steps of the small wing case (a quarter motion
    period) against the FP64 oracle: relative L2 of rho and u within 1e-5 and of the force
    history within 1e-4, the plain-path bounds, at a horizon where a per-step bias of the
    collision would show."""
    cfg = gpkg.small_case(storage="f32")
    steps = 1000
    sim = gpkg.Simulation(cfg)
    sim.run(steps)
    got = sim.solver.read_macro()
    hist = sim.ibm.force_history(steps)
    sim.close()
    ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                            cfg.X0, cfg.Y0, cfg.Z0, real="f64")
    ref_hist = ref.run(0, steps, cfg.motion())
    rho, ux, uy, uz = ref.macro()
    ref.close()
    e_rho = rel_l2(got["rho"], rho)
    e_u = rel_l2(np.stack([got["ux"], got["uy"], got["uz"]]), np.stack([ux, uy, uz]))
    e_f = rel_l2(hist, ref_hist)
    print(f"1000 steps: rel L2 rho {e_rho:.2e}, u {e_u:.2e}, force history {e_f:.2e}")
    assert e_rho < 1e-5 and e_u < 1e-5 and e_f < 1e-4


@pytest.mark.parametrize("storage,tol", [("f32", 1e-5), ("f16", 2e-3), ("bf16", 2e-2)])
def test_force_box_at_the_outlet_on_an_odd_lattice(gpkg, oracle_mod, storage, tol):
    """A wing whose stencils reach the outlet column of a lattice with odd Nx (61): the force
    box's rows start at odd and even x, the box pass's last cell pair is the single outlet
    cell, and the bulk and box passes must still cover every cell once. Float32 against the
    float32 oracle (rho, u within 1e-5, force history within 1e-4); the 16-bit forms against
    the FP64 oracle within the shifted-storage tolerances."""
    from dataclasses import replace
    cfg = replace(gpkg.wing_case(61, 40, 6, 16, storage=storage, name="wing-61x40x6-outlet"),
                  x0=61.0 - 0.75 * 16.0 - 1.0)
    steps = 100
    sim = gpkg.Simulation(cfg)
    sim.run(steps)
    got = sim.solver.read_macro()
    hist = sim.ibm.force_history(steps)
    box = sim.ibm.read_markers()
    sim.close()
    assert box["X"].max() > cfg.nx - 3   # the stencils reach the outlet column
    ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                            cfg.X0, cfg.Y0, cfg.Z0, real="f32" if storage == "f32" else "f64")
    ref_hist = ref.run(0, steps, cfg.motion())
    rho, ux, uy, uz = ref.macro()
    ref.close()
    e_rho = rel_l2(got["rho"] - 1.0, rho - 1.0) if storage != "f32" else rel_l2(got["rho"], rho)
    e_u = rel_l2(np.stack([got["ux"], got["uy"], got["uz"]]), np.stack([ux, uy, uz]))
    e_f = rel_l2(hist, ref_hist)
    print(f"{storage} odd lattice, box at the outlet: rho {e_rho:.2e}, u {e_u:.2e}, "
          f"force history {e_f:.2e}")
    if storage == "f32":
        assert e_rho <= 1e-5 and e_u <= 1e-5 and e_f <= 1e-4
    else:
        assert e_u < tol and e_f < 10 * tol


def test_loaded_device_code_is_sm_103a(gpkg):
    """The CUDA runtime reports the loaded kernels as compiled for compute capability 10.3
    (the sm_103a SASS of the library, not a PTX JIT for another target)."""
    import ctypes
    b, p = ctypes.c_int32(), ctypes.c_int32()
    assert gpkg.lib().clbm_binary_version(ctypes.byref(b), ctypes.byref(p)) == 0
    assert b.value == 103, (b.value, p.value)


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("graph", [True, False])
def test_checkpoint_resume_is_bit_exact(gpkg, tmp_path, storage, graph):
    """A run saved after 25 steps and resumed in a new Simulation continues bit for bit as
    the run that was saved (populations, macro fields through the next IBM call, lift/drag
    history, motion phase), also from a checkpoint of the initial state."""
    cfg = gpkg.small_case(storage=storage)
    for first in (25, 0):
        a = gpkg.Simulation(cfg)
        a.run(first, graph=graph)
        path = str(tmp_path / f"ck_{storage}_{first}.npz")
        a.save_checkpoint(path)
        a.run(20, graph=graph)
        b = gpkg.Simulation(cfg)
        b.load_checkpoint(path)
        assert b.ibm.step_count() == first
        b.run(20, graph=graph)
        np.testing.assert_array_equal(b.solver.read_populations(), a.solver.read_populations())
        assert b.ibm.step_count() == a.ibm.step_count() == first + 20
        np.testing.assert_array_equal(b.ibm.force_history(first + 20), a.ibm.force_history(first + 20))
        a.close()
        b.close()


def test_checkpoint_of_another_case_is_refused(gpkg, tmp_path):
    a = gpkg.Simulation(gpkg.small_case())
    path = str(tmp_path / "ck.npz")
    a.save_checkpoint(path)
    a.close()
    b = gpkg.Simulation(gpkg.small_case(storage="f16"))
    with pytest.raises(ValueError):
        b.load_checkpoint(path)
    b.close()
