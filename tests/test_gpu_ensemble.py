"""Batched ensemble: members stepped together give the same results as each case stepped
alone (same per-cell arithmetic, fixed-point spreading), in float32 and 16-bit storage."""

import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

SMALL = ((48, 24, 4), (64, 20, 6), (40, 16, 3))
# odd and even widths (the 16-bit bulk pass tiles by row segments, float32 by runs across
# row ends)
MIXED = ((47, 20, 4), (64, 20, 6), (41, 16, 3))


def _cases(pkg, storage, n=5, lattices=SMALL):
    return [pkg.config.ensemble_case(seed, storage=storage, lattices=lattices) for seed in range(n)]


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("variant", ["cell", "pair"])
@pytest.mark.parametrize("lattices", [SMALL, MIXED], ids=["even", "mixed"])
@pytest.mark.parametrize("rows", ["1", "1:3", "0", "m"])
def test_ensemble_members_equal_single_runs(built_pkg, monkeypatch, storage, graph, variant, lattices,
                                            rows):
    """The single runs use either full-grid kernel; all variants give the same bits; the
    ensemble bulk pass with whole rows per block (rows = 1: the autotuner's rows per tile;
    1:3: three rows per tile, which does not divide the members' row counts), with row
    segments / runs or whatever else the autotuner picks (0), or as one single-lattice
    launch per member over concurrent streams (m)."""
    pkg = built_pkg
    monkeypatch.setenv("CLBM_KERNEL", variant)
    if rows == "m":
        monkeypatch.setenv("CLBM_ENS_MEMBERS", "1")
        rows = "0"
    else:
        monkeypatch.setenv("CLBM_ENS_MEMBERS", "0" if rows != "0" else "-1")
    mode, _, per_tile = rows.partition(":")
    monkeypatch.setenv("CLBM_ENS_ROWS", mode)
    monkeypatch.setenv("CLBM_ENS_ROWS_R", per_tile or "0")
    cases = _cases(pkg, storage, lattices=lattices)
    ens = pkg.Ensemble(cases)
    ens.run(24, graph=graph)
    t = ens.tuning()
    assert t["tile_width"] in (-1, 0, 128, 256) and t["blocks"] > 0 and t["tiles"] > 0
    if mode == "1":
        assert t["tile_width"] == 0 and t["rows_per_block"] == int(per_tile or t["rows_per_block"]) > 0
    if os.environ.get("CLBM_ENS_MEMBERS") == "1":
        assert t["tile_width"] == -1 and t["blocks"] == len(cases)
    for cfg, member in zip(cases, ens.sims):
        alone = pkg.Simulation(cfg)
        alone.run(24, graph=graph)
        np.testing.assert_array_equal(member.solver.read_populations(),
                                      alone.solver.read_populations())
        h_e, h_a = member.ibm.force_history(24), alone.ibm.force_history(24)
        np.testing.assert_allclose(h_e, h_a, rtol=1e-12, atol=1e-14)
        assert member.ibm.step_count() == 24
        alone.close()
    ens.close()


def test_ensemble_then_member_steps(built_pkg, oracle_mod):
    """After ensemble steps a member continues on its own; the result matches the oracle."""
    pkg = built_pkg
    cases = _cases(pkg, "f32", n=3)
    ens = pkg.Ensemble(cases)
    ens.run(10)
    sim = ens.sims[1]
    cfg = sim.cfg
    sim.run(6, graph=False)
    ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                            cfg.X0, cfg.Y0, cfg.Z0)
    ref.run(0, 16, cfg.motion(), record=False)
    got = sim.solver.read_macro()
    rho, ux, uy, _ = ref.macro()
    assert rel_l2(got["rho"], rho) < 1e-5 and rel_l2(got["ux"], ux) < 1e-5
    ens.close()


def test_ensemble_tiled_spreading_is_bit_identical(built_pkg, monkeypatch):
    """The batched spreading through shared-memory tiles gives the same bits as one global
    atomic per tap, member by member."""
    pkg = built_pkg
    cases = _cases(pkg, "f16", lattices=MIXED)
    out = {}
    for mode in ("direct", "tiled"):
        monkeypatch.setenv("CLBM_SPREAD", mode)
        ens = pkg.Ensemble(cases)
        ens.run(12)
        out[mode] = [(m.solver.read_populations(), m.ibm.force_history(12)) for m in ens.sims]
        ens.close()
    for a, b in zip(out["direct"], out["tiled"]):
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("storage", ["f32", "f16"])
@pytest.mark.parametrize("form", ["launches", "persistent"])
def test_ensemble_at_its_real_sizes(built_pkg, oracle_mod, monkeypatch, storage, form):
    """The batched ensemble as the bench runs it: 64 members drawn with seeds 0..63 from the
    lattices 150x60x12, 200x80x16 and 300x100x24 (chord Nx / 6.25, Re, heave, pitch, phase
    and k drawn per seed), with the schedule the autotuner picks for them (or the whole
    step as one persistent launch), 50 steps. The first member of each lattice and the last
    member give the bits of the same case stepped alone; in float32 one member (300x100x24)
    matches the oracle within the plain-path bounds."""
    pkg = built_pkg
    cases = [pkg.config.ensemble_case(seed, storage=storage) for seed in range(64)]
    steps = 50
    if form == "persistent":
        monkeypatch.setenv("CLBM_ENS_STEP", "persistent")
    ens = pkg.Ensemble(cases)
    monkeypatch.delenv("CLBM_ENS_STEP", raising=False)
    ens.run(steps)
    ens.synchronize()
    sch = ens.schedule()
    assert sch["persistent"] == (form == "persistent")
    if form == "persistent":
        assert sch["blocks"] >= 152
    else:
        t = ens.tuning()
        assert t["blocks"] > 0 and t["tiles"] > 0 and t["bulk_us"] > 0
    firsts = {}
    for i, c in enumerate(cases):
        firsts.setdefault((c.nx, c.ny, c.nz), i)
    assert len(firsts) == 3
    picked = sorted(set(firsts.values()) | {63})
    for i in picked:
        member, cfg = ens.sims[i], cases[i]
        alone = pkg.Simulation(cfg)
        alone.run(steps)
        np.testing.assert_array_equal(member.solver.read_populations(),
                                      alone.solver.read_populations(), err_msg=f"member {i}")
        np.testing.assert_allclose(member.ibm.force_history(steps), alone.ibm.force_history(steps),
                                   rtol=1e-12, atol=1e-14)
        alone.close()
    if storage == "f32":
        i = firsts[(300, 100, 24)]
        cfg = cases[i]
        ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                                cfg.X0, cfg.Y0, cfg.Z0)
        ref_hist = ref.run(0, steps, cfg.motion())
        rho, ux, uy, uz = ref.macro()
        ref.close()
        got = ens.sims[i].solver.read_macro()
        assert rel_l2(got["rho"], rho) <= 1e-5
        assert rel_l2(np.stack([got["ux"], got["uy"], got["uz"]]), np.stack([ux, uy, uz])) <= 1e-5
        assert rel_l2(ens.sims[i].ibm.force_history(steps), ref_hist) <= 1e-4
    ens.close()


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("lattices", [SMALL, MIXED], ids=["even", "mixed"])
def test_persistent_step_equals_separate_launches(built_pkg, monkeypatch, storage, graph, lattices):
    """The whole ensemble step as one persistent cooperative launch (grid barrier between
    the IBM phases, bulk tiles shared out over the phases) gives the populations of the
    seven separate launches bit for bit; the force history is the same sums (the marker
    forces added in another fixed order)."""
    pkg = built_pkg
    cases = _cases(pkg, storage, lattices=lattices)
    out = {}
    for form in ("persistent", "launches"):
        if form == "persistent":
            monkeypatch.setenv("CLBM_ENS_STEP", "persistent")
        else:
            monkeypatch.delenv("CLBM_ENS_STEP", raising=False)
        ens = pkg.Ensemble(cases)
        assert ens.schedule()["persistent"] == (form == "persistent")
        if form == "launches":
            assert ens.schedule()["blocks"] == 0
            with pytest.raises(pkg.CLBMError):
                ens.phase_times()   # the phase clock belongs to the persistent step
        ens.run(24, graph=graph)
        if form == "persistent":
            ph = ens.phase_times()
            assert all(v >= 0 for v in ph.values()) and ph["spreading"] > 0
        out[form] = [(m.solver.read_populations(), m.ibm.force_history(24), m.ibm.step_count())
                     for m in ens.sims]
        ens.close()
    for (fa, ha, na), (fb, hb, nb) in zip(out["persistent"], out["launches"]):
        np.testing.assert_array_equal(fa, fb)
        np.testing.assert_allclose(ha, hb, rtol=1e-12, atol=1e-14)
        assert na == nb == 24


def test_grid_barrier_timeout_is_reported(built_pkg):
    """Failure detection of the persistent step without a fault: a cooperative launch whose
    grid barrier waits for a block that does not exist gives up after its bounded wait and
    reports it; the device stays usable."""
    pkg = built_pkg
    err = pkg.Ensemble.selftest_grid_barrier(2)
    assert err is not None and err.code == 4, err
    s = pkg.Solver(40, 8, 4, 1.5)
    s.step()
    s.synchronize()
    s.close()


@pytest.mark.parametrize("storage", ["f32", "f16"])
@pytest.mark.parametrize("form", ["launches", "persistent"])
def test_members_without_a_body(built_pkg, monkeypatch, storage, form):
    """Members without markers (no IBM: the plain LBM step) stepped beside members with a
    wing, in either step form: every member gives the bits of its case stepped alone."""
    from dataclasses import replace
    pkg = built_pkg
    none = np.zeros(0, np.float32)
    cases = _cases(pkg, storage, n=4, lattices=MIXED)
    cases[1] = replace(cases[1], X0=none, Y0=none, Z0=none)
    cases[3] = replace(cases[3], X0=none, Y0=none, Z0=none)
    assert [c.n_markers > 0 for c in cases] == [True, False, True, False]
    if form == "persistent":
        monkeypatch.setenv("CLBM_ENS_STEP", "persistent")
    ens = pkg.Ensemble(cases)
    monkeypatch.delenv("CLBM_ENS_STEP", raising=False)
    assert ens.schedule()["persistent"] == (form == "persistent")
    ens.run(20)
    for cfg, member in zip(cases, ens.sims):
        alone = pkg.Simulation(cfg)
        alone.run(20)
        np.testing.assert_array_equal(member.solver.read_populations(),
                                      alone.solver.read_populations())
        if cfg.n_markers:
            np.testing.assert_allclose(member.ibm.force_history(20), alone.ibm.force_history(20),
                                       rtol=1e-12, atol=1e-14)
        alone.close()
    ens.close()


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_member_checkpoint_resumes_alone(built_pkg, tmp_path, storage):
    """A member checkpointed after ensemble steps and resumed as a single Simulation
    continues with the bits of the same member stepped on in the ensemble."""
    pkg = built_pkg
    cases = _cases(pkg, storage, n=3)
    ens = pkg.Ensemble(cases)
    ens.run(16)
    path = str(tmp_path / "member1.npz")
    ens.sims[1].save_checkpoint(path)
    ens.run(12)
    alone = pkg.Simulation(cases[1])
    alone.load_checkpoint(path)
    assert alone.ibm.step_count() == 16
    alone.run(12)
    np.testing.assert_array_equal(alone.solver.read_populations(), ens.sims[1].solver.read_populations())
    np.testing.assert_allclose(alone.ibm.force_history(28), ens.sims[1].ibm.force_history(28),
                               rtol=1e-12, atol=1e-14)
    alone.close()
    ens.close()


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_ensemble_at_the_stated_horizon(built_pkg, storage):
    """The 64-member ensemble (lattices 150x60x12, 200x80x16, 300x100x24) for the 5,000
    steps its configuration states, graph-replayed: no member's divergence monitor fires,
    and the first member of each lattice still has the bits of its case stepped alone."""
    pkg = built_pkg
    cases = [pkg.config.ensemble_case(seed, storage=storage) for seed in range(64)]
    steps = 5000
    ens = pkg.Ensemble(cases)
    ens.run(steps)
    ens.synchronize()   # raises if a member's monitor saw a non-finite or too low density
    firsts = {}
    for i, c in enumerate(cases):
        firsts.setdefault((c.nx, c.ny, c.nz), i)
    for i in sorted(firsts.values()):
        alone = pkg.Simulation(cases[i])
        alone.run(steps)
        np.testing.assert_array_equal(ens.sims[i].solver.read_populations(),
                                      alone.solver.read_populations(), err_msg=f"member {i}")
        assert ens.sims[i].ibm.step_count() == steps
        alone.close()
    for m in ens.sims:
        cl = m.coefficients(100)
        assert np.all(np.isfinite(cl["cl"])) and np.all(np.isfinite(cl["cd"]))
    ens.close()
