"""The CPU oracle against golden vectors produced by the reference's own kernels
(tests/golden/make_golden.py runs clbm_moving.py / airfoil_moving.py unmodified).
The float32 oracle must match them bit for bit."""

import numpy as np
import pytest

from conftest import golden_inflow, load_golden


@pytest.mark.parametrize("case", ["A", "B"])
def test_oracle_matches_reference_kernels_bitwise(oracle_mod, case):
    d = load_golden(case)
    ux_in, uy_in = golden_inflow(d)
    o = oracle_mod.Oracle(int(d["Nx"]), int(d["Ny"]), int(d["Nz"]), float(d["s_v"]),
                          float(d["s_e"]), ux_in, uy_in, d["X0"], d["Y0"], d["Z0"])
    assert np.array_equal(o.minv(), d["M_raw_inv"])
    assert np.array_equal(o.f(), d["f_init"])
    motion = d["motion"]
    for s in range(1, int(d["n_steps"]) + 1):
        o.compute_force(*motion[s - 1])
        if s in d["record"]:
            mk = o.markers()
            for k in ("X", "Y", "Z", "VX", "VY", "Uk", "Vk", "FXk", "FYk"):
                assert np.array_equal(mk[k], d[f"s{s}_{k}"]), (case, s, k)
            fx, fy, fz = o.forces()
            assert np.array_equal(fx, d[f"s{s}_fx"]) and np.array_equal(fy, d[f"s{s}_fy"])
            assert not fz.any()
        o.lbm_step()
        if s in d["record"]:
            rho, ux, uy, uz = o.macro()
            for k, v in (("rho", rho), ("ux", ux), ("uy", uy), ("uz", uz)):
                assert np.array_equal(v, d[f"s{s}_{k}"]), (case, s, k)
        if s in d["f_record"]:
            assert np.array_equal(o.f(), d[f"s{s}_f"]), (case, s)


def test_motion_state_matches_reference_driver(oracle_mod):
    d = load_golden("A")
    m = dict(x0=float(d["x0"]), y0=float(d["y0"]), a_heave=float(d["A_heave"]),
             a_pitch=float(d["A_pitch"]), phi_pitch=float(d["phi_pitch"]),
             aoa0=float(d["AoA0_rad"]), omega=2.0 * np.pi * float(d["f_motion"]))
    for s in range(1, int(d["n_steps"]) + 1):
        assert np.array_equal(oracle_mod.motion_state(s, m), d["motion"][s - 1])
