"""config.to_config_module: a ``config_moving``-style module generated from a case, with
every name the reference's modules import, the reference's M_raw^-1 bit for bit, and the
case back unchanged through config.from_config_module."""

import os
import re

import numpy as np
import pytest

from conftest import GOLDEN

REF_DIR = os.environ.get("CLBM_REFERENCE_DIR", "/root/reference")
# the names clbm_moving.py:15-16, airfoil_moving.py:17-19 and main_moving.py:42-54 import
NAMES = ("Nx", "Ny", "Nz", "cs2", "s_v", "s_e", "s_q", "s_pi", "U_inf", "AoA0_deg",
         "M_raw_inv_np", "N_MARKERS_2D", "N_MARKERS", "X_marker_np", "Y_marker_np",
         "Z_marker_np", "Re", "x0", "y0", "z0", "f_motion", "A_heave", "A_pitch", "phi_pitch",
         "AoA0_rad", "fuse_ax", "fuse_ay", "fuse_az", "b_half", "z_wing_start", "z_wing_end",
         "x_tail_arm", "c_htail", "b_half_htail", "z_htail_start", "z_htail_end", "c_vtail",
         "h_vtail", "X_template", "Y_template", "X_htail_tmpl", "Y_htail_tmpl", "N_steps",
         "vis_interval", "DATA_DIR")


def test_raw_moment_inverse_is_the_references(pkg):
    m, inv = pkg.config.raw_moment_matrices()
    fix = np.load(os.path.join(GOLDEN, "dropin_main_moving.npz"))
    assert inv.dtype == np.float32
    np.testing.assert_array_equal(inv, fix["cfg_M_raw_inv_np"])
    np.testing.assert_array_equal(inv.astype(np.float64) @ m, np.eye(19))
    assert set(np.unique(np.abs(inv))) <= {0.0, 0.25, 0.5, 1.0}


@pytest.mark.parametrize("case", ["full_case", "fish_case", "reference_airplane_case"])
def test_cases_round_trip_through_a_config_module(pkg, case):
    cfg = getattr(pkg.config, case)()
    mod = pkg.config.to_config_module(cfg, n_steps=300, vis_interval=50)
    for name in NAMES:
        assert hasattr(mod, name), name
    assert mod.N_MARKERS == cfg.n_markers and mod.N_steps == 300 and mod.vis_interval == 50
    back = pkg.config.from_config_module(mod)
    for f in ("nx", "ny", "nz", "chord", "u_inf", "re", "s_e", "inflow_deg", "x0", "y0",
              "a_heave", "a_pitch", "phi_pitch", "aoa0", "k_reduced"):
        assert getattr(back, f) == pytest.approx(getattr(cfg, f), rel=0, abs=0), f
    for a in ("X0", "Y0", "Z0"):
        np.testing.assert_array_equal(getattr(back, a), getattr(cfg, a))
    assert back.s_v == cfg.s_v and back.f_motion == cfg.f_motion


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DIR, "main_moving.py")),
                    reason="reference checkout not present")
def test_names_cover_the_reference_imports(pkg):
    """Every name the reference's solver, IBM and driver modules import from config_moving
    (parsed from their sources) is in the generated module."""
    mod = pkg.config.to_config_module(pkg.config.small_case())
    for f in ("clbm_moving.py", "airfoil_moving.py", "main_moving.py"):
        src = open(os.path.join(REF_DIR, f)).read()
        for block in re.findall(r"from config_moving import \((.*?)\)", src, flags=re.S):
            for name in re.findall(r"\w+", block):
                assert hasattr(mod, name), (f, name)
