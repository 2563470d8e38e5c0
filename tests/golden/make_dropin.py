"""Generate the drop-in fixtures: the reference's own drivers run unmodified, twice.

Run in a container that has the reference checkout (read-only is fine):

    python tests/golden/make_dropin.py /root/reference

For each driver -- ``main_moving.py`` and ``main_highRe.py`` (which aliases its own
config module as ``config_moving`` through ``sys.modules``, main_highRe.py:26-27) -- on a
small in-memory configuration:

  (a) reference run: ``taichi`` is ``taichi_emulator`` and ``clbm_moving`` /
      ``airfoil_moving`` are the reference's own modules; the driver's ``main()`` writes
      its frames and ``meta.npz`` (main_moving.py:124-200) into a scratch directory;
  (b) drop-in run: ``taichi``, ``clbm_moving`` and ``airfoil_moving`` are this project's
      drop-in modules (``compat/``) with their package handle answered by the CPU oracle
      (``oracle_backend``), which records every call the drop-in modules make.

The frames of (b) must equal those of (a) bit for bit (the oracle is pinned to the
reference's kernels). Written per driver: ``dropin_<driver>.npz`` with the configuration
the drop-in modules read, the recorded call trace of (b), and the frames and metadata of
(a). tests/test_dropin.py re-runs (b) here and requires the same trace and frames;
tests/test_gpu_dropin.py replays the trace through the drop-in modules on the GPU and
compares with the frames of (a).
"""

import glob
import importlib.util
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
COMPAT = os.path.join(ROOT, "clbm_ibm-moving-airfoil_gb300", "compat")

for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import make_golden  # noqa: E402  (tests/golden)

# Small cases: the serial Taichi emulator runs the reference kernels in seconds per step.
DRIVERS = {
    "main_moving": dict(config="config_moving",
                        p=dict(Nx=24, Ny=16, Nz=4, U_inf=0.05, Re=10.0, chord=8.0, s_e=1.0,
                               AoA0_deg=6.0, theta0_deg=8.0, x0=9.0, y0=8.0, A_heave=1.5,
                               A_pitch_deg=5.0, k_reduced=0.5, ds=0.7, ellipsoid=(3.0, 1.0, 1.0),
                               n_steps=20), vis_interval=5),
    "main_highRe": dict(config="config_highRe",
                        p=dict(Nx=28, Ny=14, Nz=3, U_inf=0.05, Re=40.0, chord=9.0, s_e=1.0,
                               AoA0_deg=0.0, theta0_deg=4.0, x0=10.0, y0=6.5, A_heave=1.0,
                               A_pitch_deg=5.0, k_reduced=0.5, ds=0.7, ellipsoid=None,
                               n_steps=12), vis_interval=4),
}

CONFIG_KEYS = ("Nx", "Ny", "Nz", "cs2", "s_v", "s_e", "s_q", "s_pi", "U_inf", "AoA0_deg",
               "M_raw_inv_np", "N_MARKERS_2D", "N_MARKERS", "X_marker_np", "Y_marker_np",
               "Z_marker_np")


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def config_module(ref_dir, spec, data_dir):
    refcfg = _load("_reference_config_moving", os.path.join(ref_dir, "config_moving.py"))
    m = make_golden.make_config_module(refcfg, spec["p"])
    m.__name__ = spec["config"]
    m.N_steps = spec["p"]["n_steps"]
    m.vis_interval = spec["vis_interval"]
    m.DATA_DIR = data_dir
    m.c = spec["p"]["chord"]          # names only main_highRe.py imports
    return m


def _clear():
    for mod in ("taichi", "clbm_moving", "airfoil_moving", "config_moving", "config_highRe",
                "main_moving", "main_highRe", "_clbm_gb300_pkg"):
        sys.modules.pop(mod, None)
    while COMPAT in sys.path:
        sys.path.remove(COMPAT)


def read_outputs(data_dir):
    out = {}
    frames = sorted(glob.glob(os.path.join(data_dir, "frame_*.npz")))
    for k, path in enumerate(frames):
        with np.load(path) as d:
            for name in ("rho", "ux", "uy", "uz"):
                out[f"frame{k + 1}_{name}"] = d[name]
    out["n_frames"] = np.int64(len(frames))
    with np.load(os.path.join(data_dir, "meta.npz")) as d:
        for key in d.files:
            out[f"meta_{key}"] = d[key]
        out["meta_keys"] = np.array(sorted(d.files))
    return out


def run_reference(ref_dir, driver):
    """(a): the driver with the reference's own solver modules on the Taichi emulator."""
    spec = DRIVERS[driver]
    _clear()
    import taichi_emulator
    sys.modules["taichi"] = taichi_emulator
    data_dir = tempfile.mkdtemp(prefix=f"dropin_ref_{driver}_")
    sys.modules[spec["config"]] = config_module(ref_dir, spec, data_dir)
    if spec["config"] == "config_moving":
        _load("clbm_moving", os.path.join(ref_dir, "clbm_moving.py"))
        _load("airfoil_moving", os.path.join(ref_dir, "airfoil_moving.py"))
    else:
        # main_highRe.py aliases config_highRe as config_moving and then imports the
        # solver modules; make them importable from the reference checkout
        sys.path.insert(0, ref_dir)
    try:
        main = _load(driver, os.path.join(ref_dir, f"{driver}.py"))
        main.main()
    finally:
        if ref_dir in sys.path:
            sys.path.remove(ref_dir)
    out = read_outputs(data_dir)
    shutil.rmtree(data_dir)
    return out


def run_dropin(ref_dir, driver):
    """(b): the driver with the drop-in modules, package calls answered by the oracle."""
    spec = DRIVERS[driver]
    _clear()
    import oracle_backend
    oracle_backend.install()
    sys.path.insert(0, COMPAT)
    data_dir = tempfile.mkdtemp(prefix=f"dropin_compat_{driver}_")
    cfg = config_module(ref_dir, spec, data_dir)
    sys.modules[spec["config"]] = cfg
    try:
        main = _load(driver, os.path.join(ref_dir, f"{driver}.py"))
        assert sys.modules["clbm_moving"].__file__.startswith(COMPAT)
        assert sys.modules["airfoil_moving"].__file__.startswith(COMPAT)
        assert sys.modules["taichi"].__file__.startswith(COMPAT)
        main.main()
    finally:
        while COMPAT in sys.path:
            sys.path.remove(COMPAT)
    out = read_outputs(data_dir)
    shutil.rmtree(data_dir)
    trace = list(oracle_backend.TRACE)
    config = {f"cfg_{k}": np.asarray(getattr(cfg, k)) for k in CONFIG_KEYS}
    _clear()
    return out, trace, config


def encode_trace(trace):
    """Events as (kind code, 6 doubles, field code) rows: kind 0 compute_force, 1 step,
    2 read_macro; field 0..3 = rho, ux, uy, uz."""
    kinds = {"compute_force": 0, "step": 1, "read_macro": 2}
    names = {"rho": 0, "ux": 1, "uy": 2, "uz": 3}
    kind = np.zeros(len(trace), np.int32)
    args = np.zeros((len(trace), 6), np.float64)
    field = np.full(len(trace), -1, np.int32)
    for i, ev in enumerate(trace):
        kind[i] = kinds[ev[0]]
        if ev[0] == "compute_force":
            args[i] = ev[1:]
        elif ev[0] == "read_macro":
            field[i] = names[ev[1]]
    return kind, args, field


def main(argv):
    ref_dir = argv[1] if len(argv) > 1 else "/root/reference"
    sys.dont_write_bytecode = True
    for driver in argv[2:] or sorted(DRIVERS):
        ref = run_reference(ref_dir, driver)
        got, trace, config = run_dropin(ref_dir, driver)
        for k, v in ref.items():
            if not np.array_equal(np.asarray(v), np.asarray(got[k])):
                raise AssertionError(f"{driver}: drop-in output {k} differs from the reference's")
        kind, args, field = encode_trace(trace)
        path = os.path.join(HERE, f"dropin_{driver}.npz")
        np.savez_compressed(path, trace_kind=kind, trace_args=args, trace_field=field,
                            vis_interval=np.int64(DRIVERS[driver]["vis_interval"]),
                            n_steps=np.int64(DRIVERS[driver]["p"]["n_steps"]), **config, **ref)
        print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(trace)} calls)")


if __name__ == "__main__":
    main(sys.argv)
