"""The drop-in full case run to its full length in each storage form, with the lift/drag
statistics and the differences of the final fields between the forms.

Workload (lattice units): 600 x 200 x 50, NACA 0012 full-span wing, chord 80, Re 200,
U = 0.05, k = 0.5, theta = 8 + 10 sin(w t + 90) deg, h = 0.25 c sin(w t), pivot at quarter
chord at (2c, Ny/2), Peskin 4-point IBM, Zou-He inlet, zero-gradient outlet, y/z periodic,
30,000 steps (about three motion periods of 10,053 steps), as main_moving.py runs it with
config_moving.py. Each form runs the same graph-replayed steps (motion law on the device)
from f = feq(1, (U, 0, 0)); the divergence statistics are checked after every chunk.

Reported per form: wall time of the stepping, MLUPS, mean and RMS of C_L and C_D over the
last two periods and over each whole period, the final divergence statistics and mean
density (the velocity inlet and the zero-gradient outlet leave the mass in the domain
free); for the
16-bit forms also the relative L2 distance of their final u and rho - 1 fields and of
their C_L/C_D histories to the float32 run.
"""

import argparse
import json
import math
import time

import numpy as np

from . import analysis
from ._lib import DivergedError
from .config import force_coefficients, full_case
from .solver import Simulation


def _rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_form(storage, steps, chunk=2000, perturb=0.0, seed=0, log=print):
    """Run the full case in `storage` for `steps` steps. Returns (summary, coefficients,
    final fields). perturb > 0 multiplies the initial populations by 1 + perturb * N(0, 1)
    (seeded), to measure how far a rounding-sized difference carries over the run."""
    cfg = full_case(storage=storage)
    period = 2.0 * math.pi / cfg.omega_motion
    sim = Simulation(cfg)
    try:
        if perturb > 0:
            f = sim.solver.read_populations()
            noise = np.random.default_rng(seed).standard_normal(f.shape, dtype=np.float32)
            f *= 1.0 + np.float32(perturb) * noise
            del noise
            sim.solver.write_populations(f)
            del f
        done, wall, diverged, stats = 0, 0.0, None, None
        while done < steps:
            k = min(chunk, steps - done)
            t0 = time.perf_counter()
            tripped = False
            try:
                sim.run(k, graph=True)   # the collisions' divergence monitor may stop it
                sim.solver.synchronize()
            except DivergedError:
                tripped = True
            wall += time.perf_counter() - t0
            done += k
            try:
                stats = sim.solver.check(rho_floor=0.3)   # raises after a tripped monitor
            except DivergedError as e:
                diverged = dict(e.stats, step=done)
                break
            if tripped:
                diverged = dict(stats, step=done)
                break
        coeffs = force_coefficients(sim.ibm.force_history(done), cfg)
        fields = sim.solver.read_macro()
        cells = cfg.nx * cfg.ny * cfg.nz
        window = max(1, min(int(round(2 * period)), done // 2))
        out = dict(storage=storage, perturb=perturb, steps=done, period_steps=period, wall_s=wall,
                   mlups=cells * done / wall / 1e6 if wall > 0 else None,
                   diverged=diverged, check=stats, rho_mean=float(fields["rho"].mean(dtype=np.float64)),
                   last_two_periods=analysis.force_statistics(coeffs, start=done - window),
                   per_period=[])
        p = 0
        while (p + 1) * period <= done:
            a, b = int(round(p * period)), int(round((p + 1) * period))
            cl = coeffs["cl"][a:b]
            cd = coeffs["cd"][a:b]
            out["per_period"].append(dict(period=p + 1, steps=[a, b], cl_mean=float(cl.mean()),
                                          cl_rms=float(cl.std()), cd_mean=float(cd.mean()),
                                          cd_rms=float(cd.std())))
            p += 1
        log(f"{storage} (perturb {perturb:g}): {done} steps in {wall:.2f} s ({out['mlups']:.0f} MLUPS), "
            f"last two periods {out['last_two_periods']}")
        return out, coeffs, fields
    finally:
        sim.close()


def study(steps=30000, forms=("f32", "f16", "bf16"), perturb=0.0, log=print):
    """Run each form; the first must be f32 (the comparison base). perturb > 0 adds runs
    labelled '<form>+perturb' of the f32 and f16 forms with perturbed initial states."""
    res = dict(workload="600x200x50 moving NACA 0012 wing, chord 80, Re 200, 12,600 markers",
               steps=steps, forms={})
    runs = [(st, st, 0.0) for st in forms]
    if perturb > 0:
        runs += [(st + "+perturb", st, perturb) for st in ("f32", "f16") if st in forms]
    base_c, base_f = None, None
    for label, st, pert in runs:
        out, coeffs, fields = run_form(st, steps, perturb=pert, log=log)
        if label == "f32":
            base_c, base_f = coeffs, fields
        elif base_c is not None and out["diverged"] is None:
            n = min(len(coeffs["cl"]), len(base_c["cl"]))
            u = np.stack([fields[k] for k in ("ux", "uy", "uz")])
            u0 = np.stack([base_f[k] for k in ("ux", "uy", "uz")])
            s2, s0 = out["last_two_periods"], res["forms"]["f32"]["last_two_periods"]
            out["vs_f32"] = dict(
                u_rel_l2=_rel_l2(u, u0),
                rho_dev_rel_l2=_rel_l2(fields["rho"] - 1.0, base_f["rho"] - 1.0),
                cl_history_rel_l2=_rel_l2(coeffs["cl"][:n], base_c["cl"][:n]),
                cd_history_rel_l2=_rel_l2(coeffs["cd"][:n], base_c["cd"][:n]),
                cl_mean_rel=abs(s2["cl_mean"] - s0["cl_mean"]) / abs(s0["cl_mean"]),
                cd_mean_rel=abs(s2["cd_mean"] - s0["cd_mean"]) / abs(s0["cd_mean"]),
                cl_rms_rel=abs(s2["cl_rms"] - s0["cl_rms"]) / abs(s0["cl_rms"]),
                cd_rms_rel=abs(s2["cd_rms"] - s0["cd_rms"]) / abs(s0["cd_rms"]))
            log(f"{label} vs f32: {out['vs_f32']}")
        res["forms"][label] = out
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--steps", type=int, default=30000)
    ap.add_argument("--forms", default="f32,f16,bf16")
    ap.add_argument("--perturb", type=float, default=0.0,
                    help="also run f32 and f16 from initial states perturbed by this relative size")
    ap.add_argument("--out", default=None, help="write the results as JSON here")
    a = ap.parse_args(argv)
    res = study(a.steps, tuple(f for f in a.forms.split(",") if f), perturb=a.perturb)
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(res, fh, indent=1)
    return res


if __name__ == "__main__":
    main()
