"""Long-run precision of the storage forms against the FP64 oracle (test infrastructure:
the oracle under oracle/ is the checker here, nothing of it is measured or shipped).

Case: the small moving wing (200x80x16, chord 32, Re 200, the motion law of the full case),
run for a whole number of motion periods (default 2 = 8,042 steps) on the GPU in float32,
FP16 and BF16 shifted storage, and on the host cores by the oracle in FP64 and in float32.
Reported for every GPU form against both oracle runs (and for the float32 oracle against
the FP64 one): the relative L2 distance of the final u, rho and rho - 1 fields and of the
force histories, and the relative error of mean and RMS
C_L/C_D over each period and over the last one. Not collected by pytest (no test_ prefix);
run on a GPU machine:

    python tests/precision_long_run.py --periods 2 --out profiles/precision_long_run_200x80x16.json
"""

import argparse
import importlib
import json
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _stats(pkg, hist, cfg, a, b):
    c = pkg.force_coefficients(hist[a:b], cfg)
    return dict(cl_mean=float(np.mean(c["cl"])), cl_rms=float(np.std(c["cl"])),
                cd_mean=float(np.mean(c["cd"])), cd_rms=float(np.std(c["cd"])))


def _stat_errors(s, r):
    return {k: abs(s[k] - r[k]) / abs(r[k]) for k in s}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--periods", type=float, default=2.0)
    ap.add_argument("--forms", default="f32,f16,bf16")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)

    pkg = importlib.import_module("clbm_ibm-moving-airfoil_gb300")
    pkg.build()
    from oracle import build as ob
    ob.build()
    from oracle import oracle

    cfg0 = pkg.small_case()
    period = 2.0 * math.pi / cfg0.omega_motion
    steps = int(round(a.periods * period))
    bounds = []
    p = 0
    while int(round((p + 1) * period)) <= steps:
        bounds.append((int(round(p * period)), int(round((p + 1) * period))))
        p += 1
    res = dict(workload=f"{cfg0.nx}x{cfg0.ny}x{cfg0.nz} moving NACA 0012 wing, chord {cfg0.chord:g}, "
                        f"Re {cfg0.re:g}, {cfg0.n_markers} markers",
               steps=steps, period_steps=period, periods=bounds, oracle={}, forms={})
    refs = {}
    for real in ("f64", "f32"):
        t0 = time.perf_counter()
        o = oracle.Oracle(cfg0.nx, cfg0.ny, cfg0.nz, cfg0.s_v, cfg0.s_e, cfg0.ux_in, cfg0.uy_in,
                          cfg0.X0, cfg0.Y0, cfg0.Z0, real=real)
        hist = o.run(0, steps, cfg0.motion())
        rho, ux, uy, uz = (np.asarray(v, np.float64) for v in o.macro())
        o.close()
        dt = time.perf_counter() - t0
        refs[real] = dict(hist=hist, rho=rho, u=np.stack([ux, uy, uz]))
        res["oracle"][real] = dict(seconds=dt, rho_mean=float(rho.mean()),
                                   per_period=[_stats(pkg, hist, cfg0, x, y) for x, y in bounds])
        print(f"oracle {real}: {steps} steps in {dt:.1f} s", flush=True)
    # the float32 restatement against FP64: the floor float32 arithmetic itself sets
    r32, r64 = refs["f32"], refs["f64"]
    res["oracle"]["f32"]["vs_f64"] = dict(
        u_rel_l2=_rel(r32["u"], r64["u"]), rho_rel_l2=_rel(r32["rho"], r64["rho"]),
        rho_dev_rel_l2=_rel(r32["rho"] - 1.0, r64["rho"] - 1.0),
        history_rel_l2=_rel(r32["hist"], r64["hist"]),
        per_period=[_stat_errors(x, y) for x, y in zip(res["oracle"]["f32"]["per_period"],
                                                       res["oracle"]["f64"]["per_period"])])
    print(f"oracle f32 vs f64: {res['oracle']['f32']['vs_f64']}", flush=True)
    for st in (f for f in a.forms.split(",") if f):
        cfg = pkg.small_case(storage=st)
        sim = pkg.Simulation(cfg)
        sim.run(steps)
        sim.solver.synchronize()
        hist = sim.ibm.force_history(steps)
        m = sim.solver.read_macro()
        sim.close()
        u = np.stack([m["ux"], m["uy"], m["uz"]]).astype(np.float64)
        rho = m["rho"].astype(np.float64)
        per = [_stats(pkg, hist, cfg, x, y) for x, y in bounds]
        out = dict(per_period=per, rho_mean=float(rho.mean()), vs={})
        for real, r in refs.items():
            rper = res["oracle"][real]["per_period"]
            out["vs"][real] = dict(
                u_rel_l2=_rel(u, r["u"]), rho_rel_l2=_rel(rho, r["rho"]),
                rho_dev_rel_l2=_rel(rho - 1.0, r["rho"] - 1.0),
                history_rel_l2=_rel(hist, r["hist"]),
                per_period=[_stat_errors(s, q) for s, q in zip(per, rper)])
        res["forms"][st] = out
        last = {k: {q: f"{v:.2e}" for q, v in out["vs"][k]["per_period"][-1].items()} for k in out["vs"]}
        v64 = out["vs"]["f64"]
        print(f"{st}: u / rho / history vs f64 {v64['u_rel_l2']:.2e} / {v64['rho_rel_l2']:.2e} / "
              f"{v64['history_rel_l2']:.2e}; last period {last}", flush=True)
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(res, fh, indent=1)
    return res


if __name__ == "__main__":
    main()
