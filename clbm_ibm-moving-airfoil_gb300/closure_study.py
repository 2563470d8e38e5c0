"""Learned-closure study at high Reynolds number: train the closure on a plain run of the
same solver on a lattice twice as fine, then compare coarse runs with and without it
against that fine run.

Workload (all lattice units): moving NACA 0012 wing, full span, Re on the chord (default
2000: at Re 5000 the plain cascaded scheme, s_q = s_pi = 1, diverges on both lattices
within a few thousand steps, so no fine reference run exists there), U = 0.05, k = 0.5, theta = 8 + 10 sin(w t + 90) deg, h = 0.25 c sin(w t), pivot at
quarter chord at (2c, Ny/2), Peskin 4-point IBM, Zou-He inlet, zero-gradient outlet,
y/z periodic.
  coarse  600 x 200 x 50,  chord 80,  FP16 shifted storage (plain and with the closure)
  fine   1200 x 400 x 100, chord 160, FP32 (the reference run and the source of training data)
One coarse step is two fine steps (acoustic scaling: same lattice U, halved spacing).

Compared on mean and RMS C_L, C_D over the last motion period(s) and on the mid-span wake
vorticity spectrum (power along x in cycles per chord, vorticity in coarse time units).
"""

import argparse
import json
import math
import time

import numpy as np

from . import analysis, closure
from ._lib import DivergedError
from .config import body_xy_extent, force_coefficients, wing_case
from .solver import Simulation


BASE = (600, 200, 50, 80)   # coarse lattice and chord


def study_case(scale=1, storage="f16", re=5000.0, base=BASE):
    nx, ny, nz, c = (v * scale for v in base)
    return wing_case(nx, ny, nz, c, re=re, storage=storage, name=f"wing-{nx}x{ny}x{nz}-c{c}-Re{re:g}")


def _period(cfg):
    return 2.0 * math.pi / cfg.omega_motion


def _spectrum(sim, cfg, time_scale):
    """Mid-span wake spectrum: x from one chord behind the pivot to 10 cells before the
    outlet, vorticity converted to coarse time units."""
    wz = sim.solver.read_vorticity().astype(np.float64) * time_scale
    x0 = int(cfg.x0 + 1.0 * cfg.chord)
    return analysis.wake_vorticity_spectrum(wz, cfg.chord, x0, cfg.nx - max(2, cfg.nx // 60))


def _spectrum_marks(steps, period, count):
    """Steps at which the wake spectrum is sampled: `count` points spread over the last
    motion period (or the last half of a shorter run), the final step included."""
    span = min(period, steps / 2.0)
    return set(max(1, int(round(steps - i * span / count))) for i in range(count))


STAT_PERIODS = 1   # motion periods the statistics average over (the last ones of the run)


def _window(steps, period):
    return max(1, min(int(round(STAT_PERIODS * period)), steps // 2))


def _divergence_stats(sim):
    """Field statistics of a run that diverged (the check reports them with its error)."""
    try:
        return sim.solver.check(rho_floor=0.5)
    except DivergedError as e:
        return e.stats


def _run(sim, steps, chunk, on_chunk=None):
    """Advance in graph-replayed chunks; wall time of the stepping only (synchronised).
    A run that diverges stops in the chunk where the collisions' divergence monitor trips,
    or at the statistics check after the chunk (density floor 0.5)."""
    done, wall = 0, 0.0
    while done < steps:
        k = min(chunk, steps - done)
        t0 = time.perf_counter()
        try:
            sim.run(k, graph=True)
            sim.solver.synchronize()
        except DivergedError:
            wall += time.perf_counter() - t0
            done += k
            return wall, done, dict(_divergence_stats(sim), step=done)
        wall += time.perf_counter() - t0
        done += k
        try:
            sim.solver.check(rho_floor=0.5)
        except DivergedError as e:
            return wall, done, dict(e.stats, step=done)
        if on_chunk is not None:
            on_chunk(done)
    return wall, done, None


def _stats(sim, cfg, steps, window):
    coeffs = force_coefficients(sim.ibm.force_history(steps), cfg)
    return analysis.force_statistics(coeffs, start=steps - window)


def run_fine(coarse_steps, sample_every, sample_start, cells_per_snapshot, seed, spectra, log,
             base=BASE, re=5000.0):
    cfg = study_case(scale=2, storage="f32", re=re, base=base)
    coarse_shape = (cfg.nx // 2, cfg.ny // 2, cfg.nz // 2)
    sim = Simulation(cfg)
    snaps = max(0, (coarse_steps - sample_start) // sample_every + 1)
    trainer = closure.Trainer(capacity=max(1, snaps * cells_per_snapshot), fine=sim.solver)
    rng = np.random.default_rng(seed)

    def exclude_at(fine_step):
        """Coarse cells near the body at this step (its fine-lattice marker extent halved,
        widened by 3 coarse cells: the IBM stencils and forced cells), so the samples
        include the flow up to the edge of the forced region but no forced cell."""
        x0, x1, y0, y1 = body_xy_extent(cfg, cfg.motion_state(fine_step))
        return (int(math.floor(x0 / 2)) - 3, int(math.ceil(x1 / 2)) + 3,
                int(math.floor(y0 / 2)) - 3, int(math.ceil(y1 / 2)) + 3)
    fine_steps = 2 * coarse_steps
    chunk = 2000
    period = _period(cfg)
    spec_at = _spectrum_marks(fine_steps, period, spectra)
    wall_total, done, sample_wall, spec = 0.0, 0, 0.0, []
    marks = sorted(set([2 * (sample_start + i * sample_every) for i in range(snaps)]) |
                   spec_at | {fine_steps})
    for m in marks:
        if m > fine_steps or m <= done:
            continue
        w, d, bad = _run(sim, m - done, chunk)
        wall_total += w
        done += d
        if bad is not None:
            raise RuntimeError(f"fine run diverged at step {done}: {bad}")
        if m in spec_at:
            spec.append(_spectrum(sim, cfg, 2.0))
        if m < fine_steps and (m // 2 - sample_start) % sample_every == 0 and m // 2 >= sample_start:
            t0 = time.perf_counter()
            trainer.capture(0)
            w, d, bad = _run(sim, 2, 2)   # one coarse step later
            wall_total += w
            done += d
            trainer.capture(1)
            trainer.extract(closure.sample_cells(coarse_shape, exclude_at(m), cells_per_snapshot, rng))
            sample_wall += time.perf_counter() - t0 - w
        log(f"fine step {done}/{fine_steps}, samples {trainer.count}")
    window = _window(fine_steps, period)
    out = dict(case=cfg.name, steps=fine_steps, wall_s=wall_total, sampling_wall_s=sample_wall,
               mlups=cfg.cells * fine_steps / wall_total / 1e6,
               stats=_stats(sim, cfg, fine_steps, window), samples=trainer.count,
               spectrum=_mean_spectrum(spec))
    sim.close()
    return out, trainer


def _mean_spectrum(specs):
    k = specs[0][0]
    return k, np.mean([s[1] for s in specs], axis=0)


def train(trainer, iters, batch, lr, seed, log, span, mode, nu):
    n = trainer.count
    n_train = int(0.9 * n)
    mean, std, p2 = trainer.stats(0, n_train)
    wscale = 1.0 / p2[mode]
    net0 = closure.ClosureNet.initial(mean, std, span=span, seed=seed, mode=mode, nu=nu)
    held = n - n_train
    plain = trainer.loss(net0, n_train, held, wscale)
    t0 = time.perf_counter()
    net, hist = trainer.fit(net0, 0, n_train, iters, batch, lr, wscale, seed=seed)
    wall = time.perf_counter() - t0
    trained = trainer.loss(net, n_train, held, wscale)
    log(f"closure training: held-out loss plain {plain:.4f} -> trained {trained:.4f} ({wall:.2f} s)")
    return net, dict(mode=mode, span=span, samples=n, train=n_train, held_out=held, iters=iters,
                     batch=batch, lr=lr,
                     wall_s=wall, loss_plain=plain, loss_trained=trained,
                     loss_first=float(hist[:20].mean()), loss_last=float(hist[-20:].mean()))


def run_coarse(net, coarse_steps, spectra, log, storage="f16", base=BASE, re=5000.0):
    cfg = study_case(scale=1, storage=storage, re=re, base=base)
    sim = Simulation(cfg)
    if net is not None:
        sim.solver.set_closure(net)
    period = _period(cfg)
    spec_at = sorted(_spectrum_marks(coarse_steps, period, spectra))
    done, wall, spec, bad = 0, 0.0, [], None
    for m in spec_at + [coarse_steps]:
        if m <= done:
            continue
        w, d, bad = _run(sim, m - done, 2000)
        wall += w
        done += d
        if bad is not None:
            break
        if m in spec_at:
            spec.append(_spectrum(sim, cfg, 1.0))
    window = _window(done, period)
    out = dict(case=cfg.name, closure=net is not None, steps=done, wall_s=wall,
               mlups=cfg.cells * done / max(wall, 1e-9) / 1e6)
    if bad is not None:
        out["diverged"] = bad
    else:
        out["stats"] = _stats(sim, cfg, done, window)
        out["spectrum"] = _mean_spectrum(spec)
    log(f"coarse {'closure' if net is not None else 'plain'}: {out.get('stats', 'diverged')}")
    sim.close()
    return out


def compare(fine, coarse):
    if "stats" not in coarse:
        return dict(diverged=True)
    f, c = fine["stats"], coarse["stats"]
    rel = lambda a, b: abs(a - b) / max(abs(b), 1e-12)
    kf, pf = fine["spectrum"]
    kc, pc = coarse["spectrum"]
    return dict(cl_mean_err=rel(c["cl_mean"], f["cl_mean"]), cd_mean_err=rel(c["cd_mean"], f["cd_mean"]),
                cl_rms_err=rel(c["cl_rms"], f["cl_rms"]), cd_rms_err=rel(c["cd_rms"], f["cd_rms"]),
                spectrum_distance=analysis.spectrum_distance(kc, pc, kf, pf, k_max=8.0),
                wall_ratio=fine["wall_s"] / max(coarse["wall_s"], 1e-9))


def span_sweep(net_path, fine_json, scales, coarse_steps, log, base=BASE, re=2000.0):
    """A trained network with its output range (span) scaled at inference, each scale one
    coarse run, compared with the fine run's statistics saved by an earlier study."""
    with open(fine_json) as fh:
        fine = json.load(fh)["fine"]
    out = []
    for m in scales:
        net = closure.ClosureNet.load(net_path)
        net.view("span")[:] *= m
        r = run_coarse(net, coarse_steps, 1, log, base=base, re=re)
        row = dict(span_scale=m, span=float(net.view("span")[0]), wall_s=r["wall_s"])
        if "stats" in r:
            f, c = fine["stats"], r["stats"]
            row.update({k: c[k] for k in ("cl_mean", "cd_mean", "cl_rms", "cd_rms")})
            row.update({k + "_err": abs(c[k] - f[k]) / abs(f[k])
                        for k in ("cl_mean", "cd_mean", "cl_rms", "cd_rms")})
        else:
            row["diverged"] = r.get("diverged")
        log(f"span x{m}: {row}")
        out.append(row)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--coarse-steps", type=int, default=20000)
    ap.add_argument("--sample-every", type=int, default=500)
    ap.add_argument("--sample-start", type=int, default=2000)
    ap.add_argument("--cells-per-snapshot", type=int, default=200000)
    ap.add_argument("--iters", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--spectra", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--re", type=float, default=2000.0)
    ap.add_argument("--mode", type=int, default=closure.EDDY_VISCOSITY, choices=[0, 1],
                    help="0: rate of the third/fourth-order moments; 1: eddy viscosity")
    ap.add_argument("--span", type=float, default=None,
                    help="output range: mode 0 s_h = 1 +- span (default 0.5); mode 1 viscosity "
                         "factor 2^(+-span) (default 2)")
    ap.add_argument("--extra-re", type=float, default=None,
                    help="also run the coarse case at this Re with and without the trained closure")
    ap.add_argument("--base", type=int, nargs=4, default=list(BASE),
                    help="coarse nx ny nz chord (the fine lattice doubles each)")
    ap.add_argument("--save-net", default=None)
    ap.add_argument("--out", default=None)
    ap.add_argument("--span-sweep", type=float, nargs="+", default=None,
                    help="no fine run or training: scale the output range of --load-net by "
                         "each factor and compare coarse runs with the fine statistics of "
                         "--fine-json (an earlier --out file)")
    ap.add_argument("--load-net", default=None)
    ap.add_argument("--fine-json", default=None)
    ap.add_argument("--periods", type=int, default=1,
                    help="statistics over the last PERIODS motion periods (at most half the run)")
    args = ap.parse_args(argv)
    global STAT_PERIODS
    STAT_PERIODS = max(1, args.periods)
    log = lambda m: print(m, flush=True)
    base = tuple(args.base)
    if args.span_sweep:
        rows = span_sweep(args.load_net, args.fine_json, args.span_sweep, args.coarse_steps, log,
                          base=base, re=args.re)
        text = json.dumps(dict(span_sweep=rows, net=args.load_net), indent=1, default=float)
        print(text)
        if args.out:
            with open(args.out, "w") as fh:
                fh.write(text + "\n")
        return rows
    fine, trainer = run_fine(args.coarse_steps, args.sample_every, args.sample_start,
                             args.cells_per_snapshot, args.seed, args.spectra, log, base=base,
                             re=args.re)
    span = args.span if args.span is not None else (0.5 if args.mode == 0 else 2.0)
    nu_coarse = study_case(scale=1, re=args.re, base=base).nu
    net, tr = train(trainer, args.iters, args.batch, args.lr, args.seed, log, span, args.mode,
                    nu_coarse)
    trainer.close()
    if args.save_net:
        net.save(args.save_net)
    plain = run_coarse(None, args.coarse_steps, args.spectra, log, base=base, re=args.re)
    learned = run_coarse(net, args.coarse_steps, args.spectra, log, base=base, re=args.re)
    result = dict(workload=dict(base=base, re=args.re, coarse_steps=args.coarse_steps),
                  fine={k: v for k, v in fine.items() if k != "spectrum"}, training=tr,
                  coarse_plain={k: v for k, v in plain.items() if k != "spectrum"},
                  coarse_closure={k: v for k, v in learned.items() if k != "spectrum"},
                  plain_vs_fine=compare(fine, plain), closure_vs_fine=compare(fine, learned))
    if args.extra_re:
        extra = {}
        for name, n in (("plain", None), ("closure", net)):
            r = run_coarse(n, args.coarse_steps, args.spectra, log, base=base, re=args.extra_re)
            extra[name] = {k: v for k, v in r.items() if k != "spectrum"}
        result["extra_re"] = dict(re=args.extra_re, **extra)
    text = json.dumps(result, indent=1, default=float)
    print(text)
    if args.out:
        with open(args.out, "w") as fh:
            fh.write(text + "\n")
    return result


if __name__ == "__main__":
    main()
