"""Generate the long-horizon oracle fixtures of the drop-in case (test infrastructure).

Runs the CPU oracle (oracle/clbm_oracle.c: the reference's unfused step, clbm_moving.py:
326-343 and airfoil_moving.py:230-255, restated in C and pinned bit for bit to the
reference's own kernels by golden_A/golden_B) on the 600x200x50 moving wing (chord 80,
Re 200, 12,600 markers, the motion law of main_moving.py:62-74) and stores

  * hist     [steps, 4] float64: per step the sums (sx, sy) of the clipped Eulerian force
             and (mx, my) of the marker forces, the lift/drag record;
  * rho, ux, uy, uz: the final macroscopic fields sampled on a strided sub-lattice
             (every `stride` cell along x, y, z), stored as float32;
  * the case, the arithmetic (f32 / f64), the step count and the strides.

Two fixtures are used by tests/test_gpu_long_horizon.py:

    python tests/golden/make_long_horizon.py --real f32 --steps 2000 \\
        --out tests/golden/long_f32_600x200x50_2000.npz
    python tests/golden/make_long_horizon.py --real f64 --steps 10053 \\
        --out tests/golden/long_f64_600x200x50_10053.npz

The first (float32, 2,000 steps) is the plain path's parity target at the drop-in case's
size; the second (FP64 everywhere, one motion period = 10,053 steps) judges the 16-bit
storage forms. They take about 20 minutes and 2.5 hours on 6 x86-64 cores.
"""

import argparse
import importlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

STRIDE = (8, 4, 2)


def sample(a, stride=STRIDE):
    return np.ascontiguousarray(a[::stride[0], ::stride[1], ::stride[2]], np.float32)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--real", choices=("f32", "f64"), default="f32")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=500)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)

    pkg = importlib.import_module("clbm_ibm-moving-airfoil_gb300")
    from oracle import build as ob
    ob.build()
    from oracle.oracle import Oracle

    cfg = pkg.full_case()
    o = Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
               cfg.X0, cfg.Y0, cfg.Z0, real=a.real, threads=a.threads or None)
    m = cfg.motion()
    hist = np.zeros((a.steps, 4), np.float64)
    t0 = time.time()
    done = 0
    while done < a.steps:
        n = min(a.chunk, a.steps - done)
        hist[done:done + n] = o.run(done, n, m)
        done += n
        print(f"{done}/{a.steps} steps, {time.time() - t0:.0f} s", flush=True)
    rho, ux, uy, uz = o.macro()
    o.close()
    np.savez_compressed(a.out, hist=hist, rho=sample(rho), ux=sample(ux), uy=sample(uy),
                        uz=sample(uz), stride=np.array(STRIDE), steps=np.int64(a.steps),
                        real=a.real, case=cfg.name, seconds=np.float64(time.time() - t0))
    print("wrote", a.out)


if __name__ == "__main__":
    main()
