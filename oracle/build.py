"""Build recipe for the CPU oracle (test infrastructure; see clbm_oracle.c).

Produces oracle/_build/liboracle_f32.so and liboracle_f64.so with gcc. No fast-math and
no FMA contraction, so float32 results follow IEEE single precision in source order on
both x86-64 and aarch64.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "clbm_oracle.c")
SRCS = [SRC, os.path.join(HERE, "closure_oracle.c")]

FLAGS = ["-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
         "-fno-math-errno", "-Wall", "-Wno-unused-variable"]


def lib_path(real="f32"):
    return os.path.join(BUILD, f"liboracle_{real}.so")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    procs = []
    for real, ctype in (("f32", "float"), ("f64", "double")):
        out = lib_path(real)
        if (not force and os.path.exists(out)
                and os.path.getmtime(out) >= max(os.path.getmtime(f) for f in SRCS)):
            continue
        cmd = ["gcc", *FLAGS, f"-DORACLE_REAL={ctype}", *SRCS, "-o", out + ".tmp", "-lm"]
        procs.append((subprocess.Popen(cmd), out))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {out}")
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(lib_path("f32"), lib_path("f64"))
