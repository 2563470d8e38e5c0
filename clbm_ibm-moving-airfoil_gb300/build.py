"""Build the CUDA library for sm_103a in-tree: ``_build/libclbm_gb300.so``.

Each translation unit is compiled by its own nvcc process in parallel, then linked with
the CUDA runtime into one shared library whose entry points are declared in
``include/clbm_gb300.h``.
"""

import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libclbm_gb300.so")
# record of the nvcc command lines that produced LIB (the target architecture is checked
# from it on machines without a GPU)
INFO = os.path.join(BUILD, "build_info.json")
SOURCES = ["lbm_kernels.cu", "ibm_kernels.cu", "ensemble.cu", "closure.cu", "capi.cu", "closure_api.cu",
           "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "clbm_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose_ptxas=False):
    """Compile the library unless it is newer than every source. Returns the .so path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    procs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src, obj))
    objs, errors, cmds = [], [], []
    for p, src, obj in procs:
        cmds.append(p.args)
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            errors.append(f"--- {src}\n{out}")
        elif verbose_ptxas and out:
            print(out)
        objs.append(obj)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    subprocess.run(cmd, check=True)
    cmds.append(cmd)
    with open(INFO, "w") as fh:
        json.dump({"arch": ARCH, "commands": cmds}, fh, indent=1)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
