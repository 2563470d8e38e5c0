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
# the bounds-checked library (-DCLBM_CHECK): the same entry points, every population,
# field and stencil access tested against its array first (a debug build; selected by
# CLBM_CHECK_BUILD=1 when the package loads the library)
BUILD_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(BUILD_CHECK, "libclbm_gb300.so")
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


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose_ptxas=False, check=False):
    """Compile the library unless it is newer than every source. Returns the .so path.
    check: the bounds-checked library (LIB_CHECK) instead."""
    out_dir, lib_file = (BUILD_CHECK, LIB_CHECK) if check else (BUILD, LIB)
    if not force and up_to_date(lib_file):
        return lib_file
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    if check:
        extra = extra + ["-DCLBM_CHECK"]
    procs = []
    for src in SOURCES:
        obj = os.path.join(out_dir, src.replace(".cu", ".o"))
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
    tmp = lib_file + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    subprocess.run(cmd, check=True)
    cmds.append(cmd)
    with open(os.path.join(out_dir, "build_info.json"), "w") as fh:
        json.dump({"arch": ARCH, "commands": cmds}, fh, indent=1)
    os.replace(tmp, lib_file)
    return lib_file


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, check="--check" in sys.argv))
