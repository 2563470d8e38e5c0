"""Import shim for ``taichi`` so the reference driver (main_moving.py:28-37) runs with the
GB300 drop-in modules and without Taichi installed.

``init(arch=gpu)`` checks that the CUDA library loads; there is no CPU backend, so
``init(arch=cpu)`` raises instead of falling back.
"""

gpu = "gpu"
cuda = "gpu"
cpu = "cpu"
f32 = "f32"
f64 = "f64"
i32 = "i32"


def init(arch=gpu, **kwargs):
    if arch != gpu:
        raise RuntimeError("the GB300 drop-in has no CPU backend")
    import _clbm_gb300_pkg as g
    g.pkg.lib()
