"""Pure-Python stand-in for the subset of the Taichi API that the reference solver uses.

Test infrastructure only. It lets ``make_golden.py`` import and run the reference's own
``clbm_moving.py`` / ``airfoil_moving.py`` kernels, unmodified, on tiny lattices in this
container (Taichi itself is not installed), so that golden vectors come from the
reference code rather than from a restatement of it.

Semantics emulated:
  * ``ti.field(ti.f32, shape)`` is a float32 NumPy array; element reads return
    ``np.float32`` scalars, so kernel arithmetic stays in float32 (NumPy 2 treats Python
    floats and ints as weakly typed, which matches Taichi's ``default_fp=f32`` literals).
  * ``@ti.kernel`` runs the Python body serially. Arguments annotated ``ti.f32`` are
    truncated to float32, as Taichi does at the kernel boundary.
  * ``ti.atomic_add(field[idx], v)`` is rewritten at decoration time (AST transform) into
    a read-modify-write on the field, applied in loop order.
  * ``ti.static(x)`` returns ``x`` (Python floats become float32 literals).
  * integer ``%`` already follows Python semantics in both Taichi and Python.

Not emulated: Taichi's ``fast_math`` GPU intrinsics and any FMA contraction; the golden
vectors are plain IEEE float32 evaluations of the reference kernels in source order.
"""

import ast
import inspect
import itertools
import textwrap

import numpy as np

f32 = np.float32
f64 = np.float64
i32 = np.int32
gpu = "gpu"
cpu = "cpu"


def init(*args, **kwargs):
    return None


class Field:
    def __init__(self, dtype, shape):
        if not isinstance(shape, tuple):
            shape = (int(shape),)
        self.dtype = dtype
        self.shape = shape
        self.arr = np.zeros(shape, dtype=dtype)

    def __getitem__(self, idx):
        return self.arr[idx]

    def __setitem__(self, idx, value):
        self.arr[idx] = value

    def from_numpy(self, a):
        self.arr[...] = np.asarray(a, dtype=self.dtype)

    def to_numpy(self):
        return self.arr.copy()

    def fill(self, v):
        self.arr[...] = v


def field(dtype, shape):
    return Field(dtype, shape)


def data_oriented(cls):
    return cls


def func(fn):
    return fn


def template():
    return None


def static(x):
    if isinstance(x, float):
        return np.float32(x)
    return x


def ndrange(*dims):
    return itertools.product(*[range(int(d)) for d in dims])


def Vector(values):
    return list(values)


def _is_float(v):
    return isinstance(v, (float, np.floating))


def max(a, b):  # noqa: A001
    r = a if a >= b else b
    return np.float32(r) if (_is_float(a) or _is_float(b)) else r


def min(a, b):  # noqa: A001
    r = a if a <= b else b
    return np.float32(r) if (_is_float(a) or _is_float(b)) else r


def abs(x):  # noqa: A001
    return np.abs(np.float32(x)) if _is_float(x) else (x if x >= 0 else -x)


def sqrt(x):
    return np.sqrt(np.float32(x))


def cos(x):
    return np.cos(np.float32(x))


def sin(x):
    return np.sin(np.float32(x))


def floor(x):
    return np.floor(np.float32(x))


def cast(x, dtype):
    if dtype is i32:
        return int(x)
    return np.float32(x)


def _atomic_add_at(fld, idx, value):
    old = fld.arr[idx]
    fld.arr[idx] = np.float32(old + value)
    return old


class _AtomicRewriter(ast.NodeTransformer):
    def visit_Call(self, node):
        self.generic_visit(node)
        fn = node.func
        if (isinstance(fn, ast.Attribute) and fn.attr == "atomic_add"
                and isinstance(node.args[0], ast.Subscript)):
            sub = node.args[0]
            new = ast.Call(
                func=ast.Attribute(value=ast.Name(id="ti", ctx=ast.Load()),
                                   attr="_atomic_add_at", ctx=ast.Load()),
                args=[sub.value, sub.slice, node.args[1]], keywords=[])
            return ast.copy_location(new, node)
        return node


def kernel(fn):
    src = textwrap.dedent(inspect.getsource(fn))
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_AtomicRewriter().visit(tree))
    ns = {}
    exec(compile(tree, inspect.getsourcefile(fn), "exec"), fn.__globals__, ns)
    body = ns[fdef.name]
    sig = inspect.signature(fn)
    casts = [p.annotation is f32 for p in sig.parameters.values()]

    def wrapper(*args):
        args = [np.float32(a) if c else a for a, c in zip(args, casts)]
        return body(*args)

    wrapper.__name__ = fn.__name__
    return wrapper
