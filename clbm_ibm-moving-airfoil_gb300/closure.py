"""Learned sub-grid closure for the coarse high-Re cascaded collision.

A 19 -> 32 -> 32 -> 1 network (GELU, BF16 weights, FP32 accumulation) maps the 19
normalised non-equilibrium central moments of a cell (moment order of M_raw,
config_moving.py:62-68) to one relaxation rate of its collision, in one of two forms:

  mode 0, higher-order rate: the third- and fourth-order central moments, which the
  reference relaxes fully (s_q = s_pi = 1, clbm_moving.py:186-194), relax with s_h:
      k3* = (1 - s_h) k3,   k4* = rho/9 + (1 - s_h)(k4 - rho/9),   s_h = 1 + span tanh(z3);
  mode 1, eddy viscosity: the deviatoric second-order moments relax with
      s_eff = 1 / (1/2 + 3 nu 2^(span g))   instead of s_v, nu the lattice viscosity,
  g = tanh(z3) where positive and tanh(z3) / 20 below: the network adds an eddy viscosity
  and may remove at most a factor 2^(-span/20) (a leak that keeps the gradient alive).

Training data come from a plain run of the same solver on a lattice twice as fine in each
direction: at a coarse step n (fine step 2n) the fine post-stream populations are box
filtered onto the coarse lattice (f0), and again two fine steps later (f1). A sample is a
coarse cell away from the body: features from f0; for mode 0 the third- and
fourth-order central moments of the ideal post-collision state f*_q(x) = f1_q(x + e_q)
(about the velocity of f0), loss sum_j (t_j - (1 - s_h) p_j)^2 with p_j the pre-collision
values; for mode 1 the sub-grid stress of the filtered fine velocity,
tau = <u u> - <u><u>, and the filtered strain rate S, loss sum_j (tau_j + 2 nu_t S_j)^2 over
the deviatoric components (the eddy-viscosity model tau = -2 nu_t S). The untrained
network (z3 = 0) is the plain method in both forms.

Forward, backward and weight-gradient products run on the tensor cores (tcgen05) in the
CUDA library; this module holds the parameter layout and the host-side orchestration.
"""

import ctypes
import math

import numpy as np

from ._lib import check, lib

N_IN = 19
N_HID = 32
N_TARGETS = 9
N_SGS = 10
SAMPLE_FLOATS = N_IN + N_TARGETS + N_SGS
HIGHER_ORDER, EDDY_VISCOSITY = 0, 1


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Layout:
    """Offsets of the parameter array (from the library, clbm_closure_layout)."""

    _names = ("mu", "sinv", "W1", "b1", "W2", "b2", "W3", "b3", "span", "total", "n_in",
              "n_hid", "n_targets", "n_trainable", "sample_floats", "mode", "nu", "n_sgs",
              "n_stats")

    def __init__(self):
        out = (ctypes.c_int32 * 19)()
        check(lib().clbm_closure_layout(out))
        for name, v in zip(self._names, out):
            setattr(self, name, int(v))
        if (self.n_in, self.n_hid, self.n_targets, self.n_sgs, self.sample_floats) != \
                (N_IN, N_HID, N_TARGETS, N_SGS, SAMPLE_FLOATS):
            raise RuntimeError("closure layout of the library does not match this module")


class ClosureNet:
    """Parameter array of the closure network with named views."""

    def __init__(self, params=None, layout=None):
        self.layout = layout or Layout()
        L = self.layout
        self.params = (np.zeros(L.total, np.float32) if params is None
                       else np.array(params, np.float32).copy())
        if self.params.shape != (L.total,):
            raise ValueError(f"closure parameters must have {L.total} entries")

    def view(self, name):
        L = self.layout
        sizes = {"mu": N_IN, "sinv": N_IN, "W1": N_HID * N_HID, "b1": N_HID,
                 "W2": N_HID * N_HID, "b2": N_HID, "W3": N_HID, "b3": 1, "span": 1,
                 "mode": 1, "nu": 1}
        off = getattr(L, name)
        v = self.params[off:off + sizes[name]]
        return v.reshape(N_HID, N_HID) if name in ("W1", "W2") else v

    # Features 0-3 (k000 - rho and the first-order central moments about the cell's own
    # velocity) vanish in every cell the closure acts on; what they hold is rounding, so
    # the network does not see them.
    SILENT = (0, 1, 2, 3)

    @property
    def mode(self):
        return int(self.view("mode")[0])

    @classmethod
    def initial(cls, mean, std, span=0.8, seed=0, mode=HIGHER_ORDER, nu=0.0):
        """Standardisation from feature statistics, He-scaled hidden layers, and a zero
        output layer, so the untrained network gives the plain method. mode 1 (eddy
        viscosity) needs the lattice viscosity nu the samples come from."""
        net = cls()
        rng = np.random.default_rng(seed)
        net.view("mu")[:] = mean
        sinv = np.where(std > 0, 1.0 / np.maximum(std, 1e-30), 0.0)
        sinv[list(cls.SILENT)] = 0.0
        net.view("mu")[list(cls.SILENT)] = 0.0
        net.view("sinv")[:] = sinv
        w1 = net.view("W1")
        w1[:, :N_IN] = rng.standard_normal((N_HID, N_IN)) * math.sqrt(2.0 / N_IN)
        net.view("W2")[:] = rng.standard_normal((N_HID, N_HID)) * math.sqrt(2.0 / N_HID)
        net.view("span")[:] = span
        net.view("mode")[:] = mode
        net.view("nu")[:] = nu
        return net

    def trainable(self):
        L = self.layout
        return self.params[L.W1:L.span]

    def copy(self):
        return ClosureNet(self.params, self.layout)

    def save(self, path):
        np.save(path, self.params)

    @classmethod
    def load(cls, path):
        return cls(np.load(path))


class Trainer:
    """Training samples and Adam training on the device (clbm_trainer_*)."""

    def __init__(self, capacity, fine=None, device=0):
        Layout()   # checks the sample layout against the library
        self._h = ctypes.c_void_p()
        fh = fine.handle if fine is not None else None
        check(lib().clbm_trainer_create(int(device), fh, int(capacity), ctypes.byref(self._h)))
        self.capacity = int(capacity)
        self.fine = fine
        if fine is not None:
            self.coarse_shape = tuple(n // 2 for n in fine.shape)

    def close(self):
        if self._h is not None and self._h.value:
            lib().clbm_trainer_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def count(self):
        n = ctypes.c_int64()
        check(lib().clbm_trainer_count(self._h, ctypes.byref(n)))
        return n.value

    def capture(self, slot):
        check(lib().clbm_trainer_capture(self._h, int(slot)))

    def read_slot(self, slot):
        """Filtered populations (19 channels), velocity (3) and velocity products
        (xx, yy, zz, xy, xz, yz) of a capture, reference layout."""
        out = np.empty(self.coarse_shape + (28,), np.float32)
        check(lib().clbm_trainer_read_slot(self._h, int(slot), _ptr(out)))
        return out

    def extract(self, cells):
        c = np.ascontiguousarray(cells, np.int64)
        check(lib().clbm_trainer_extract(self._h, _ptr(c), int(c.size)))

    def write_samples(self, off, samples):
        s = np.ascontiguousarray(samples, np.float32)
        check(lib().clbm_trainer_write_samples(self._h, int(off), int(s.shape[0]), _ptr(s)))

    def read_samples(self, off, n):
        out = np.empty((int(n), SAMPLE_FLOATS), np.float32)
        check(lib().clbm_trainer_read_samples(self._h, int(off), int(n), _ptr(out)))
        return out

    def stats(self, off, n):
        """Feature means and standard deviations over a sample range and the mean squared
        sums of the two closure forms' reference quantities (pre-collision higher-order
        moments; deviatoric sub-grid stress), the loss scales:
        (mean, std, {HIGHER_ORDER: ..., EDDY_VISCOSITY: ...})."""
        out = np.zeros(2 * N_IN + 2, np.float64)
        check(lib().clbm_trainer_stats(self._h, int(off), int(n), _ptr(out)))
        mean = out[:N_IN] / n
        var = np.maximum(out[N_IN:2 * N_IN] / n - mean ** 2, 0.0)
        return mean, np.sqrt(var), {HIGHER_ORDER: out[2 * N_IN] / n,
                                    EDDY_VISCOSITY: out[2 * N_IN + 1] / n}

    def loss(self, net, off, n, wscale):
        p = np.ascontiguousarray(net.params, np.float32)
        s = ctypes.c_double()
        check(lib().clbm_trainer_loss(self._h, _ptr(p), int(off), int(n), float(wscale),
                                      ctypes.byref(s)))
        return s.value / n

    def grad(self, net, off, n, wscale):
        p = np.ascontiguousarray(net.params, np.float32)
        g = np.empty(net.layout.n_trainable, np.float32)
        s = ctypes.c_double()
        check(lib().clbm_trainer_grad(self._h, _ptr(p), int(off), int(n), float(wscale), _ptr(g),
                                      ctypes.byref(s)))
        return g, s.value / n

    def fit(self, net, off, n, iters, batch, lr, wscale, seed=0):
        """Adam with cosine decay; returns the trained copy and the minibatch mean losses."""
        out = net.copy()
        hist = np.empty(int(iters), np.float64)
        check(lib().clbm_trainer_fit(self._h, _ptr(out.params), int(off), int(n), int(iters),
                                     int(batch), float(lr), float(wscale), int(seed), _ptr(hist)))
        return out, hist / batch


def tc_selftest(A, B, device=0):
    """D = A B^T through the tensor-core path (BF16 operands, FP32 accumulation)."""
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    D = np.empty((128, B.shape[0]), np.float32)
    check(lib().clbm_tc_selftest(int(device), _ptr(A), _ptr(B), _ptr(D), int(A.shape[1]),
                                 int(B.shape[0])))
    return D


def sample_cells(shape, exclude, n, rng):
    """n distinct coarse cells (linear index x + nx (y + ny z), sorted) with
    2 <= x <= nx - 3, outside the rectangle exclude = (x0, x1, y0, y1) in x-y (all z)."""
    nx, ny, nz = shape
    x0, x1, y0, y1 = exclude
    idx = np.arange(nx * ny * nz, dtype=np.int64)
    x = idx % nx
    y = (idx // nx) % ny
    keep = (x >= 2) & (x <= nx - 3) & ~((x >= x0) & (x <= x1) & (y >= y0) & (y <= y1))
    valid = idx[keep]
    n = min(int(n), valid.size)
    return np.sort(rng.choice(valid, size=n, replace=False))
