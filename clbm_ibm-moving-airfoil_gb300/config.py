"""Case configuration and Lagrangian marker geometry.

The geometry builders reproduce the reference's marker generators exactly (same NumPy
expressions, so the float32 arrays are bit-identical):
  naca0012_section   config_moving.py:105-125  (_naca0012_2d, cosine spacing)
  naca0012_interior  config_moving.py:128-152  (_naca0012_interior, tip-cap fill)
  ellipsoid_markers  config_moving.py:155-190  (_ellipsoid_markers)
  airplane_markers   config_moving.py:196-307  (wing, tips, fuselage, H-tail, V-fin)
and add the full-span extruded wing used by the benchmark cases: one NACA 0012 section
per z layer 0..Nz-1 (the extrusion pattern of fish/config_fish.py:101-108), with the
pitch pivot at a chosen chord fraction.

Relaxation rates follow config_moving.py:37-43 (nu = U c / Re, tau = 1/2 + 3 nu,
s_v = 1/tau) and the motion law main_moving.py:62-74 with omega = 2 pi k U / (pi c).
"""

import math
from dataclasses import dataclass, field, replace

import numpy as np


# ---------------------------------------------------------------------------- geometry
def naca0012_section(chord, ds):
    """Closed NACA 0012 contour, chord-centred (x in [-c/2, c/2]), cosine spaced."""
    t_max = 0.12
    n = max(int(np.ceil(np.pi * chord / ds)), 64)
    if n % 2 != 0:
        n += 1
    ang = np.linspace(0.0, 2.0 * np.pi, n + 1)[:-1]
    xu = 0.5 * (1.0 - np.cos(ang))
    half = (5.0 * t_max
            * (0.2969 * np.sqrt(xu) - 0.1260 * xu - 0.3516 * xu**2
               + 0.2843 * xu**3 - 0.1015 * xu**4))
    side = np.where(ang <= np.pi, 1.0, -1.0)
    X = ((xu - 0.5) * chord).astype(np.float32)
    Y = (side * half * chord).astype(np.float32)
    return X, Y


def naca0012_interior(chord, ds):
    """Grid fill of the NACA 0012 interior (tip caps)."""
    t_max = 0.12
    xs, ys = [], []
    for xi in np.arange(-chord / 2.0 + ds * 0.5, chord / 2.0, ds):
        xn = max(float(xi) / chord + 0.5, 1e-6)
        half = (chord * 5.0 * t_max
                * (0.2969 * np.sqrt(xn) - 0.1260 * xn - 0.3516 * xn**2
                   + 0.2843 * xn**3 - 0.1015 * xn**4))
        if half < ds * 0.5:
            continue
        for yi in np.arange(-half + ds * 0.5, half, ds):
            xs.append(xi)
            ys.append(yi)
    return np.array(xs, dtype=np.float32), np.array(ys, dtype=np.float32)


def ellipsoid_markers(ax, ay, az, ds):
    """Surface markers of an axis-aligned ellipsoid centred at the origin."""
    bands = max(int(np.ceil(np.pi * az / ds)), 8)
    xs, ys, zs = [], [], []
    for i in range(bands + 1):
        phi = np.pi * i / bands
        zl = az * np.cos(phi)
        frac = np.sin(phi)
        if frac < 1e-8:
            xs.append(0.0)
            ys.append(0.0)
            zs.append(float(zl))
            continue
        a, b = ax * frac, ay * frac
        h = ((a - b) / (a + b)) ** 2
        circ = np.pi * (a + b) * (1.0 + 3.0 * h / (10.0 + np.sqrt(4.0 - 3.0 * h)))
        nth = max(int(np.ceil(circ / ds)), 4)
        for th in np.linspace(0.0, 2.0 * np.pi, nth, endpoint=False):
            xs.append(ax * frac * np.cos(th))
            ys.append(ay * frac * np.sin(th))
            zs.append(float(zl))
    return (np.array(xs, dtype=np.float32), np.array(ys, dtype=np.float32),
            np.array(zs, dtype=np.float32))


def ellipse_section(chord, thickness, ds):
    """Ellipse contour with semi-axes chord/2 (x) and thickness/2 (y), fish/config_fish.py:74-91
    (perimeter by Ramanujan's first approximation)."""
    a = chord / 2.0
    b = thickness / 2.0
    perim = np.pi * (3 * (a + b) - np.sqrt((3 * a + b) * (a + 3 * b)))
    n = max(int(np.ceil(perim / ds)), 64)
    if n % 2 != 0:
        n += 1
    ang = np.linspace(0.0, 2.0 * np.pi, n + 1)[:-1]
    return (a * np.cos(ang)).astype(np.float32), (b * np.sin(ang)).astype(np.float32)


def extrude_layers(X2, Y2, nz):
    """One copy of a 2-D section on every z layer 0..nz-1 (fish/config_fish.py:101-108)."""
    layers = np.arange(0, nz, 1.0, dtype=np.float32)
    return (np.tile(X2, len(layers)).astype(np.float32), np.tile(Y2, len(layers)).astype(np.float32),
            np.repeat(layers, len(X2)).astype(np.float32))


def wing_fullspan_markers(chord, nz, ds=1.0, pivot_frac=0.25):
    """NACA 0012 section on every z layer 0..nz-1; body frame origin at the pivot,
    which sits at `pivot_frac` of the chord from the leading edge."""
    X2, Y2 = naca0012_section(chord, ds)
    if pivot_frac != 0.5:
        X2 = (X2 + np.float32((0.5 - pivot_frac) * chord)).astype(np.float32)
    layers = np.arange(0, nz, 1.0, dtype=np.float32)
    X = np.tile(X2, len(layers)).astype(np.float32)
    Y = np.tile(Y2, len(layers)).astype(np.float32)
    Z = np.repeat(layers, len(X2)).astype(np.float32)
    return X, Y, Z


def airplane_markers(nz=160, c=80, b_half=60, ds=0.7, fuse=(75.0, 10.0, 10.0),
                     x_tail_arm=80.0, c_htail=36.0, b_half_htail=32.0, c_vtail=36.0,
                     h_vtail=28.0):
    """Simplified airplane of the reference case; returns X0, Y0 (body frame), Z0
    (absolute) and the templates main_moving.py records in meta.npz."""
    z0 = float(nz) / 2.0
    ds_z = 1.0
    Xt, Yt = naca0012_section(c, ds)
    n2 = len(Xt)
    zw0, zw1 = z0 - b_half, z0 + b_half
    zl = np.arange(zw0, zw1 + ds_z * 0.5, ds_z, dtype=np.float32)
    parts = [(np.tile(Xt, len(zl)), np.tile(Yt, len(zl)), np.repeat(zl, n2))]
    Xi, Yi = naca0012_interior(c, ds)
    parts.append((np.tile(Xi, 2), np.tile(Yi, 2),
                   np.concatenate([np.full(len(Xi), zw0, np.float32),
                                   np.full(len(Xi), zw1, np.float32)])))
    fx, fy, fz = ellipsoid_markers(*fuse, ds)
    parts.append((fx.copy(), fy.copy(), (z0 + fz).astype(np.float32)))
    Xh, Yh = naca0012_section(c_htail, ds)
    zh0, zh1 = z0 - b_half_htail, z0 + b_half_htail
    zlh = np.arange(zh0, zh1 + ds_z * 0.5, ds_z, dtype=np.float32)
    parts.append((np.tile(Xh + x_tail_arm, len(zlh)), np.tile(Yh, len(zlh)),
                  np.repeat(zlh, len(Xh))))
    Xhi, Yhi = naca0012_interior(c_htail, ds)
    parts.append((np.tile(Xhi + x_tail_arm, 2), np.tile(Yhi, 2),
                  np.concatenate([np.full(len(Xhi), zh0, np.float32),
                                  np.full(len(Xhi), zh1, np.float32)])))
    Xv, Yv = naca0012_section(c_vtail, ds)
    yv1 = fuse[1] + h_vtail
    yl = np.arange(fuse[1], yv1 + ds_z * 0.5, ds_z, dtype=np.float32)
    parts.append((np.tile(Xv + x_tail_arm, len(yl)), np.repeat(yl, len(Xv)),
                  np.tile(Yv + z0, len(yl))))
    Xvi, Yvi = naca0012_interior(c_vtail, ds)
    parts.append(((Xvi + x_tail_arm), np.full(len(Xvi), yv1, np.float32), (Yvi + z0)))
    X = np.concatenate([p[0].astype(np.float32) for p in parts]).astype(np.float32)
    Y = np.concatenate([p[1].astype(np.float32) for p in parts]).astype(np.float32)
    Z = np.concatenate([p[2].astype(np.float32) for p in parts]).astype(np.float32)
    return X, Y, Z


# ---------------------------------------------------------------------------- config
@dataclass
class SimConfig:
    """One airfoil case: lattice, flow, collision rates, motion law and markers."""
    nx: int
    ny: int
    nz: int
    chord: float
    u_inf: float = 0.05
    re: float = 200.0
    s_e: float = 1.0
    inflow_deg: float = 0.0      # inlet velocity (U cos a, -U sin a), clbm_moving.py:33-35
    x0: float = 0.0              # pivot position
    y0: float = 0.0
    a_heave: float = 0.0
    a_pitch: float = 0.0         # rad
    phi_pitch: float = math.pi / 2.0
    aoa0: float = 0.0            # mean pitch angle, rad
    k_reduced: float = 0.5
    storage: str = "f32"
    span: float = 0.0            # spanwise length used for force coefficients
    name: str = "case"
    templates: dict = field(default=None, repr=False)   # 2-D sections recorded in meta.npz
    geometry: dict = field(default=None, repr=False)    # body dimensions recorded in grid_meta
    X0: np.ndarray = field(default=None, repr=False)
    Y0: np.ndarray = field(default=None, repr=False)
    Z0: np.ndarray = field(default=None, repr=False)

    @property
    def nu(self):
        return self.u_inf * self.chord / self.re

    @property
    def tau(self):
        return 0.5 + self.nu / (1.0 / 3.0)

    @property
    def s_v(self):
        return 1.0 / self.tau

    @property
    def ux_in(self):
        return float(self.u_inf * math.cos(math.radians(self.inflow_deg)))

    @property
    def uy_in(self):
        return float(-self.u_inf * math.sin(math.radians(self.inflow_deg)))

    @property
    def f_motion(self):
        return self.k_reduced * self.u_inf / (np.pi * self.chord)

    @property
    def omega_motion(self):
        return 2.0 * math.pi * self.f_motion

    @property
    def cells(self):
        return self.nx * self.ny * self.nz

    @property
    def n_markers(self):
        return 0 if self.X0 is None else len(self.X0)

    def motion(self):
        """Motion law parameters as a dict (x0, y0, a_heave, a_pitch, phi_pitch, aoa0, omega)."""
        return dict(x0=float(self.x0), y0=float(self.y0), a_heave=float(self.a_heave),
                    a_pitch=float(self.a_pitch), phi_pitch=float(self.phi_pitch),
                    aoa0=float(self.aoa0), omega=float(self.omega_motion))

    def motion_state(self, step):
        """_motion_state(step) of main_moving.py:65-74 (double precision)."""
        t = float(step)
        w = self.omega_motion
        return (self.x0, self.y0 + self.a_heave * math.sin(w * t),
                self.aoa0 + self.a_pitch * math.sin(w * t + self.phi_pitch), 0.0,
                self.a_heave * w * math.cos(w * t),
                self.a_pitch * w * math.cos(w * t + self.phi_pitch))

    def with_storage(self, storage):
        return replace(self, storage=storage)


def wing_case(nx, ny, nz, chord, re=200.0, u_inf=0.05, k=0.5, name="wing", storage="f32",
              heave_frac=0.25, pitch_amp_deg=10.0, aoa0_deg=8.0, phase_deg=90.0,
              ds=1.0, pivot_frac=0.25):
    """Full-span NACA 0012 wing with theta = aoa0 + A_p sin(w t + phase),
    h = heave_frac * c * sin(w t), unrotated inflow, pivot at `pivot_frac` chord placed at
    x0 = 2c, y0 = Ny/2 (x0 = 160 for c = 80, as in config_moving.py:84-85)."""
    X, Y, Z = wing_fullspan_markers(chord, nz, ds=ds, pivot_frac=pivot_frac)
    n2 = len(X) // nz
    tmpl = dict(X_template=X[:n2].copy(), Y_template=Y[:n2].copy())
    return SimConfig(nx=nx, ny=ny, nz=nz, chord=float(chord), u_inf=u_inf, re=re,
                     inflow_deg=0.0, x0=2.0 * chord, y0=float(ny) / 2.0,
                     a_heave=heave_frac * chord, a_pitch=math.radians(pitch_amp_deg),
                     phi_pitch=math.radians(phase_deg), aoa0=math.radians(aoa0_deg),
                     k_reduced=k, storage=storage, span=float(nz), name=name,
                     templates=tmpl, X0=X, Y0=Y, Z0=Z)


def small_case(storage="f32"):
    """200x80x16 lattice, chord 32, Re 200 (1,632 markers)."""
    return wing_case(200, 80, 16, 32, name="wing-200x80x16-c32", storage=storage)


def full_case(storage="f32"):
    """600x200x50 lattice, chord 80, Re 200 (12,600 markers)."""
    return wing_case(600, 200, 50, 80, name="wing-600x200x50-c80", storage=storage)


def _airplane_extras(nz, c, b_half, ds, fuse, x_tail_arm, c_htail, b_half_htail, c_vtail,
                     h_vtail):
    z0 = float(nz) / 2.0
    Xt, Yt = naca0012_section(c, ds)
    Xh, Yh = naca0012_section(c_htail, ds)
    templates = dict(X_template=Xt, Y_template=Yt, X_htail_tmpl=Xh, Y_htail_tmpl=Yh)
    geometry = dict(fuse_ax=fuse[0], fuse_ay=fuse[1], fuse_az=fuse[2], b_half=b_half,
                    z_wing_start=z0 - b_half, z_wing_end=z0 + b_half, x_tail_arm=x_tail_arm,
                    c_htail=c_htail, b_half_htail=b_half_htail,
                    z_htail_start=z0 - b_half_htail, z_htail_end=z0 + b_half_htail,
                    c_vtail=c_vtail, h_vtail=h_vtail)
    return templates, geometry


def reference_airplane_case(storage="f32"):
    """The reference's own case: 600x200x160 airplane at Re 200 (config_moving.py)."""
    X, Y, Z = airplane_markers()
    cfg = SimConfig(nx=600, ny=200, nz=160, chord=80.0, u_inf=0.05, re=200.0,
                     inflow_deg=8.0, x0=160.0, y0=100.0, a_heave=10.0,
                     a_pitch=float(np.radians(5.0)), phi_pitch=np.pi / 2.0,
                     aoa0=float(np.radians(8.0)), k_reduced=0.5, storage=storage,
                     span=120.0, name="airplane-600x200x160", X0=X, Y0=Y, Z0=Z)
    cfg.templates, cfg.geometry = _airplane_extras(160, 80, 60, 0.7, (75.0, 10.0, 10.0), 80.0,
                                                   36.0, 32.0, 36.0, 28.0)
    return cfg


ENSEMBLE_LATTICES = ((150, 60, 12), (200, 80, 16), (300, 100, 24))


def ensemble_case(seed, storage="f32", lattices=ENSEMBLE_LATTICES):
    """One member of the batched ensemble, drawn from numpy's default_rng(seed): a lattice
    uniformly from `lattices` with chord Nx / 6.25, Re in [100, 400], heave amplitude in
    [0.1c, 0.4c], pitch amplitude in [0, 20] deg, phase in [0, 180] deg, k in [0.25, 1];
    the rest as the wing cases (mean pitch 8 deg, quarter-chord pivot, unrotated inflow)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = lattices[int(rng.integers(len(lattices)))]
    chord = nx / 6.25
    re = float(rng.uniform(100.0, 400.0))
    heave = float(rng.uniform(0.1, 0.4))
    pitch = float(rng.uniform(0.0, 20.0))
    phase = float(rng.uniform(0.0, 180.0))
    k = float(rng.uniform(0.25, 1.0))
    return wing_case(nx, ny, nz, chord, re=re, k=k, heave_frac=heave, pitch_amp_deg=pitch,
                     phase_deg=phase, storage=storage, name=f"ensemble-{seed}")


def highre_airplane_case(storage="f32"):
    """The reference's high-Re variant (config_highRe.py): 800x260x220 airplane, chord 120,
    Re 1000, heave 15 lu, pitch 5 deg about 8 deg, inflow rotated by 8 deg."""
    X, Y, Z = airplane_markers(nz=220, c=120, b_half=90, ds=0.7, fuse=(112.5, 15.0, 15.0),
                               x_tail_arm=120.0, c_htail=54.0, b_half_htail=48.0, c_vtail=54.0,
                               h_vtail=42.0)
    cfg = SimConfig(nx=800, ny=260, nz=220, chord=120.0, u_inf=0.05, re=1000.0,
                     inflow_deg=8.0, x0=200.0, y0=130.0, a_heave=15.0,
                     a_pitch=float(np.radians(5.0)), phi_pitch=np.pi / 2.0,
                     aoa0=float(np.radians(8.0)), k_reduced=0.5, storage=storage,
                     span=180.0, name="airplane-800x260x220-re1000", X0=X, Y0=Y, Z0=Z)
    cfg.templates, cfg.geometry = _airplane_extras(220, 120, 90, 0.7, (112.5, 15.0, 15.0), 120.0,
                                                   54.0, 48.0, 54.0, 42.0)
    return cfg


def fish_case(storage="f32"):
    """The reference's swimmer variant (fish/config_fish.py): 800x250x25, 4:1 ellipse of
    chord 100, Re 300, heave 0.25c, pitch 15 deg, k = 0.8, no mean incidence."""
    X2, Y2 = ellipse_section(100, 25, 0.7)
    X, Y, Z = extrude_layers(X2, Y2, 25)
    return SimConfig(nx=800, ny=250, nz=25, chord=100.0, u_inf=0.05, re=300.0,
                     inflow_deg=0.0, x0=200.0, y0=125.0, a_heave=25.0,
                     a_pitch=float(np.radians(15.0)), phi_pitch=np.pi / 2.0,
                     aoa0=float(np.radians(0.0)), k_reduced=0.8, storage=storage, span=25.0,
                     name="fish-800x250x25-re300", templates=dict(X_template=X2, Y_template=Y2),
                     X0=X, Y0=Y, Z0=Z)


# D3Q19 velocities in the reference's population order (clbm_moving.py:21-30) and the raw
# moments e_x^p e_y^q e_z^r of M_raw in its row order (config_moving.py:62-68): the same
# tables as csrc/clbm_internal.cuh (ex, ey, ez) and csrc/closure_device.cuh (pqr_code).
D3Q19_E = np.array([(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1),
                    (0, 0, -1), (1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0), (1, 0, 1),
                    (-1, 0, 1), (1, 0, -1), (-1, 0, -1), (0, 1, 1), (0, -1, 1), (0, 1, -1),
                    (0, -1, -1)], np.int64)
MOMENT_PQR = ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1),
              (2, 0, 0), (0, 2, 0), (0, 0, 2), (2, 1, 0), (1, 2, 0), (2, 0, 1), (0, 2, 1),
              (1, 0, 2), (0, 1, 2), (2, 2, 0), (2, 0, 2), (0, 2, 2))


def raw_moment_matrices():
    """M_raw (19 x 19, rows the moments of MOMENT_PQR, columns the populations) and its
    inverse as float32; every entry of the inverse is 0, +-1/4, +-1/2 or +-1, so the float32
    values are exact."""
    e = D3Q19_E
    m = np.array([[float(e[q, 0] ** p * e[q, 1] ** r1 * e[q, 2] ** r2) for q in range(19)]
                  for (p, r1, r2) in MOMENT_PQR])
    inv = np.round(np.linalg.inv(m) * 4.0) / 4.0
    assert np.allclose(inv @ m, np.eye(19), atol=1e-12)
    return m, inv.astype(np.float32)


def to_config_module(cfg, n_steps=1000, vis_interval=100, data_dir="data_moving",
                     name="config_moving"):
    """A ``config_moving``-style module for `cfg`: every name the reference's
    clbm_moving.py (:15-16), airfoil_moving.py (:17-19) and main_moving.py (:42-54) import,
    so the reference's driver runs this case through the drop-in modules
    (``sys.modules["config_moving"] = to_config_module(cfg)``, as main_highRe.py:26-27 selects
    its configuration). Body dimensions and templates the case does not have are zeros and
    empty arrays (they only go into meta.npz)."""
    import types
    mod = types.ModuleType(name)
    mod.Nx, mod.Ny, mod.Nz = int(cfg.nx), int(cfg.ny), int(cfg.nz)
    mod.c = float(cfg.chord)
    mod.U_inf, mod.Re = float(cfg.u_inf), float(cfg.re)
    mod.cs2 = 1.0 / 3.0
    mod.nu, mod.tau = cfg.nu, cfg.tau
    mod.s_v, mod.s_e, mod.s_q, mod.s_pi = cfg.s_v, float(cfg.s_e), 1.0, 1.0
    mod.AoA0_deg = float(cfg.inflow_deg)
    mod.M_raw_np, mod.M_raw_inv_np = raw_moment_matrices()
    mod.x0, mod.y0, mod.z0 = float(cfg.x0), float(cfg.y0), float(cfg.nz) / 2.0
    mod.f_motion = cfg.f_motion
    mod.omega = cfg.omega_motion
    mod.k_reduced = float(cfg.k_reduced)
    mod.A_heave, mod.A_pitch = float(cfg.a_heave), float(cfg.a_pitch)
    mod.phi_pitch, mod.AoA0_rad = float(cfg.phi_pitch), float(cfg.aoa0)
    geo = dict(fuse_ax=0.0, fuse_ay=0.0, fuse_az=0.0, b_half=0.0, z_wing_start=0.0,
               z_wing_end=float(cfg.nz), x_tail_arm=0.0, c_htail=0.0, b_half_htail=0.0,
               z_htail_start=0.0, z_htail_end=0.0, c_vtail=0.0, h_vtail=0.0)
    geo.update(cfg.geometry or {})
    for k, v in geo.items():
        setattr(mod, k, v)
    empty = np.zeros(0, np.float32)
    tmpl = dict(X_template=empty, Y_template=empty, X_htail_tmpl=empty, Y_htail_tmpl=empty)
    tmpl.update(cfg.templates or {})
    for k, v in tmpl.items():
        setattr(mod, k, np.asarray(v, np.float32))
    X0 = cfg.X0 if cfg.X0 is not None else empty
    mod.X_marker_np = np.asarray(X0, np.float32)
    mod.Y_marker_np = np.asarray(cfg.Y0 if cfg.Y0 is not None else empty, np.float32)
    mod.Z_marker_np = np.asarray(cfg.Z0 if cfg.Z0 is not None else empty, np.float32)
    mod.N_MARKERS = int(len(X0))
    mod.N_MARKERS_2D = int(len(mod.X_template)) if len(mod.X_template) else mod.N_MARKERS
    mod.N_steps, mod.vis_interval, mod.DATA_DIR = int(n_steps), int(vis_interval), str(data_dir)
    return mod


def from_config_module(mod, storage="f32"):
    """Build a SimConfig from a ``config_moving``-style module (the names the reference's
    clbm_moving.py, airfoil_moving.py and main_moving.py import)."""
    g = lambda k, d=None: getattr(mod, k, d)  # noqa: E731
    cfg = SimConfig(nx=int(mod.Nx), ny=int(mod.Ny), nz=int(mod.Nz), chord=float(g("c", 80.0)),
                    u_inf=float(mod.U_inf), re=float(g("Re", 200.0)),
                    s_e=float(g("s_e", 1.0)), inflow_deg=float(g("AoA0_deg", 0.0)),
                    x0=float(g("x0", 0.0)), y0=float(g("y0", 0.0)),
                    a_heave=float(g("A_heave", 0.0)), a_pitch=float(g("A_pitch", 0.0)),
                    phi_pitch=float(g("phi_pitch", math.pi / 2.0)),
                    aoa0=float(g("AoA0_rad", 0.0)), k_reduced=float(g("k_reduced", 0.5)),
                    storage=storage, span=float(mod.Nz), name=str(g("__name__", "module")),
                    X0=np.asarray(g("X_marker_np"), np.float32) if g("X_marker_np") is not None else None,
                    Y0=np.asarray(g("Y_marker_np"), np.float32) if g("Y_marker_np") is not None else None,
                    Z0=np.asarray(g("Z_marker_np"), np.float32) if g("Z_marker_np") is not None else None)
    return cfg


def body_xy_extent(cfg, state):
    """x and y extent (min, max) of the markers for one motion state (xc, yc, theta, ...)."""
    xc, yc, th = (np.float32(v) for v in state[:3])
    c, s = np.cos(th), np.sin(th)
    x = xc + cfg.X0 * c - cfg.Y0 * s
    y = yc + cfg.X0 * s + cfg.Y0 * c
    return float(x.min()), float(x.max()), float(y.min()), float(y.max())


def stencil_box_cells(cfg, state):
    """Cells of the box that bounds every 4x4x4 Peskin stencil for one motion state
    (xc, yc, theta, ...), by the rule the marker kernel applies: stencil base floor(x) - 1,
    x clamped to the lattice, y and z unwrapped and capped at Ny and Nz."""
    if cfg.n_markers == 0:
        return 0
    xc, yc, th = (np.float32(v) for v in state[:3])
    c, s = np.cos(th), np.sin(th)
    x = xc + cfg.X0 * c - cfg.Y0 * s
    y = yc + cfg.X0 * s + cfg.Y0 * c
    ib = np.floor(x).astype(np.int64) - 1
    jb = np.floor(y).astype(np.int64) - 1
    kb = np.floor(cfg.Z0).astype(np.int64) - 1
    imin = int(np.clip(ib.min(), 0, cfg.nx - 1))
    imax = int(np.clip(ib.max() + 3, 0, cfg.nx - 1))
    jl = min(int(jb.max() + 3 - jb.min() + 1), cfg.ny)
    kl = min(int(kb.max() + 3 - kb.min() + 1), cfg.nz)
    return (imax - imin + 1) * jl * kl


def force_coefficients(sums, cfg):
    """Lift/drag coefficients from per-step force sums (rows: sum fx, sum fy of the clipped
    Eulerian force, sum FX_k, sum FY_k). The force on the body is minus the force injected
    into the fluid. Drag is along the inflow direction, lift normal to it (90 deg
    counter-clockwise); both are scaled by 1/2 rho U^2 c span with rho = 1.
    Returns dict with cd, cl (Eulerian sums) and cd_m, cl_m (marker sums)."""
    s = np.asarray(sums, np.float64).reshape(-1, 4)
    a = math.radians(-cfg.inflow_deg)          # inflow direction angle (uy_in = -U sin)
    e = np.array([math.cos(a), math.sin(a)])
    n = np.array([-math.sin(a), math.cos(a)])
    q = 0.5 * cfg.u_inf ** 2 * cfg.chord * (cfg.span if cfg.span > 0 else cfg.nz)
    fb = -s[:, 0:2]
    fm = -s[:, 2:4]
    return dict(cd=fb @ e / q, cl=fb @ n / q, cd_m=fm @ e / q, cl_m=fm @ n / q)
