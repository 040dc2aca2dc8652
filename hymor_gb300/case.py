"""Case set-up: configuration, freestream and the initial solution (host side).

This is the CPG part of the reference's initialisation, run once before the
hot path:

* ``freestream_cpg`` restates SET_FREESTREAM_PROPERTIES.jl:26-113 for a
  calorically perfect gas with the defaults of VERIFY_INPUT_DATA.jl:104-115
  (rho = T = 1, so U = 1 and every ``*_factor`` is 1);
* ``initial_state`` fills the freestream (INITIAL_SOLUTION.jl:33-57), places the
  shock line (SHOCK_LINE_INITIALIZATION.jl:36-53), finds the shocked cells
  (DETECT_CELLS_SHOCKED.jl:34-88) and writes the CPG oblique-shock state below
  it (INITIAL_SOLUTION_POST_SHOCK.jl:64-95); the local shock angle comes from a
  finite-difference slope of the initial shock line instead of a spline fit.
  Seeded Gaussian noise (std = ``noise`` x |q|) is then added to every interior
  cell below the shock.

The resulting :class:`Case` carries everything the hot path needs: the
configuration record, the mesh arrays and the ghosted state, all in the
reference's column-major layout.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import mesh as meshmod

BC_CODES = {
    "symmetry": 0,
    "no_slip_adiabatic": 1,
    "no_slip_isothermal": 2,
    "outflow_supersonic": 3,
    "outflow_supersonic_1st": 4,
    "outflow_subsonic": 5,
    "outflow_NRCBC": 6,
    "inflow_supersonic": 7,
    "inflow_subsonic": 8,
    "periodic": 9,
    "shock": 10,
}
MAP_CODES = {"circle": 0, "blunt_cone": 1, "channel": 2, "wedge": 3}


class ConfigStruct(ctypes.Structure):
    """Binary layout of ``hymor_config`` (include/hymor.h)."""

    _fields_ = [
        ("nchi", ctypes.c_int32), ("neta", ctypes.c_int32),
        ("axisymmetric", ctypes.c_int32),
        ("bc_chi0", ctypes.c_int32), ("bc_chi1", ctypes.c_int32),
        ("bc_eta0", ctypes.c_int32), ("bc_eta1", ctypes.c_int32),
        ("shock_enabled", ctypes.c_int32), ("shock_feedback", ctypes.c_int32),
        ("shock_interp", ctypes.c_int32), ("shock_eulerian", ctypes.c_int32),
        ("mapping", ctypes.c_int32), ("rk_variant", ctypes.c_int32),
        ("viscosity_model", ctypes.c_int32), ("perturb_shock", ctypes.c_int32),
        ("gamma", ctypes.c_double), ("Pr", ctypes.c_double), ("Re", ctypes.c_double),
        ("Mach", ctypes.c_double),
        ("Tw_chi0", ctypes.c_double), ("Tw_eta0", ctypes.c_double), ("Tw_eta1", ctypes.c_double),
        ("cv", ctypes.c_double), ("energy_factor", ctypes.c_double),
        ("rho_0", ctypes.c_double), ("rho_u_0", ctypes.c_double), ("rho_v_0", ctypes.c_double),
        ("rho_E_0", ctypes.c_double), ("p_0", ctypes.c_double),
        ("dist_kx", ctypes.c_double), ("dist_ky", ctypes.c_double),
        ("dist_amp", ctypes.c_double * 4),
        ("relaxation", ctypes.c_double), ("spline_param", ctypes.c_double),
        ("R", ctypes.c_double), ("dRs", ctypes.c_double), ("dRe", ctypes.c_double),
        ("circle_angle_extra", ctypes.c_double),
        ("L", ctypes.c_double), ("theta", ctypes.c_double), ("initial_beta", ctypes.c_double),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("channel_angle", ctypes.c_double),
        ("eta_refinement_power", ctypes.c_double),
        ("rho_min", ctypes.c_double),
        ("CFL", ctypes.c_double), ("max_dt", ctypes.c_double),
        ("perturbation_magnitude", ctypes.c_double),
        ("sutherland_S", ctypes.c_double),
    ]


class MeshStruct(ctypes.Structure):
    """Binary layout of ``hymor_mesh`` (include/hymor.h)."""

    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in (
        "lr_xn", "lr_yn", "lr_a", "bt_xn", "bt_yn", "bt_a", "vol", "x_ext", "y_ext",
        "x_corner", "y_corner", "chi1", "fb_area")] + [
        ("fb_yn_front", ctypes.c_double), ("fb_yn_back", ctypes.c_double)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.flags.c_contiguous)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@dataclass
class Config:
    """Input configuration (the fields of the reference's input Dict the hot path reads)."""

    nchi: int = 100
    neta: int = 80
    pde_dimension: str = "2D"
    bc_chi0: str = "symmetry"
    bc_chi1: str = "outflow_NRCBC"
    bc_eta0: str = "no_slip_isothermal"
    bc_eta1: str = "shock"
    Tw_chi0: float = 1.0
    Tw_eta0: float = 3.0
    Tw_eta1: float = 1.0
    gamma: float = 1.4
    Pr: float = 0.72
    Re: float = 1.0e4
    Mach: float = 5.0
    shock_enabled: bool = True
    shock_feedback: bool = True
    shock_interp: str = "2nd"
    shock_formulation: str = "Lagrangian"
    relaxation: float = 1.0
    initial_shock_dist: float = 0.4
    spline_param: float | None = None   # default 1 - 1e-8 * 100^3 / Nchi^3
    mapping: meshmod.Mapping = field(default_factory=meshmod.Mapping)
    eta_stretch_ratio: float = 1.0
    rho_min: float = 0.05
    CFL: float = 0.5
    max_dt: float = 0.3
    rk_variant: str = "julia"            # "julia" (reference aliasing) or "classical"
    viscosity: str = "constant"          # "constant" (reference CPG) or "sutherland"
    sutherland_S: float = 110.4 / 300.0
    perturbation_magnitude: float = 1e-8
    perturb_shock: bool = False          # stability_analysis.perturb_shock: shock-position unknowns
    disturbance_k: tuple = (1.0, 1.0)
    disturbance_amplitude: tuple = (0.0, 0.0, 0.0, 0.0)

    @property
    def axisymmetric(self) -> bool:
        return self.pde_dimension == "3D-axisymmetric"

    def spline_p(self) -> float:
        if self.spline_param is not None:
            return self.spline_param
        return 1 - 1e-8 * 100**3 / self.nchi**3


def freestream_cpg(cfg: Config) -> dict:
    """SET_FREESTREAM_PROPERTIES.jl:26-113 with u = 1, v = 0, rho = 1, T = 1."""
    u, v, rho, T = 1.0, 0.0, 1.0, 1.0
    U = math.sqrt(u**2 + v**2)
    kin = 0.5 * U**2
    energy_factor = U**2
    rho_factor = rho
    e = energy_factor * 1 / (cfg.gamma - 1) / cfg.gamma / cfg.Mach**2
    E = e + kin
    cv = e / T
    p = rho * e * (cfg.gamma - 1)
    return dict(
        U=U, e=e, E=E, cv=cv, energy_factor=energy_factor, p=p,
        rho_0=rho / rho_factor,
        rho_u_0=rho * u / (U * rho_factor),
        rho_v_0=rho * v / (U * rho_factor),
        rho_E_0=rho * E / (energy_factor * rho_factor),
        p_0=p / (rho_factor * U**2),
        a_0=(U / cfg.Mach) / U,
    )


def config_struct(cfg: Config) -> ConfigStruct:
    fs = freestream_cpg(cfg)
    mp = cfg.mapping
    c = ConfigStruct()
    c.nchi, c.neta = cfg.nchi, cfg.neta
    c.axisymmetric = int(cfg.axisymmetric)
    c.bc_chi0, c.bc_chi1 = BC_CODES[cfg.bc_chi0], BC_CODES[cfg.bc_chi1]
    c.bc_eta0, c.bc_eta1 = BC_CODES[cfg.bc_eta0], BC_CODES[cfg.bc_eta1]
    c.shock_enabled, c.shock_feedback = int(cfg.shock_enabled), int(cfg.shock_feedback)
    c.shock_interp = {"1st": 1, "2nd": 2, "3rd": 3}[cfg.shock_interp]
    c.shock_eulerian = int(cfg.shock_formulation == "Eulerian")
    c.mapping = MAP_CODES[mp.boundary_type]
    c.rk_variant = {"julia": 0, "classical": 1}[cfg.rk_variant]
    c.viscosity_model = {"constant": 0, "sutherland": 1}[cfg.viscosity]
    c.gamma, c.Pr, c.Re, c.Mach = cfg.gamma, cfg.Pr, cfg.Re, cfg.Mach
    c.Tw_chi0, c.Tw_eta0, c.Tw_eta1 = cfg.Tw_chi0, cfg.Tw_eta0, cfg.Tw_eta1
    c.cv, c.energy_factor = fs["cv"], fs["energy_factor"]
    c.rho_0, c.rho_u_0, c.rho_v_0 = fs["rho_0"], fs["rho_u_0"], fs["rho_v_0"]
    c.rho_E_0, c.p_0 = fs["rho_E_0"], fs["p_0"]
    c.dist_kx, c.dist_ky = cfg.disturbance_k
    for k in range(4):
        c.dist_amp[k] = cfg.disturbance_amplitude[k]
    c.relaxation, c.spline_param = cfg.relaxation, cfg.spline_p()
    c.R, c.dRs, c.dRe, c.circle_angle_extra = mp.R, mp.dRs, mp.dRe, mp.circle_angle_extra
    c.L, c.theta, c.initial_beta = mp.L, mp.theta, mp.initial_beta
    c.Lx, c.Ly, c.channel_angle = mp.Lx, mp.Ly, mp.channel_angle
    c.eta_refinement_power = mp.eta_refinement_power
    c.rho_min, c.CFL, c.max_dt = cfg.rho_min, cfg.CFL, cfg.max_dt
    c.perturbation_magnitude = cfg.perturbation_magnitude
    c.perturb_shock = int(cfg.perturb_shock)
    c.sutherland_S = cfg.sutherland_S
    return c


@dataclass
class Case:
    cfg: Config
    mesh: meshmod.Mesh
    fs: dict
    q: np.ndarray          # (4, Nchi+2, Neta+2) Fortran-ordered per variable
    pts_x: np.ndarray
    pts_y: np.ndarray
    pts_chi: np.ndarray
    pts_eta: np.ndarray
    cell_idx: np.ndarray   # int32, 1-based
    a: np.ndarray          # ghosted sound speed
    t: float = 0.0

    def mesh_struct(self) -> tuple[MeshStruct, list]:
        a = self.mesh.arrays
        keep = []

        def P(name):
            if name not in a:
                return ctypes.POINTER(ctypes.c_double)()
            arr = np.asfortranarray(a[name], dtype=np.float64)
            keep.append(arr)
            return dptr(arr)
        m = MeshStruct()
        for n in ("lr_xn", "lr_yn", "lr_a", "bt_xn", "bt_yn", "bt_a", "vol", "x_ext", "y_ext",
                  "x_corner", "y_corner", "chi1", "fb_area"):
            setattr(m, n, P(n))
        m.fb_yn_front = float(a.get("fb_yn_front", 0.0))
        m.fb_yn_back = float(a.get("fb_yn_back", 0.0))
        return m, keep

    def q_flat(self) -> np.ndarray:
        """The 4 ghosted arrays back to back, each column-major: [rho; rho_u; rho_v; rho_E]."""
        return np.concatenate([np.asfortranarray(self.q[v]).ravel(order="F") for v in range(4)])


def thermo_sound_speed(cfg: Config, q: np.ndarray) -> np.ndarray:
    rho, ru, rv, rE = q
    e = (rE - (ru**2 + rv**2) / rho / 2) / rho
    p = rho * e * (cfg.gamma - 1)
    return np.asfortranarray(np.sqrt(cfg.gamma * p / rho))


def detect_cells(msh: meshmod.Mesh, px, py) -> np.ndarray:
    """DETECT_CELLS_SHOCKED.jl:50-65 (first minimum of the squared distance)."""
    x, y = msh["x"], msh["y"]
    d2 = (px[:, None] - x) ** 2 + (py[:, None] - y) ** 2
    return (np.argmin(d2, axis=1) + 1).astype(np.int32)


def initial_state(cfg: Config, seed: int = 1, noise: float = 1e-6) -> Case:
    fs = freestream_cpg(cfg)
    msh = meshmod.generate_mesh(cfg.mapping, cfg.nchi, cfg.neta, cfg.axisymmetric,
                                cfg.eta_stretch_ratio)
    nchi, neta = cfg.nchi, cfg.neta
    shape = (nchi + 2, neta + 2)
    q = np.empty((4,) + shape, order="F")
    mp = cfg.mapping
    if mp.boundary_type == "channel":
        # INITIAL_SOLUTION.jl:44-57: plane Poiseuille profile
        yy = 2 * msh["y_ext"] / mp.Ly
        u_profile = yy * (2 - yy)
        q[0] = fs["rho_0"]
        q[2] = 0.0
        q[1] = fs["rho_u_0"] * u_profile
        rho_e_int = fs["rho_E_0"] - 0.5 * (fs["rho_u_0"] ** 2 + fs["rho_v_0"] ** 2) / fs["rho_0"]
        q[3] = rho_e_int + 0.5 * q[1] ** 2 / q[0]
    else:
        q[0], q[1], q[2], q[3] = fs["rho_0"], fs["rho_u_0"], fs["rho_v_0"], fs["rho_E_0"]
    chi1 = msh["chi1"].copy()
    if cfg.shock_enabled:
        eta_s = np.full(nchi, cfg.initial_shock_dist / mp.dRs)
        px, py = meshmod.physical_space(mp, chi1, eta_s)
        if mp.boundary_type != "circle":
            chi1_s, eta_s = meshmod.element_space(mp, px, py)
        else:
            chi1_s = chi1.copy()
        cell_idx = detect_cells(msh, px, py)
        # local shock angle from the slope of the shock line (COMPUTE_BETA.jl:37-50 form)
        dx = np.gradient(px, chi1_s)
        dy = np.gradient(py, chi1_s)
        u_inf, v_inf = fs["rho_u_0"] / fs["rho_0"], fs["rho_v_0"] / fs["rho_0"]
        beta = np.arctan2(np.abs(dx * v_inf - dy * u_inf), np.abs(dx * u_inf + dy * v_inf))
        if cfg.bc_chi0 == "symmetry":
            beta[0] = math.pi / 2
        M, g = cfg.Mach, cfg.gamma
        rng = np.random.Generator(np.random.PCG64(seed))
        for i in range(nchi):
            b = beta[i]
            top = cell_idx[i] + 2  # ghosted rows 1 .. sc+2 (1-based)
            if M * math.sin(b) > 1:
                ang = b - math.atan2(fs["rho_v_0"], fs["rho_u_0"])
                temp = (g + 1) * (M * math.sin(b)) ** 2 / ((g - 1) * (M * math.sin(b)) ** 2 + 2)
                vn = math.sin(ang) / temp
                vt = math.cos(ang)
                ru = temp * (vn * math.sin(b) + vt * math.cos(b))
                rv = temp * (-vn * math.cos(b) + vt * math.sin(b))
                p_inf = 1 / g / M**2
                k = (ru**2 + rv**2) / 2 / temp**2
                p = p_inf * (2 * g * (M * math.sin(b)) ** 2 - (g - 1)) / (g + 1)
                rE = p / (g - 1) + k * temp
                q[0, i + 1, :top] = temp
                q[1, i + 1, :top] = ru
                q[2, i + 1, :top] = rv
                q[3, i + 1, :top] = rE
        # seeded noise on interior cells below the shock
        for v in range(4):
            z = rng.standard_normal((nchi, neta))
            below = np.arange(1, neta + 1)[None, :] < cell_idx[:, None]
            blk = q[v, 1:-1, 1:-1]
            q[v, 1:-1, 1:-1] = np.where(below, blk + noise * np.abs(blk) * z, blk)
        pts_chi, pts_eta = chi1_s, eta_s
    else:
        rng = np.random.Generator(np.random.PCG64(seed))
        for v in range(4):
            z = rng.standard_normal((nchi, neta))
            blk = q[v, 1:-1, 1:-1]
            q[v, 1:-1, 1:-1] = blk + noise * np.abs(blk) * z
        px = py = np.zeros(nchi)
        pts_chi = chi1.copy()
        pts_eta = np.zeros(nchi)
        cell_idx = np.full(nchi, neta + 1, dtype=np.int32)
    a = thermo_sound_speed(cfg, q)
    return Case(cfg=cfg, mesh=msh, fs=fs, q=q, pts_x=np.ascontiguousarray(px, dtype=np.float64),
                pts_y=np.ascontiguousarray(py, dtype=np.float64),
                pts_chi=np.ascontiguousarray(pts_chi, dtype=np.float64),
                pts_eta=np.ascontiguousarray(pts_eta, dtype=np.float64),
                cell_idx=np.ascontiguousarray(cell_idx, dtype=np.int32), a=a)


def cylinder_config(nchi: int = 100, neta: int = 80, **kw) -> Config:
    """The shock-fitted CPG cylinder (radius 1, M 5, Re 1e4, Tw/T_inf = 3, bow shock
    initially 0.4 off the wall). The wall-normal stretching ratio is 1.05 at Neta = 80 and
    keeps the same overall first-to-last cell ratio (1.05^80) on other grids."""
    ratio = 1.05 ** (80.0 / neta)
    base = dict(nchi=nchi, neta=neta, eta_stretch_ratio=ratio)
    base.update(kw)
    return Config(**base)


def channel_config(nchi: int = 180, neta: int = 60, **kw) -> Config:
    """tutorials/channel_flow/input_file.jl: CPG plane Poiseuille flow, M 0.05, Re 7500."""
    mp = meshmod.Mapping(boundary_type="channel", Lx=2 * math.pi, Ly=2.0, channel_angle=0.0,
                         eta_refinement_power=1.6)
    base = dict(nchi=nchi, neta=neta, mapping=mp, bc_chi0="periodic", bc_chi1="periodic",
                bc_eta0="no_slip_adiabatic", bc_eta1="no_slip_adiabatic", Mach=0.05, Pr=0.73,
                Re=7500.0, shock_enabled=False, CFL=2.0, max_dt=0.3)
    base.update(kw)
    return Config(**base)


def blunt_cone_config(nchi: int = 1200, neta: int = 400, **kw) -> Config:
    """Axisymmetric sphere-cone, nose radius 1, 7 degree half-angle (theta = 83 degrees in
    the reference's blunt_cone mapping), CPG M 6, Re 2e4."""
    mp = meshmod.Mapping(boundary_type="blunt_cone", R=1.0, L=3.0, theta=math.radians(83.0),
                         dRs=0.4, dRe=0.6, initial_beta=math.radians(55.0))
    base = dict(nchi=nchi, neta=neta, mapping=mp, pde_dimension="3D-axisymmetric",
                bc_chi0="symmetry", bc_chi1="outflow_NRCBC", bc_eta0="no_slip_adiabatic",
                bc_eta1="shock", Mach=6.0, Re=2.0e4, initial_shock_dist=0.3)
    base.update(kw)
    return Config(**base)
