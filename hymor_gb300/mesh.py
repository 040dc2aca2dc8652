"""Host-side mesh generation and metrics (one-time set-up, not the hot path).

Restates, in numpy, the parts of the reference's mesh layer that produce the
arrays the residual reads:

* ``GO_TO_PHYSICAL_SPACE`` / ``GO_TO_ELEMENT_SPACE`` for the circle, blunt-cone,
  channel and wedge mappings (utils/Mesh/GO_TO_PHYSICAL_SPACE.jl:28-160,
  utils/Mesh/GO_TO_ELEMENT_SPACE.jl:28-140);
* face normals, areas and cell volumes, 2-D and 3-D-axisymmetric
  (utils/Mesh/GENERATE_MESH.jl:144-300);
* cell centres and the ghost-extended centres
  (utils/Mesh/GET_EXTENDED_CELL_CENTERS.jl:26-88).

Every array is Fortran-ordered (chi index fastest) with the reference's shapes:
lr faces (Nchi+1, Neta), bt faces (Nchi, Neta+1), cells (Nchi, Neta), corners
(Nchi+1, Neta+1), ghosted (Nchi+2, Neta+2).

One addition: ``eta_stretch_ratio`` places the wall-normal corner lines with a
geometric progression (cell k+1 / cell k = ratio) instead of the reference's
uniform ``range(0, 1, length=Neta+1)``; ratio 1 reproduces the reference.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ARC_3D = 0.001  # GENERATE_MESH.jl:130, arc angle of the axisymmetric wedge


def _f(a):
    return np.asfortranarray(a, dtype=np.float64)


@dataclass
class Mapping:
    """Curvilinear mapping parameters (the reference's ``curvilinear_mapping``)."""

    boundary_type: str = "circle"
    R: float = 1.0
    dRs: float = 0.5
    dRe: float = 1.5
    circle_angle_extra: float = 0.0
    L: float = 3.0
    theta: float = math.radians(83.0)
    initial_beta: float = math.radians(55.0)
    Lx: float = 2 * math.pi
    Ly: float = 2.0
    channel_angle: float = 0.0
    eta_refinement_power: float = 1.0


def physical_space(mp: Mapping, chi, eta):
    """GO_TO_PHYSICAL_SPACE.jl:28-160."""
    chi = np.asarray(chi, dtype=np.float64)
    eta = np.asarray(eta, dtype=np.float64)
    if mp.boundary_type == "circle":
        angle_min = -mp.circle_angle_extra
        angle_max = math.pi / 2
        angle = angle_max - chi * (angle_max - angle_min)
        distance_max = mp.dRs + (mp.dRe - mp.dRs) * chi**2
        r = mp.R + eta * distance_max
        return -r * np.sin(angle), r * np.cos(angle)
    if mp.boundary_type == "blunt_cone":
        chi_arc = (1 - chi) / 2
        s_Str_sh = ((mp.L - mp.R) + mp.R * math.cos(mp.initial_beta)) / math.sin(mp.initial_beta)
        s_Crv_sh = mp.initial_beta * mp.R
        s_tot_sh = 2 * s_Crv_sh + 2 * s_Str_sh
        slope = math.sin(mp.theta - mp.initial_beta)
        distance_max = np.where(chi_arc < s_Str_sh / s_tot_sh,
                                mp.dRs + (s_Str_sh - chi_arc * s_tot_sh) * slope, mp.dRs)
        eta_phys = eta * distance_max
        th = mp.theta
        s_Straight = ((mp.L - mp.R) + mp.R * math.cos(th)) / math.sin(th)
        s_Curve = 2 * th * mp.R
        s_tot = s_Curve + 2 * s_Straight
        x = np.zeros(np.broadcast(chi, eta).shape)
        y = np.zeros_like(x)
        chi_arc_b = np.broadcast_to(chi_arc, x.shape)
        eta_b = np.broadcast_to(eta_phys, x.shape)
        seg1 = (0 <= chi_arc_b) & (chi_arc_b < s_Straight / s_tot)
        seg2 = (s_Straight / s_tot <= chi_arc_b) & (chi_arc_b < (s_Straight + s_Curve) / s_tot)
        seg3 = ~(seg1 | seg2)
        lam = s_Straight / s_tot - chi_arc_b
        xb1 = eta_b * math.sin(th) + mp.R * math.sin(th) + lam * math.cos(th) * s_tot
        yb1 = eta_b * math.cos(th) + (mp.L - mp.R) + mp.R * math.cos(th) - lam * math.sin(th) * s_tot
        ang = (chi_arc_b - s_Straight / s_tot) * 2 * th * s_tot / s_Curve + math.pi / 2 - th
        xb2 = (eta_b + mp.R) * np.cos(ang)
        yb2 = (eta_b + mp.R) * np.sin(ang) - mp.R + mp.L
        lam3 = chi_arc_b - (s_Straight + s_Curve) / s_tot
        xb3 = -eta_b * math.sin(th) - mp.R * math.sin(th) - lam3 * math.cos(th) * s_tot
        yb3 = eta_b * math.cos(th) + (mp.L - mp.R) + mp.R * math.cos(th) - lam3 * math.sin(th) * s_tot
        xb = np.where(seg1, xb1, np.where(seg2, xb2, xb3))
        yb = np.where(seg1, yb1, np.where(seg2, yb2, yb3))
        x[...] = -yb
        y[...] = xb
        return x, y
    if mp.boundary_type == "channel":
        p = mp.eta_refinement_power
        eta_r = np.where(eta <= 0.5, 2 ** (p - 1) * np.abs(eta) ** p,
                         1 - 2 ** (p - 1) * np.abs(1 - eta) ** p)
        ca, sa = math.cos(mp.channel_angle), math.sin(mp.channel_angle)
        x = chi * ca * mp.Lx - eta_r * sa * mp.Ly
        y = eta_r * ca * mp.Ly + chi * sa * mp.Lx
        return x, y
    if mp.boundary_type == "wedge":
        distance_max = mp.dRs + (mp.dRe - mp.dRs) * (1 - chi)
        return -eta * distance_max, mp.Lx * (1 - chi)
    raise ValueError(f"unknown boundary_type {mp.boundary_type!r}")


def element_space(mp: Mapping, x, y):
    """GO_TO_ELEMENT_SPACE.jl:28-140 (circle, blunt_cone, channel, wedge)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    if mp.boundary_type == "circle":
        angle_min = -mp.circle_angle_extra
        angle_max = math.pi / 2
        angle = np.mod(np.arctan2(-x, y) + math.pi / 2, 2 * math.pi) - math.pi / 2
        chi = (angle_max - angle) / (angle_max - angle_min)
        r = np.sqrt(x**2 + y**2)
        distance_max = mp.dRs + (mp.dRe - mp.dRs) * chi**2
        return chi, (r - mp.R) / distance_max
    if mp.boundary_type == "blunt_cone":
        th = mp.theta
        s_Straight = ((mp.L - mp.R) + mp.R * math.cos(th)) / math.sin(th)
        s_Curve = 2 * th * mp.R
        s_tot = s_Curve + 2 * s_Straight
        xb = y
        yb = -x
        tang = (yb - (mp.L - mp.R)) / xb
        c1 = (tang < math.tan(math.pi / 2 - th)) & (xb > 0)
        c2 = ~c1 & (-math.tan(math.pi / 2 - th) < tang) & (xb < 0)
        e1 = yb * math.cos(th) + xb * math.sin(th) - mp.R - (mp.L - mp.R) * math.cos(th)
        l1 = (xb / math.cos(th) - (e1 * math.sin(th) + mp.R * math.sin(th)) / math.cos(th)) / s_tot
        a1 = s_Straight / s_tot - l1
        e2 = yb * math.cos(th) - xb * math.sin(th) - mp.R - (mp.L - mp.R) * math.cos(th)
        l2 = (-xb / math.cos(th) - (e2 * math.sin(th) + mp.R * math.sin(th)) / math.cos(th)) / s_tot
        a2 = (s_Straight + s_Curve) / s_tot + l2
        ang = np.arctan2(yb + mp.R - mp.L, xb)
        e3 = xb / np.cos(ang) - mp.R
        a3 = (ang - math.pi / 2 + th) / (2 * th * s_tot / s_Curve) + s_Straight / s_tot
        eta_phys = np.where(c1, e1, np.where(c2, e2, e3))
        chi_arc = np.where(c1, a1, np.where(c2, a2, a3))
        chi = 1 - 2 * chi_arc
        ib = mp.initial_beta
        s_Str_sh = ((mp.L - mp.R) + mp.R * math.cos(ib)) / math.sin(ib)
        s_Crv_sh = ib * mp.R
        s_tot_sh = 2 * s_Crv_sh + 2 * s_Str_sh
        slope = math.sin(th - ib)
        distance_max = np.where(chi_arc < s_Str_sh / s_tot_sh,
                                mp.dRs + (s_Str_sh - chi_arc * s_tot_sh) * slope, mp.dRs)
        return chi, eta_phys / distance_max
    if mp.boundary_type == "channel":
        ca, sa = math.cos(mp.channel_angle), math.sin(mp.channel_angle)
        chi = (x * ca + y * sa) / mp.Lx
        eta_r = (-x * sa + y * ca) / mp.Ly
        p = mp.eta_refinement_power
        eta = np.where(eta_r <= 0.5, (np.abs(eta_r) / 2 ** (p - 1)) ** (1 / p),
                       1 - (np.abs(1 - eta_r) / 2 ** (p - 1)) ** (1 / p))
        return chi, eta
    if mp.boundary_type == "wedge":
        chi = 1 - y / mp.Lx
        distance_max = mp.dRs + (mp.dRe - mp.dRs) * (1 - chi)
        return chi, -x / distance_max
    raise ValueError(f"unknown boundary_type {mp.boundary_type!r}")


@dataclass
class Mesh:
    nchi: int
    neta: int
    axisymmetric: bool
    arrays: dict = field(default_factory=dict)

    def __getitem__(self, k):
        return self.arrays[k]


def _eta_lines(neta: int, ratio: float) -> np.ndarray:
    if ratio == 1.0:
        return np.linspace(0.0, 1.0, neta + 1)
    k = np.arange(neta + 1, dtype=np.float64)
    return (ratio**k - 1.0) / (ratio**neta - 1.0)


def _tet_volume(p1, p2, p3, p4):
    v1, v2, v3 = p2 - p1, p3 - p1, p4 - p1
    return np.abs(np.einsum("...i,...i->...", v1, np.cross(v2, v3))) / 6


def generate_mesh(mp: Mapping, nchi: int, neta: int, axisymmetric: bool = False,
                  eta_stretch_ratio: float = 1.0) -> Mesh:
    """GENERATE_MESH.jl:33-319 (no restart/remesh, no corner smoothing)."""
    chi_1d = np.linspace(0.0, 1.0, nchi + 1)
    eta_1d = _eta_lines(neta, eta_stretch_ratio)
    chi_2d = np.repeat(chi_1d[:, None], neta + 1, axis=1)
    eta_2d = np.repeat(eta_1d[None, :], nchi + 1, axis=0)
    xc, yc = physical_space(mp, chi_2d, eta_2d)
    xc, yc = _f(xc), _f(yc)

    # GET_EXTENDED_CELL_CENTERS.jl:26-88
    x = (xc[:-1, :-1] + xc[1:, :-1] + xc[:-1, 1:] + xc[1:, 1:]) / 4
    y = (yc[:-1, :-1] + yc[1:, :-1] + yc[:-1, 1:] + yc[1:, 1:]) / 4
    x_ext = np.zeros((nchi + 2, neta + 2))
    y_ext = np.zeros((nchi + 2, neta + 2))
    x_ext[1:-1, 1:-1] = x
    y_ext[1:-1, 1:-1] = y
    for A, C in ((x_ext, xc), (y_ext, yc)):
        A[1:-1, 0] = (C[:-1, 0] + C[1:, 0]) / 2
        A[1:-1, -1] = (C[:-1, -1] + C[1:, -1]) / 2
        A[0, 1:-1] = (C[0, :-1] + C[0, 1:]) / 2
        A[-1, 1:-1] = (C[-1, :-1] + C[-1, 1:]) / 2
        A[0, 0], A[0, -1], A[-1, 0], A[-1, -1] = C[0, 0], C[0, -1], C[-1, 0], C[-1, -1]
        A[:, 0] = 2 * A[:, 0] - A[:, 1]
        A[:, -1] = 2 * A[:, -1] - A[:, -2]
        A[0, :] = 2 * A[0, :] - A[1, :]
        A[-1, :] = 2 * A[-1, :] - A[-2, :]
    chi_c, eta_c = element_space(mp, x, y)

    # lr faces (GENERATE_MESH.jl:150-195)
    dxl = xc[:, 1:] - xc[:, :-1]
    dyl = yc[:, 1:] - yc[:, :-1]
    edge = np.sqrt(dxl**2 + dyl**2)
    lr_xn = -dyl / edge
    lr_yn = dxl / edge
    nxt_dx = np.empty_like(dxl)
    nxt_dy = np.empty_like(dyl)
    nxt_dx[:-1] = xc[1:, :-1] - xc[:-1, :-1]
    nxt_dy[:-1] = yc[1:, :-1] - yc[:-1, :-1]
    nxt_dx[-1] = xc[-1, :-1] - xc[-2, :-1]
    nxt_dy[-1] = yc[-1, :-1] - yc[-2, :-1]
    sgn = np.sign(lr_xn * nxt_dx + lr_yn * nxt_dy)
    lr_xn, lr_yn = lr_xn * sgn, lr_yn * sgn
    lr_a = edge * (np.abs(yc[:, 1:] + yc[:, :-1]) / 2 * ARC_3D) if axisymmetric else edge

    # bt faces (GENERATE_MESH.jl:197-239)
    dxb = xc[1:, :] - xc[:-1, :]
    dyb = yc[1:, :] - yc[:-1, :]
    edge_b = np.sqrt(dxb**2 + dyb**2)
    bt_xn = dyb / edge_b
    bt_yn = -dxb / edge_b
    up_dx = np.empty_like(dxb)
    up_dy = np.empty_like(dyb)
    up_dx[:, :-1] = xc[:-1, 1:] - xc[:-1, :-1]
    up_dy[:, :-1] = yc[:-1, 1:] - yc[:-1, :-1]
    up_dx[:, -1] = xc[:-1, -1] - xc[:-1, -2]
    up_dy[:, -1] = yc[:-1, -1] - yc[:-1, -2]
    sgn = np.sign(bt_xn * up_dx + bt_yn * up_dy)
    bt_xn, bt_yn = bt_xn * sgn, bt_yn * sgn
    bt_a = edge_b * (np.abs(yc[1:, :] + yc[:-1, :]) / 2 * ARC_3D) if axisymmetric else edge_b

    # polygon (shoelace) area of each cell (GENERATE_MESH.jl:259-271)
    x1, y1 = xc[:-1, :-1], yc[:-1, :-1]
    x2, y2 = xc[1:, :-1], yc[1:, :-1]
    x3, y3 = xc[1:, 1:], yc[1:, 1:]
    x4, y4 = xc[:-1, 1:], yc[:-1, 1:]
    shoe = -x1 * y2 + x2 * y1
    shoe = shoe - x2 * y3 + x3 * y2
    shoe = shoe - x3 * y4 + x4 * y3
    shoe = shoe - x4 * y1 + x1 * y4
    area = np.abs(shoe / 2)
    arrays = {}
    if axisymmetric:
        # six tetrahedra of the wedge cell (GENERATE_MESH.jl:272-295)
        def P(xx, yy, sgn_):
            return np.stack([xx, yy, sgn_ * yy / 2 * ARC_3D], axis=-1)
        c1, c2, c3, c4 = P(x1, y1, 1), P(x2, y2, 1), P(x3, y3, 1), P(x4, y4, 1)
        c5, c6, c7, c8 = P(x1, y1, -1), P(x2, y2, -1), P(x3, y3, -1), P(x4, y4, -1)
        vol = (_tet_volume(c1, c2, c4, c6) + _tet_volume(c2, c6, c4, c3) + _tet_volume(c6, c4, c3, c7)
               + _tet_volume(c1, c4, c8, c6) + _tet_volume(c8, c4, c6, c7) + _tet_volume(c5, c1, c6, c8))
        th_fb = math.atan(ARC_3D / 2)
        arrays["fb_area"] = _f(area)
        arrays["fb_yn_front"] = math.sin(th_fb)
        arrays["fb_yn_back"] = -math.sin(th_fb)
    else:
        vol = area
    arrays.update(
        lr_xn=_f(lr_xn), lr_yn=_f(lr_yn), lr_a=_f(lr_a),
        bt_xn=_f(bt_xn), bt_yn=_f(bt_yn), bt_a=_f(bt_a),
        vol=_f(vol), x_ext=_f(x_ext), y_ext=_f(y_ext),
        x_corner=xc, y_corner=yc, x=_f(x), y=_f(y),
        chi=_f(chi_c), eta=_f(eta_c), chi1=np.ascontiguousarray(chi_c[:, 0]),
    )
    return Mesh(nchi=nchi, neta=neta, axisymmetric=axisymmetric, arrays=arrays)


def check_mesh_closure(mesh: Mesh) -> float:
    """CHECK_MESH.jl:36-77: max over cells of |Σ face area * normal| (2-D identity)."""
    a = mesh.arrays
    sx = (a["lr_xn"][1:] * a["lr_a"][1:] - a["lr_xn"][:-1] * a["lr_a"][:-1]
          + a["bt_xn"][:, 1:] * a["bt_a"][:, 1:] - a["bt_xn"][:, :-1] * a["bt_a"][:, :-1])
    sy = (a["lr_yn"][1:] * a["lr_a"][1:] - a["lr_yn"][:-1] * a["lr_a"][:-1]
          + a["bt_yn"][:, 1:] * a["bt_a"][:, 1:] - a["bt_yn"][:, :-1] * a["bt_a"][:, :-1])
    return float(max(np.abs(sx).max(), np.abs(sy).max()))
