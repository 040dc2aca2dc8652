// HYMOR hot-path ORACLE — CPU restatement of the reference Julia path.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product (`hymor_gb300/`, `libhymor`)
// links, loads or calls this file; only `tests/`, `__graft_entry__.smoke()` and
// `bench.py`'s CPU-baseline leg do, and only as the checker / the timed CPU
// baseline.
//
// Parity status: PARTIALLY PINNED. The reference is Julia (+ MATLAB twin); no
// Julia, MATLAB or Octave exists on either machine and the reference ships no
// golden vectors or test suite, so the oracle cannot be compared against the
// reference's own outputs. It is pinned by the known answers the reference
// states or implies (uniform-freestream fixed point, CPG normal-shock ratios of
// INITIAL_SOLUTION_POST_SHOCK, the closed-surface mesh identity of CHECK_MESH,
// the CHECK_LINEARIZATION_L consistency metric), by an independent numpy
// restatement of the residual (tests/golden/make_golden.py), and — for the
// smoothing spline taken from BSplineKit, which is not vendored — by scipy's
// make_smoothing_spline, which minimises the same objective.
//
// Every function restates one reference function, cited as file:line relative to
// the reference project root. Arrays follow the reference layout: column-major,
// chi (i) fastest; conserved variables and p/T/a are ghosted (Nchi+2)x(Neta+2);
// fluxes and cell arrays are Nchi x Neta; lr faces (Nchi+1) x Neta; bt faces
// Nchi x (Neta+1); corners (Nchi+1) x (Neta+1). Indices below are 1-based like
// the reference, through the accessor lambdas.
//
// Compile with -ffp-contract=off: the reference's broadcasts never fuse a*b+c,
// and the restatement keeps each expression's association order.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Boundary-condition codes (names as in APPLY_BOUNDARY_CONDITIONS.jl).
enum {
  ORC_BC_SYMMETRY = 0,
  ORC_BC_NO_SLIP_ADIABATIC = 1,
  ORC_BC_NO_SLIP_ISOTHERMAL = 2,
  ORC_BC_OUTFLOW_SUPERSONIC = 3,
  ORC_BC_OUTFLOW_SUPERSONIC_1ST = 4,
  ORC_BC_OUTFLOW_SUBSONIC = 5,
  ORC_BC_OUTFLOW_NRCBC = 6,
  ORC_BC_INFLOW_SUPERSONIC = 7,
  ORC_BC_INFLOW_SUBSONIC = 8,
  ORC_BC_PERIODIC = 9,
  ORC_BC_SHOCK = 10,
};

enum { ORC_MAP_CIRCLE = 0, ORC_MAP_BLUNT_CONE = 1, ORC_MAP_CHANNEL = 2, ORC_MAP_WEDGE = 3 };

// Same field layout as `hymor_config` in include/hymor.h (the Python side builds
// one ctypes structure for both).
typedef struct {
  int32_t nchi, neta;
  int32_t axisymmetric;   // PDE_dimension: 0 = "2D", 1 = "3D-axisymmetric"
  int32_t bc_chi0, bc_chi1, bc_eta0, bc_eta1;
  int32_t shock_enabled, shock_feedback;
  int32_t shock_interp;       // 1, 2, 3 ("1st", "2nd", "3rd")
  int32_t shock_eulerian;     // 0 = Lagrangian, 1 = Eulerian
  int32_t mapping;            // ORC_MAP_*
  int32_t rk_variant;         // 0 = reference Julia (aliased stages), 1 = classical RK4
  int32_t viscosity_model;    // 0 = constant (reference CPG), 1 = Sutherland (extension)
  int32_t perturb_shock;      // stability_analysis.perturb_shock
  double gamma, Pr, Re, Mach;
  double Tw_chi0, Tw_eta0, Tw_eta1;  // wall temperature ratios (T_w / T_inf)
  double cv, energy_factor;          // freestream cv and energy factor (SET_FREESTREAM_PROPERTIES)
  double rho_0, rho_u_0, rho_v_0, rho_E_0, p_0;
  double dist_kx, dist_ky, dist_amp[4];
  double relaxation, spline_param;
  double R, dRs, dRe, circle_angle_extra;
  double L, theta, initial_beta;
  double Lx, Ly, channel_angle, eta_refinement_power;
  double rho_min;
  double CFL, max_dt;
  double perturbation_magnitude;
  double sutherland_S;  // S / T_inf for the Sutherland extension
} orc_config;

typedef struct {
  const double *lr_xn, *lr_yn, *lr_a;  // (Nchi+1) x Neta
  const double *bt_xn, *bt_yn, *bt_a;  // Nchi x (Neta+1)
  const double *vol;                   // Nchi x Neta
  const double *x_ext, *y_ext;         // (Nchi+2) x (Neta+2)
  const double *x_corner, *y_corner;   // (Nchi+1) x (Neta+1)
  const double *chi1;                  // Nchi: mesh["chi"][:, 1]
  const double *fb_area;               // Nchi x Neta (axisymmetric only, else NULL)
  double fb_yn_front, fb_yn_back;
} orc_mesh;

}  // extern "C"

namespace {

typedef std::vector<double> vec;

struct Mesh {
  int nchi, neta;
  vec lr_xn, lr_yn, lr_a, bt_xn, bt_yn, bt_a, vol, x_ext, y_ext, x_corner, y_corner, chi1,
      fb_area, x, y;
  double fb_yn_front = 0, fb_yn_back = 0;
};

// One solution "Dict": the fields of the reference's `s` that the hot path reads
// or writes.
struct State {
  vec rho, rho_u, rho_v, rho_E;  // ghosted
  vec p, T, a;                   // ghosted derived fields (persist like the Dict's)
  vec pts_x, pts_y, pts_chi, pts_eta;
  std::vector<int> cell_idx;  // 1-based, like shock["cell_indices"]
  vec flow;                   // Nchi x Neta, shock["flow_cells"]
  vec beta, speed_x, speed_y, rel_vel;
  vec flux_rho, flux_rho_u, flux_rho_v, flux_rho_E;  // Nchi x Neta
  // prescribed per-column upstream state (s["rho_0_upstream_p"] with freestream
  // rho_0_p, rho_u_0_p, rho_v_0_p, rho_E_0_p, 4 x Nchi), empty when absent
  vec up_cols;
  double t = 0, dt = 0;
  int rho_limited = 0;
  int rh_warnings = 0;
};

struct Ctx {
  orc_config c;
  Mesh m;
  State s;
  int nthreads = 1;
};

inline double sq(double x) { return x * x; }
inline double jsign(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); }

// ---------------------------------------------------------------------------
// Index helpers (1-based).
struct Dims {
  int nchi, neta;
  int gi(int i, int j) const { return (i - 1) + (j - 1) * (nchi + 2); }    // ghosted
  int ci(int i, int j) const { return (i - 1) + (j - 1) * nchi; }          // cells
  int lri(int i, int j) const { return (i - 1) + (j - 1) * (nchi + 1); }   // lr faces
  int bti(int i, int j) const { return (i - 1) + (j - 1) * nchi; }         // bt faces
  int cni(int i, int j) const { return (i - 1) + (j - 1) * (nchi + 1); }   // corners
};

// ---------------------------------------------------------------------------
// utils/Operators/UPDATE_THERMODYNAMIC_PROPERTIES.jl:1-34 (CPG: cv* = 1).
void update_thermo(const orc_config& c, State& s) {
  const Dims d{c.nchi, c.neta};
  const int G = (c.nchi + 2) * (c.neta + 2);
  const double gs = c.gamma;  // gamma_star filled with freestream gamma (UPDATE_CHEMISTRY_EQUILIBRIUM.jl:73-76)
  s.p.resize(G);
  s.T.resize(G);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < G; ++k) {
    double e = (s.rho_E[k] - (s.rho_u[k] * s.rho_u[k] + s.rho_v[k] * s.rho_v[k]) / s.rho[k] / 2) /
               s.rho[k];
    s.p[k] = s.rho[k] * e * (gs - 1);
    s.T[k] = e / 1.0;
  }
  if (c.bc_eta0 == ORC_BC_NO_SLIP_ISOTHERMAL) {
    for (int i = 1; i <= c.nchi + 2; ++i) s.p[d.gi(i, 1)] = 2 * s.p[d.gi(i, 2)] - s.p[d.gi(i, 3)];
  }
}

// utils/Operators/UPDATE_SOUND_SPEED.jl:31-36 (CPG branch).
void update_sound_speed(const orc_config& c, State& s) {
  const int G = (c.nchi + 2) * (c.neta + 2);
  s.a.resize(G);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < G; ++k) s.a[k] = std::sqrt(c.gamma * s.p[k] / s.rho[k]);
}

// ---------------------------------------------------------------------------
// utils/Mesh/GO_TO_ELEMENT_SPACE.jl:28-140 (circle, blunt_cone, channel, wedge).
void go_to_element_space(const orc_config& c, int n, const double* x, const double* y, double* chi,
                         double* eta) {
  if (c.mapping == ORC_MAP_CIRCLE) {
    const double angle_min = -c.circle_angle_extra;
    const double angle_max = M_PI / 2;
    for (int k = 0; k < n; ++k) {
      // mod(atan(-x, y) + pi/2, 2pi) - pi/2 ; Julia mod has the sign of the divisor.
      double t = std::atan2(-x[k], y[k]) + M_PI / 2;
      double m = std::fmod(t, 2 * M_PI);
      if (m != 0 && m < 0) m += 2 * M_PI;
      double angle = m - M_PI / 2;
      double ch = (angle_max - angle) / (angle_max - angle_min);
      double r = std::sqrt(x[k] * x[k] + y[k] * y[k]);
      double distance_max = c.dRs + (c.dRe - c.dRs) * (ch * ch);
      chi[k] = ch;
      eta[k] = (r - c.R) / distance_max;
    }
  } else if (c.mapping == ORC_MAP_BLUNT_CONE) {
    const double Lm = c.L, Rm = c.R, th = c.theta, ib = c.initial_beta;
    const double s_Straight = ((Lm - Rm) + Rm * std::cos(th)) / std::sin(th);
    const double s_Curve = 2 * th * Rm;
    const double s_tot = s_Curve + 2 * s_Straight;
    const double s_Str_sh = ((Lm - Rm) + Rm * std::cos(ib)) / std::sin(ib);
    const double s_Crv_sh = ib * Rm;
    const double s_tot_sh = 2 * s_Crv_sh + 2 * s_Str_sh;
    const double slope = std::sin(th - ib);
    for (int k = 0; k < n; ++k) {
      double x_body = y[k];
      double y_body = -x[k];
      double tang = (y_body - (Lm - Rm)) / x_body;
      double eta_phys, chi_arc;
      if ((tang < std::tan(M_PI / 2 - th)) && (x_body > 0)) {
        eta_phys = y_body * std::cos(th) + x_body * std::sin(th) - Rm - (Lm - Rm) * std::cos(th);
        double lambda = (x_body / std::cos(th) - (eta_phys * std::sin(th) + Rm * std::sin(th)) / std::cos(th)) / s_tot;
        chi_arc = s_Straight / s_tot - lambda;
      } else if ((-std::tan(M_PI / 2 - th) < tang) && (x_body < 0)) {
        eta_phys = y_body * std::cos(th) - x_body * std::sin(th) - Rm - (Lm - Rm) * std::cos(th);
        double lambda = (-x_body / std::cos(th) - (eta_phys * std::sin(th) + Rm * std::sin(th)) / std::cos(th)) / s_tot;
        chi_arc = (s_Straight + s_Curve) / s_tot + lambda;
      } else {
        double angle = std::atan2((y_body + Rm - Lm), x_body);
        eta_phys = x_body / std::cos(angle) - Rm;
        chi_arc = (angle - M_PI / 2 + th) / (2 * th * s_tot / s_Curve) + s_Straight / s_tot;
      }
      double ch = 1 - 2 * chi_arc;
      double distance_max;
      if (chi_arc < s_Str_sh / s_tot_sh)
        distance_max = c.dRs + (s_Str_sh - chi_arc * s_tot_sh) * slope;
      else
        distance_max = c.dRs;
      chi[k] = ch;
      eta[k] = eta_phys / distance_max;
    }
  } else if (c.mapping == ORC_MAP_CHANNEL) {
    const double p = c.eta_refinement_power;
    for (int k = 0; k < n; ++k) {
      double ch = (x[k] * std::cos(c.channel_angle) + y[k] * std::sin(c.channel_angle)) / c.Lx;
      double eta_r = (-x[k] * std::sin(c.channel_angle) + y[k] * std::cos(c.channel_angle)) / c.Ly;
      double e;
      if (eta_r <= 0.5)
        e = std::pow(eta_r / std::pow(2.0, p - 1), 1 / p);
      else
        e = 1 - std::pow((1 - eta_r) / std::pow(2.0, p - 1), 1 / p);
      chi[k] = ch;
      eta[k] = e;
    }
  } else {  // wedge
    for (int k = 0; k < n; ++k) {
      double ch = 1 - y[k] / c.Lx;
      double distance_max = c.dRs + (c.dRe - c.dRs) * (1 - ch);
      chi[k] = ch;
      eta[k] = -x[k] / distance_max;
    }
  }
}

// ---------------------------------------------------------------------------
// Natural cubic smoothing spline (the objective of BSplineKit 0.19.2
// `fit(BSplineOrder(4), x, y, λ)`: minimise Σ (y_i - f(x_i))² + λ ∫ f''²),
// solved with Reinsch's algorithm (Green & Silverman 1994, §2.3): with knot
// spacings h, tridiagonal R and Q, solve (R + λ QᵀQ) γ = Qᵀ y for the interior
// second derivatives γ, then g = y - λ Q γ. Call sites:
// utils/Shock_fitting/LEAST_SQUARES_SHOCK_POINTS.jl:52-58 (fit + Linear()
// extrapolation) and CSAPS.jl:23-31 (first derivative).
struct SmoothingSpline {
  int n = 0;
  vec x, g, gam;  // knots, fitted values, second derivatives (gam[0] = gam[n-1] = 0)

  void fit(int n_, const double* xs, const double* ys, double lambda) {
    n = n_;
    x.assign(xs, xs + n);
    g.assign(n, 0.0);
    gam.assign(n, 0.0);
    if (n < 3) {
      for (int k = 0; k < n; ++k) g[k] = ys[k];
      return;
    }
    vec h(n - 1);
    for (int k = 0; k < n - 1; ++k) h[k] = x[k + 1] - x[k];
    const int m = n - 2;  // unknowns gam[1..n-2]
    // Q columns j = 1..n-2 (0-based interior index jj = j-1): nonzeros at rows j-1, j, j+1.
    auto qm = [&](int j) { return 1.0 / h[j - 1]; };                     // row j-1
    auto q0 = [&](int j) { return -1.0 / h[j - 1] - 1.0 / h[j]; };      // row j
    auto qp = [&](int j) { return 1.0 / h[j]; };                         // row j+1
    // Symmetric pentadiagonal A = R + λ QᵀQ, stored as bands d0, d1, d2.
    vec d0(m), d1(m, 0.0), d2(m, 0.0), rhs(m);
    for (int jj = 0; jj < m; ++jj) {
      int j = jj + 1;
      d0[jj] = (h[j - 1] + h[j]) / 3 + lambda * (qm(j) * qm(j) + q0(j) * q0(j) + qp(j) * qp(j));
      if (jj + 1 < m) {
        int k = j + 1;  // column k shares rows j, j+1 with column j
        d1[jj] = h[j] / 6 + lambda * (q0(j) * qm(k) + qp(j) * q0(k));
      }
      if (jj + 2 < m) {
        int k = j + 2;  // shares row j+1
        d2[jj] = lambda * (qp(j) * qm(k));
      }
      rhs[jj] = qm(j) * ys[j - 1] + q0(j) * ys[j] + qp(j) * ys[j + 1];
    }
    // Banded Cholesky A = L Lᵀ, L lower with bands l0, l1, l2.
    vec l0(m), l1(m, 0.0), l2(m, 0.0);
    for (int jj = 0; jj < m; ++jj) {
      double a = d0[jj];
      if (jj >= 1) a -= l1[jj - 1] * l1[jj - 1];
      if (jj >= 2) a -= l2[jj - 2] * l2[jj - 2];
      l0[jj] = std::sqrt(a);
      if (jj + 1 < m) {
        double b = d1[jj];
        if (jj >= 1) b -= l2[jj - 1] * l1[jj - 1];
        l1[jj] = b / l0[jj];
      }
      if (jj + 2 < m) l2[jj] = d2[jj] / l0[jj];
    }
    vec z(m);
    for (int jj = 0; jj < m; ++jj) {
      double v = rhs[jj];
      if (jj >= 1) v -= l1[jj - 1] * z[jj - 1];
      if (jj >= 2) v -= l2[jj - 2] * z[jj - 2];
      z[jj] = v / l0[jj];
    }
    for (int jj = m - 1; jj >= 0; --jj) {
      double v = z[jj];
      if (jj + 1 < m) v -= l1[jj] * gam[jj + 2];
      if (jj + 2 < m) v -= l2[jj] * gam[jj + 3];
      gam[jj + 1] = v / l0[jj];
    }
    // g = y - λ Q γ
    for (int r = 0; r < n; ++r) {
      double qg = 0;
      if (r - 1 >= 1 && r - 1 <= n - 2) qg += qp(r - 1) * gam[r - 1];
      if (r >= 1 && r <= n - 2) qg += q0(r) * gam[r];
      if (r + 1 >= 1 && r + 1 <= n - 2) qg += qm(r + 1) * gam[r + 1];
      g[r] = ys[r] - lambda * qg;
    }
  }

  int interval(double t) const {
    // index k with x[k] <= t < x[k+1], clamped to [0, n-2]
    int lo = 0, hi = n - 1;
    if (t <= x[0]) return 0;
    if (t >= x[n - 1]) return n - 2;
    while (hi - lo > 1) {
      int mid = (lo + hi) / 2;
      if (x[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
  }
  double eval_in(int k, double t) const {
    double h = x[k + 1] - x[k];
    double a = x[k + 1] - t, b = t - x[k];
    return (a * g[k] + b * g[k + 1]) / h +
           ((a * a * a - h * h * a) * gam[k] + (b * b * b - h * h * b) * gam[k + 1]) / (6 * h);
  }
  double deriv_in(int k, double t) const {
    double h = x[k + 1] - x[k];
    double a = x[k + 1] - t, b = t - x[k];
    return (g[k + 1] - g[k]) / h +
           ((h * h - 3 * a * a) * gam[k] + (3 * b * b - h * h) * gam[k + 1]) / (6 * h);
  }
  // Value with BSplineKit.Linear() extrapolation outside [x_1, x_n].
  double eval(double t) const {
    if (n < 2) return g.empty() ? 0.0 : g[0];
    if (t < x[0]) return g[0] + deriv_in(0, x[0]) * (t - x[0]);
    if (t > x[n - 1]) return g[n - 1] + deriv_in(n - 2, x[n - 1]) * (t - x[n - 1]);
    int k = interval(t);
    return eval_in(k, t);
  }
  double deriv(double t) const {
    if (n < 2) return 0.0;
    if (t < x[0]) return deriv_in(0, x[0]);
    if (t > x[n - 1]) return deriv_in(n - 2, x[n - 1]);
    return deriv_in(interval(t), t);
  }
};

// ---------------------------------------------------------------------------
// Shock fitting.

// utils/Shock_fitting/LEAST_SQUARES_SHOCK_POINTS.jl:36-73; the fitted splines are
// returned for COMPUTE_BETA.
void least_squares_shock_points(const orc_config& c, const Mesh& m, State& s, SmoothingSpline& sx,
                                SmoothingSpline& sy) {
  const double p = c.spline_param;
  const double lambda = (1 - p) / p;
  const int n = c.nchi;
  sx.fit(n, s.pts_chi.data(), s.pts_x.data(), lambda);
  sy.fit(n, s.pts_chi.data(), s.pts_y.data(), lambda);
  for (int i = 0; i < n; ++i) {
    s.pts_x[i] = sx.eval(m.chi1[i]);
    s.pts_y[i] = sy.eval(m.chi1[i]);
  }
  go_to_element_space(c, n, s.pts_x.data(), s.pts_y.data(), s.pts_chi.data(), s.pts_eta.data());
}

// utils/Shock_fitting/COMPUTE_UPSTREAM_CONDITIONS.jl:31-112 (UPDATE_SHOCK_UPSTREAM
// + COMPUTE_UPSTREAM_CONDITIONS): freestream state at the shock points.
void compute_upstream_conditions(const orc_config& c, const State& s, vec& p_inf, vec& u_inf,
                                 vec& v_inf, vec& rho_inf) {
  const int n = c.nchi;
  const double u_y = c.rho_v_0 / c.rho_0, u_x = c.rho_u_0 / c.rho_0;
  const double two_pi_ky = 2.0 * M_PI * c.dist_ky, two_pi_kx = 2.0 * M_PI * c.dist_kx;
  const double u_y_t = u_y * s.t, u_x_t = u_x * s.t;
  p_inf.resize(n);
  u_inf.resize(n);
  v_inf.resize(n);
  rho_inf.resize(n);
  const double gm1 = c.gamma - 1.0;
  for (int i = 0; i < n; ++i) {
    double pert = std::cos(two_pi_ky * (s.pts_y[i] - u_y_t)) * std::sin(two_pi_kx * (s.pts_x[i] - u_x_t));
    double rho = c.rho_0 + pert * c.dist_amp[0];
    double rho_u = c.rho_u_0 + pert * c.dist_amp[1];
    double rho_v = c.rho_v_0 + pert * c.dist_amp[2];
    double rho_E = c.rho_E_0 + pert * c.dist_amp[3];
    if (!s.up_cols.empty()) {  // :87-91
      rho = s.up_cols[i];
      rho_u = s.up_cols[n + i];
      rho_v = s.up_cols[2 * n + i];
      rho_E = s.up_cols[3 * n + i];
    }
    if (c.axisymmetric && i == 0) rho_v = 0;
    double vi = rho_v / rho;
    double ui = rho_u / rho;
    double u_mag = std::sqrt(vi * vi + ui * ui);
    double e_inf = (rho_E - rho * (u_mag * u_mag) * 0.5) / rho;
    p_inf[i] = e_inf * rho * gm1;
    u_inf[i] = ui;
    v_inf[i] = vi;
    rho_inf[i] = rho;
  }
}

// utils/Shock_fitting/COMPUTE_BETA.jl:30-53 (+ UPDATE_SHOCK_BC.jl:31-34 symmetry fix
// applied by the caller).
void compute_beta(const orc_config& c, const Mesh& m, State& s, const SmoothingSpline& sx,
                  const SmoothingSpline& sy) {
  vec p_inf, u_inf, v_inf, rho_inf;
  compute_upstream_conditions(c, s, p_inf, u_inf, v_inf, rho_inf);
  s.beta.resize(c.nchi);
  for (int i = 0; i < c.nchi; ++i) {
    double dx = sx.deriv(m.chi1[i]);
    double dy = sy.deriv(m.chi1[i]);
    double cross_tv = dx * v_inf[i] - dy * u_inf[i];
    double dot_tv = dx * u_inf[i] + dy * v_inf[i];
    s.beta[i] = std::atan2(std::fabs(cross_tv), std::fabs(dot_tv));
  }
}

// utils/Shock_fitting/UPDATE_FIELD_UPSTREAM.jl:32-113: cells j >= sc+2 (ghosted
// sc+3:end) of every interior column become the (disturbed) freestream.
void update_field_upstream(const orc_config& c, const Mesh& m, State& s) {
  const Dims d{c.nchi, c.neta};
  const double u_y = c.rho_v_0 / c.rho_0, u_x = c.rho_u_0 / c.rho_0;
  const double two_pi_ky = 2.0 * M_PI * c.dist_ky, two_pi_kx = 2.0 * M_PI * c.dist_kx;
  const double u_x_t = u_x * s.t, u_y_t = u_y * s.t;
  for (int i = 1; i <= c.nchi; ++i) {
    int sc = s.cell_idx[i - 1];
    for (int jg = sc + 3; jg <= c.neta + 2; ++jg) {
      int k = d.gi(i + 1, jg);
      if (!s.up_cols.empty()) {  // prescribed per-column upstream state (:75-90)
        const int n = c.nchi;
        s.rho[k] = s.up_cols[i - 1];
        s.rho_u[k] = s.up_cols[n + i - 1];
        s.rho_v[k] = s.up_cols[2 * n + i - 1];
        s.rho_E[k] = s.up_cols[3 * n + i - 1];
        continue;
      }
      double pert = std::cos(two_pi_ky * (m.y_ext[k] - u_y_t)) * std::sin(two_pi_kx * (m.x_ext[k] - u_x_t));
      s.rho[k] = c.rho_0 + pert * c.dist_amp[0];
      s.rho_u[k] = c.rho_u_0 + pert * c.dist_amp[1];
      s.rho_v[k] = c.rho_v_0 + pert * c.dist_amp[2];
      s.rho_E[k] = c.rho_E_0 + pert * c.dist_amp[3];
    }
  }
}

// The shock chain reads rows sc-1 .. sc+2 of each column (UPDATE_SHOCK_JUMP_PROPERTIES.jl,
// EXTRAPOLATE_CELLS_SHOCK.jl), so a shocked row outside 2..Neta-1 is a Julia BoundsError
// in the reference; the oracle raises it as an exception instead of indexing past its arrays.
void check_shock_rows(const orc_config& c, const State& s) {
  for (int i = 0; i < c.nchi; ++i) {
    const int sc = s.cell_idx[i];
    if (sc < 2 || sc > c.neta - 1)
      throw std::out_of_range("shocked row " + std::to_string(sc) + " of column " + std::to_string(i + 1) +
                              " outside 2.." + std::to_string(c.neta - 1));
  }
}

// utils/Shock_fitting/EXTRAPOLATE_CELLS_SHOCK.jl:39-176.
void extrapolate_cells_shock(const orc_config& c, State& s) {
  check_shock_rows(c, s);
  const Dims d{c.nchi, c.neta};
  for (int i = 1; i <= c.nchi; ++i) {
    int j = s.cell_idx[i - 1];
    int i0 = d.gi(i + 1, j + 1), i1 = d.gi(i + 1, j + 2), i2 = d.gi(i + 1, j + 3);
    int im1 = d.gi(i + 1, j), im2 = d.gi(i + 1, j - 1);
    double* arr[5] = {s.rho.data(), s.rho_u.data(), s.rho_v.data(), s.rho_E.data(), s.p.data()};
    if (c.shock_interp == 1) {
      for (int v = 0; v < 5; ++v) { arr[v][i1] = arr[v][i0]; arr[v][i2] = arr[v][i0]; }
    } else if (c.shock_interp == 2) {
      for (int v = 0; v < 5; ++v) arr[v][i1] = 2 * arr[v][i0] - arr[v][im1];
      for (int v = 0; v < 4; ++v) arr[v][i2] = 2 * arr[v][i1] - arr[v][i0];
    } else {
      for (int v = 0; v < 5; ++v) arr[v][i1] = 3 * arr[v][i0] - 3 * arr[v][im1] + arr[v][im2];
      for (int v = 0; v < 4; ++v) arr[v][i2] = 3 * arr[v][i1] - 3 * arr[v][i0] + arr[v][im1];
    }
  }
}

// utils/Shock_fitting/UPDATE_SHOCK_JUMP_PROPERTIES.jl:324-522
// (UPDATE_SHOCK_JUMP_PROPERTIES_PRESSURE_3, CPG branch).
void update_shock_jump_properties(const orc_config& c, const Mesh& m, State& s) {
  check_shock_rows(c, s);
  const Dims d{c.nchi, c.neta};
  const int n = c.nchi;
  vec p_inf, u_inf, v_inf, rho_inf;
  compute_upstream_conditions(c, s, p_inf, u_inf, v_inf, rho_inf);
  update_field_upstream(c, m, s);
  s.speed_x.resize(n);
  s.speed_y.resize(n);
  s.rel_vel.resize(n);
  const double gamma_s = c.gamma, gamma_inf = c.gamma;
  for (int i = 1; i <= n; ++i) {
    int sc = s.cell_idx[i - 1];
    // cell centres (mesh x, y = interior of x_Ext, y_Ext)
    double x_0 = m.x_ext[d.gi(i + 1, sc + 1)], y_0 = m.y_ext[d.gi(i + 1, sc + 1)];
    double x_1 = m.x_ext[d.gi(i + 1, sc)], y_1 = m.y_ext[d.gi(i + 1, sc)];
    double x_2 = m.x_ext[d.gi(i + 1, sc - 1)], y_2 = m.y_ext[d.gi(i + 1, sc - 1)];
    double x_s = s.pts_x[i - 1], y_s = s.pts_y[i - 1];
    double dist01 = std::sqrt(sq(x_0 - x_1) + sq(y_0 - y_1));
    double dist12 = std::sqrt(sq(x_1 - x_2) + sq(y_1 - y_2));
    double dist1s = ((x_s - x_1) * (x_1 - x_2) + (y_s - y_1) * (y_1 - y_2)) / dist12;
    double dist0s = ((x_s - x_0) * (x_0 - x_1) + (y_s - y_0) * (y_0 - y_1)) / dist01;
    int g1 = d.gi(i + 1, sc + 1 - 1), g2 = d.gi(i + 1, sc + 1 - 2);
    double p_1 = s.p[g1], p_2 = s.p[g2];
    double slope_p = (p_1 - p_2) / dist12;
    double rho_1 = s.rho[g1], rho_2 = s.rho[g2];
    double slope_rho = (rho_1 - rho_2) / dist12;
    double slope_rho_u = (s.rho_u[g1] - s.rho_u[g2]) / dist12;
    double slope_rho_v = (s.rho_v[g1] - s.rho_v[g2]) / dist12;
    double slope_rho_E = (s.rho_E[g1] - s.rho_E[g2]) / dist12;
    double p_s = slope_p * dist1s + p_1;
    double y = p_s / p_inf[i - 1];
    if (y < 1) s.rh_warnings++;
    double A = (gamma_s + 1) / (gamma_s - 1);
    double B = (gamma_inf + 1) / (gamma_inf - 1);
    double rho_s = rho_inf[i - 1] * (y * A + 1) / (y + B);
    double e_s = p_s / ((gamma_s - 1) * rho_s);
    double beta = s.beta[i - 1];
    double ang_inf = beta - std::atan2(v_inf[i - 1], u_inf[i - 1]);
    double vmag = std::sqrt(sq(u_inf[i - 1]) + sq(v_inf[i - 1]));
    double normal_velocity_inf = std::sin(ang_inf) * vmag;
    double temp1 = 2 * y / (gamma_s - 1) - 2 / (gamma_inf - 1);
    double temp2 = y * A + 1;
    double temp3 = p_inf[i - 1] * (y - 1) / rho_inf[i - 1];
    double rel = -normal_velocity_inf + std::sqrt(temp3 * temp2 / temp1);
    s.rel_vel[i - 1] = rel;
    double tangential_velocity_s = std::cos(ang_inf) * vmag;
    double normal_velocity_s = -rel + rho_inf[i - 1] / rho_s * (rel + normal_velocity_inf);
    if (!c.shock_eulerian) {
      s.speed_x[i - 1] = -rel * std::sin(beta);
      s.speed_y[i - 1] = rel * std::cos(beta);
    } else {
      double sx = -rel * std::sin(beta);
      double sy = rel * std::cos(beta);
      s.speed_x[i - 1] = sx - sy * std::tan(M_PI / 2 - beta);
      s.speed_y[i - 1] = 0.0;
    }
    double rho_u_s = rho_s * (normal_velocity_s * std::sin(beta) + tangential_velocity_s * std::cos(beta));
    double rho_v_s = rho_s * (-normal_velocity_s * std::cos(beta) + tangential_velocity_s * std::sin(beta));
    double rho_E_s = e_s * rho_s + (sq(rho_u_s) + sq(rho_v_s)) / (2 * rho_s);
    int g0 = d.gi(i + 1, sc + 1);
    s.rho[g0] = -slope_rho * dist0s + rho_s;
    s.rho_u[g0] = -slope_rho_u * dist0s + rho_u_s;
    s.rho_v[g0] = -slope_rho_v * dist0s + rho_v_s;
    s.rho_E[g0] = -slope_rho_E * dist0s + rho_E_s;
    s.p[g0] = -slope_p * dist0s + p_s;
  }
  extrapolate_cells_shock(c, s);
}

// utils/Shock_fitting/UPDATE_SHOCK_BC.jl:26-40.
void update_shock_bc(const orc_config& c, const Mesh& m, State& s) {
  if (!c.shock_enabled) return;
  SmoothingSpline sx, sy;
  least_squares_shock_points(c, m, s, sx, sy);
  compute_beta(c, m, s, sx, sy);
  if (c.bc_chi0 == ORC_BC_SYMMETRY) s.beta[0] = M_PI / 2;
  update_shock_jump_properties(c, m, s);
  extrapolate_cells_shock(c, s);
}

// utils/Shock_fitting/DETECT_CELLS_SHOCKED.jl:34-88.
void detect_cells_shocked(const orc_config& c, const Mesh& m, State& s) {
  const Dims d{c.nchi, c.neta};
  s.cell_idx.resize(c.nchi);
  s.flow.assign((size_t)c.nchi * c.neta, 0.0);
  for (int i = 1; i <= c.nchi; ++i) {
    double px = s.pts_x[i - 1], py = s.pts_y[i - 1];
    double min_d = std::numeric_limits<double>::infinity();
    int min_j = 1;
    for (int j = 1; j <= c.neta; ++j) {
      double dx = px - m.x_ext[d.gi(i + 1, j + 1)];
      double dy = py - m.y_ext[d.gi(i + 1, j + 1)];
      double dsq = dx * dx + dy * dy;
      if (dsq < min_d) { min_d = dsq; min_j = j; }
    }
    s.cell_idx[i - 1] = min_j;
    for (int j = 1; j <= min_j - 1; ++j) s.flow[d.ci(i, j)] = 1.0;
  }
}

// utils/Shock_fitting/MOVE_SHOCK.jl:29-49.
void move_shock(const orc_config& c, State& s, const State& ds, double w) {
  const double w_relax = w * c.relaxation;
  for (int i = 0; i < c.nchi; ++i) {
    s.pts_x[i] = s.pts_x[i] + ds.speed_x[i] * w_relax;
    s.pts_y[i] = s.pts_y[i] + ds.speed_y[i] * w_relax;
  }
  if (c.bc_chi0 == ORC_BC_SYMMETRY) s.pts_x[0] = s.pts_x[1];
}

// utils/Shock_fitting/UPDATE_FLOW_CELLS.jl:25-37.
void update_flow_cells(const orc_config& c, const Mesh& m, State& s) {
  if (!c.shock_enabled) return;
  detect_cells_shocked(c, m, s);
  update_field_upstream(c, m, s);
  extrapolate_cells_shock(c, s);
  update_thermo(c, s);
  update_sound_speed(c, s);
}

// utils/Operators/MIN_RHO.jl:1-32.
void min_rho(const orc_config& c, State& s) {
  const Dims d{c.nchi, c.neta};
  for (int j = 2; j <= c.neta + 1; ++j)
    for (int i = 2; i <= c.nchi + 1; ++i) {
      int k = d.gi(i, j);
      if (s.rho[k] < c.rho_min) { s.rho[k] = c.rho_min; s.rho_limited++; }
    }
}

// ---------------------------------------------------------------------------
// utils/Operators/APPLY_BOUNDARY_CONDITIONS.jl:1-828 (all CPG branches except
// lid_driven_cavity). `at(depth, k)` addresses the ghost line (depth 0) and the
// first two interior lines (depth 1, 2) at position k along the edge.
void apply_edge_bc(const orc_config& c, const Mesh& m, State& s, int edge, int bc) {
  const Dims d{c.nchi, c.neta};
  const int NI = c.nchi + 2, NJ = c.neta + 2;
  const bool is_chi = (edge == 0 || edge == 1);
  const int len = is_chi ? NJ : NI;
  // position k (1-based) along the edge -> ghosted linear index of ghost/adjacent/next/periodic source
  auto at = [&](int depth, int k) -> int {
    // depth 0 = ghost, 1 = adjacent interior, 2 = next interior
    if (edge == 0) return d.gi(1 + depth, k);
    if (edge == 1) return d.gi(NI - depth, k);
    if (edge == 2) return d.gi(k, 1 + depth);
    return d.gi(k, NJ - depth);
  };
  auto per = [&](int k) -> int {
    if (edge == 0) return d.gi(NI - 1, k);
    if (edge == 1) return d.gi(2, k);
    if (edge == 2) return d.gi(k, NJ - 1);
    return d.gi(k, 2);
  };
  double* R = s.rho.data();
  double* U = s.rho_u.data();
  double* V = s.rho_v.data();
  double* E = s.rho_E.data();
  double* P = s.p.data();
  double* T = s.T.data();
  auto copy = [&](double* A) { for (int k = 1; k <= len; ++k) A[at(0, k)] = A[at(1, k)]; };
  auto neg = [&](double* A) { for (int k = 1; k <= len; ++k) A[at(0, k)] = -A[at(1, k)]; };
  auto extrap = [&](double* A) {
    for (int k = 1; k <= len; ++k) A[at(0, k)] = 2 * A[at(1, k)] - A[at(2, k)];
  };
  auto fix = [&](double* A, double v) { for (int k = 1; k <= len; ++k) A[at(0, k)] = v; };
  auto wallT = [&](double Tw_ratio) {
    double T_w = Tw_ratio * c.cv / c.energy_factor;
    for (int k = 1; k <= len; ++k) T[at(0, k)] = 2 * T_w - T[at(1, k)];
  };
  auto periodic = [&](double* A) { for (int k = 1; k <= len; ++k) A[at(0, k)] = A[per(k)]; };
  // face normal of the boundary face at position k (2..len-1)
  auto normal = [&](int k, double& nx, double& ny) {
    if (edge == 0) { nx = m.lr_xn[d.lri(1, k - 1)]; ny = m.lr_yn[d.lri(1, k - 1)]; }
    else if (edge == 1) { nx = m.lr_xn[d.lri(c.nchi + 1, k - 1)]; ny = m.lr_yn[d.lri(c.nchi + 1, k - 1)]; }
    else if (edge == 2) { nx = m.bt_xn[d.bti(k - 1, 1)]; ny = m.bt_yn[d.bti(k - 1, 1)]; }
    else { nx = m.bt_xn[d.bti(k - 1, c.neta + 1)]; ny = m.bt_yn[d.bti(k - 1, c.neta + 1)]; }
  };
  const double sgn_out = (edge == 0 || edge == 2) ? -1.0 : 1.0;
  auto lodi = [&]() {
    for (int k = 2; k <= len - 1; ++k) {
      int g = at(0, k), a1 = at(1, k);
      double nx, ny;
      normal(k, nx, ny);
      double a = s.a[a1];
      double rho_int = R[a1];
      double u_n_ghost, u_n_int;
      if (sgn_out < 0) {
        u_n_ghost = -(U[g] * nx + V[g] * ny) / R[g];
        u_n_int = -(U[a1] * nx + V[a1] * ny) / rho_int;
      } else {
        u_n_ghost = (U[g] * nx + V[g] * ny) / R[g];
        u_n_int = (U[a1] * nx + V[a1] * ny) / rho_int;
      }
      bool subsonic = u_n_ghost < a;
      if (subsonic) {
        double p_int = P[a1];
        double p_lodi = p_int + rho_int * a * (u_n_ghost - u_n_int);
        P[g] = p_lodi;
        double rho_e = P[g] / (c.gamma - 1);
        E[g] = rho_e + 0.5 * (U[g] * U[g] + V[g] * V[g]) / R[g];
      }
    }
  };
  auto reflect = [&]() {
    for (int k = 2; k <= len - 1; ++k) {
      int g = at(0, k), a1 = at(1, k);
      double nx, ny;
      normal(k, nx, ny);
      double flux_vel = U[a1] * nx + V[a1] * ny;
      U[g] = U[a1] - 2 * flux_vel * nx;
      V[g] = V[a1] - 2 * flux_vel * ny;
    }
  };
  switch (bc) {
    case ORC_BC_INFLOW_SUBSONIC:
      fix(R, c.rho_0); fix(U, c.rho_u_0); fix(V, c.rho_v_0); extrap(E); extrap(P);
      break;
    case ORC_BC_INFLOW_SUPERSONIC:
      fix(R, c.rho_0); fix(U, c.rho_u_0); fix(V, c.rho_v_0); fix(E, c.rho_E_0); fix(P, c.p_0);
      break;
    case ORC_BC_NO_SLIP_ADIABATIC:
      copy(R); neg(U); neg(V); extrap(E); extrap(P); copy(T);
      break;
    case ORC_BC_NO_SLIP_ISOTHERMAL: {
      copy(R); neg(U); neg(V); extrap(E); extrap(P);
      // the chi1 branch reads boundary_chi0's Tw (APPLY_BOUNDARY_CONDITIONS.jl:275)
      double Tw = (edge == 0 || edge == 1) ? c.Tw_chi0 : (edge == 2 ? c.Tw_eta0 : c.Tw_eta1);
      wallT(Tw);
      break;
    }
    case ORC_BC_OUTFLOW_SUBSONIC:
      extrap(R); extrap(E); extrap(U); extrap(V); copy(P);
      if (edge != 1) copy(T);  // the chi1 branch leaves T untouched (:308-317)
      break;
    case ORC_BC_OUTFLOW_SUPERSONIC:
      extrap(R); extrap(E); extrap(U); extrap(V); extrap(P); copy(T);
      break;
    case ORC_BC_OUTFLOW_SUPERSONIC_1ST:
      copy(U); copy(V); copy(R); copy(E); copy(P); copy(T);
      break;
    case ORC_BC_OUTFLOW_NRCBC:
      extrap(R); extrap(U); extrap(V); extrap(E); extrap(P); copy(T);
      lodi();
      break;
    case ORC_BC_PERIODIC:
      periodic(U); periodic(V); periodic(R); periodic(E); periodic(P); periodic(T);
      break;
    case ORC_BC_SYMMETRY: {
      copy(R); copy(P);
      reflect();
      // ends of the ghost line copy their neighbours on the same line
      if (is_chi) {
        U[at(0, 1)] = U[at(0, 2)]; V[at(0, 1)] = V[at(0, 2)];
        U[at(0, len)] = U[at(0, len - 1)]; V[at(0, len)] = V[at(0, len - 1)];
      } else {
        // eta edges: rho_u[1, g] = rho_u[2, g]; rho_u[end, g] = rho_u[end-1, g]
        U[at(0, 1)] = U[at(0, 2)]; V[at(0, 1)] = V[at(0, 2)];
        U[at(0, len)] = U[at(0, len - 1)]; V[at(0, len)] = V[at(0, len - 1)];
      }
      copy(E); copy(T);
      break;
    }
    case ORC_BC_SHOCK:
      break;
    default:
      break;
  }
}

void apply_boundary_conditions(const orc_config& c, const Mesh& m, State& s) {
  apply_edge_bc(c, m, s, 0, c.bc_chi0);
  apply_edge_bc(c, m, s, 1, c.bc_chi1);
  apply_edge_bc(c, m, s, 2, c.bc_eta0);
  apply_edge_bc(c, m, s, 3, c.bc_eta1);
}

// ---------------------------------------------------------------------------
// Transport coefficients: CPG constant mu* = k* = 1
// (UPDATE_CHEMISTRY_EQUILIBRIUM.jl:103-124), averaged to faces as in VISCOUS_FLUX.jl:136-137.
// Sutherland extension: mu* = T*^{3/2} (1 + S*) / (T* + S*), k* = mu*, evaluated at the
// face temperature T* = (T_L + T_R) / (2 T_inf) (on a wall face this is the wall value).
struct Transport {
  int model;
  double S, Tinf_inv;
  double face(double TL, double TR, double muL = 1.0, double muR = 1.0) const {
    if (model == 1) {
      double Ts = (TL + TR) / 2 * Tinf_inv;
      return Ts * std::sqrt(Ts) * (1 + S) / (Ts + S);
    }
    return (muR + muL) / 2;
  }
};

// utils/Operators/FLUX_MASS.jl:1-44, FLUX_MOMENTUM.jl:1-75, FLUX_TOTAL_ENERGY.jl:1-55,
// and the *_3D variants (FLUX_MOMENTUM_3D.jl:120-125 adds the front/back pressure term).
void inviscid_fluxes(const orc_config& c, const Mesh& m, State& s) {
  const Dims d{c.nchi, c.neta};
  const int nchi = c.nchi, neta = c.neta;
  const size_t N = (size_t)nchi * neta;
  s.flux_rho.assign(N, 0.0);
  s.flux_rho_u.assign(N, 0.0);
  s.flux_rho_v.assign(N, 0.0);
  s.flux_rho_E.assign(N, 0.0);
  const double *R = s.rho.data(), *U = s.rho_u.data(), *V = s.rho_v.data(), *E = s.rho_E.data(),
               *P = s.p.data();
  // face temporaries
  vec f_m((size_t)(nchi + 1) * neta), f_u(f_m.size()), f_v(f_m.size()), f_E(f_m.size());
  vec g_m((size_t)nchi * (neta + 1)), g_u(g_m.size()), g_v(g_m.size()), g_E(g_m.size());
  // lr faces: face (i, j) between ghosted cells (i, j+1) and (i+1, j+1)
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi + 1; ++i) {
      int L = d.gi(i, j + 1), Rr = d.gi(i + 1, j + 1), f = d.lri(i, j);
      double xn = m.lr_xn[f], yn = m.lr_yn[f];
      // FLUX_MASS.jl:24-25
      f_m[f] = (U[L] + U[Rr]) * xn / 2 + (V[L] + V[Rr]) * yn / 2;
      // FLUX_MOMENTUM.jl:71-76
      double rho_u_face = (U[L] + U[Rr]) / 2;
      double P_face_x = (P[L] + P[Rr]) * xn / 2;
      double vel_face = (U[L] + U[Rr]) / (R[Rr] + R[L]) * xn + (V[L] + V[Rr]) / (R[Rr] + R[L]) * yn;
      f_u[f] = (rho_u_face * vel_face + P_face_x);
      double rho_v_face = (V[L] + V[Rr]) / 2;
      double P_face_y = (P[L] + P[Rr]) * yn / 2;
      f_v[f] = (rho_v_face * vel_face + P_face_y);
      // FLUX_TOTAL_ENERGY.jl:146-151
      double rho_E_face = (E[L] + E[Rr]) / 2;
      double P_face = (P[L] + P[Rr]) / 2;
      f_E[f] = ((rho_E_face + P_face) * vel_face);
    }
  // bt faces: face (i, j) between ghosted cells (i+1, j) and (i+1, j+1)
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= neta + 1; ++j)
    for (int i = 1; i <= nchi; ++i) {
      int B = d.gi(i + 1, j), Tt = d.gi(i + 1, j + 1), f = d.bti(i, j);
      double xn = m.bt_xn[f], yn = m.bt_yn[f];
      g_m[f] = (U[B] + U[Tt]) * xn / 2 + (V[B] + V[Tt]) * yn / 2;
      double rho_u_face = (U[B] + U[Tt]) / 2;
      double P_face_x = (P[B] + P[Tt]) * xn / 2;
      double vel_face = (U[B] + U[Tt]) / (R[Tt] + R[B]) * xn + (V[B] + V[Tt]) / (R[Tt] + R[B]) * yn;
      g_u[f] = (rho_u_face * vel_face + P_face_x);
      double rho_v_face = (V[B] + V[Tt]) / 2;
      double P_face_y = (P[B] + P[Tt]) * yn / 2;
      g_v[f] = (rho_v_face * vel_face + P_face_y);
      double rho_E_face = (E[B] + E[Tt]) / 2;
      double P_face = (P[B] + P[Tt]) / 2;
      g_E[f] = ((rho_E_face + P_face) * vel_face);
    }
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi; ++i) {
      int k = d.ci(i, j);
      int fw = d.lri(i, j), fe = d.lri(i + 1, j), fs = d.bti(i, j), fn = d.bti(i, j + 1);
      double aw = m.lr_a[fw], ae = m.lr_a[fe], as = m.bt_a[fs], an = m.bt_a[fn];
      double vol = m.vol[k];
      // FLUX_MASS.jl:28-41
      double fr = -f_m[fe] * ae;
      fr = fr + f_m[fw] * aw;
      fr = fr - g_m[fn] * an;
      fr = fr + g_m[fs] * as;
      s.flux_rho[k] = fr / vol;
      // FLUX_MOMENTUM.jl:79-95
      double fu = -(f_u[fe]) * ae;
      fu = fu + (f_u[fw]) * aw;
      fu = fu - (g_u[fn]) * an;
      fu = fu + (g_u[fs]) * as;
      s.flux_rho_u[k] = fu / vol;
      double fv = -(f_v[fe]) * ae;
      fv = fv + (f_v[fw]) * aw;
      fv = fv - (g_v[fn]) * an;
      fv = fv + (g_v[fs]) * as;
      if (c.axisymmetric) {
        // FLUX_MOMENTUM_3D.jl:120-122
        double pc = P[d.gi(i + 1, j + 1)];
        double front = pc * m.fb_yn_front, back = pc * m.fb_yn_back;
        fv = fv + (front - back) * m.fb_area[k] * jsign(m.y[k]);
      }
      s.flux_rho_v[k] = fv / vol;
      // FLUX_TOTAL_ENERGY.jl:154-171
      double fE = -(f_E[fe]) * ae;
      fE = fE + (f_E[fw]) * aw;
      fE = fE - (g_E[fn]) * an;
      fE = fE + (g_E[fs]) * as;
      s.flux_rho_E[k] = fE / vol;
    }
}

// utils/Operators/VISCOUS_FLUX.jl:36-210 and VISCOUS_FLUX_3D.jl:36-231.
void viscous_flux(const orc_config& c, const Mesh& m, State& s) {
  const Dims d{c.nchi, c.neta};
  const int nchi = c.nchi, neta = c.neta;
  const double Re_infty = c.Re, gamma_star_fs = c.gamma, Pr_fs = c.Pr;
  const int NI = nchi + 2, NJ = neta + 2;
  const int G = NI * NJ;
  const Transport tr{c.viscosity_model, c.sutherland_S, c.energy_factor / c.cv};
  vec u(G), v(G);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < G; ++k) { u[k] = s.rho_u[k] / s.rho[k]; v[k] = s.rho_v[k] / s.rho[k]; }
  // corner values (Nchi+1) x (Neta+1): corner (i, j) averages ghosted cells i..i+1, j..j+1
  const int NC = (nchi + 1) * (neta + 1);
  vec u_c(NC), v_c(NC), T_c(NC);
  const double* T = s.T.data();
  for (int j = 1; j <= neta + 1; ++j)
    for (int i = 1; i <= nchi + 1; ++i) {
      int a = d.gi(i, j), b = d.gi(i + 1, j), cc = d.gi(i, j + 1), dd = d.gi(i + 1, j + 1);
      int k = d.cni(i, j);
      u_c[k] = (u[a] + u[b] + u[cc] + u[dd]) / 4;
      v_c[k] = (v[a] + v[b] + v[cc] + v[dd]) / 4;
      T_c[k] = (T[a] + T[b] + T[cc] + T[dd]) / 4;
    }
  const double *X = m.x_ext.data(), *Y = m.y_ext.data();
  const double *xc = m.x_corner.data(), *yc = m.y_corner.data();
  // ---- lr faces (index 1): (Nchi+1) x Neta, between ghosted (i, j+1) and (i+1, j+1)
  const int NLR = (nchi + 1) * neta;
  vec tau_1x(NLR), tau_1y(NLR), w1(NLR), q_n1(NLR), tth_1(NLR);
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi + 1; ++i) {
      int f = d.lri(i, j);
      int L = d.gi(i, j + 1), Rr = d.gi(i + 1, j + 1);
      double xn = m.lr_xn[f], yn = m.lr_yn[f];
      double cld = std::sqrt(sq(Y[Rr] - Y[L]) + sq(X[Rr] - X[L]));
      double lr_dist = std::sqrt(sq(xc[d.cni(i, j + 1)] - xc[d.cni(i, j)]) + sq(yc[d.cni(i, j + 1)] - yc[d.cni(i, j)]));
      double c1_x = -(X[Rr] - X[L]) / cld;
      double c1_y = -(Y[Rr] - Y[L]) / cld;
      double Cn1_Fn1 = -c1_x * xn - c1_y * yn;
      double Cn1_Ft1 = c1_x * yn - c1_y * xn;
      double du_dc1 = -(u[Rr] - u[L]) / cld;
      double dv_dc1 = -(v[Rr] - v[L]) / cld;
      double du_dt1 = (u_c[d.cni(i, j + 1)] - u_c[d.cni(i, j)]) / lr_dist;
      double dv_dt1 = (v_c[d.cni(i, j + 1)] - v_c[d.cni(i, j)]) / lr_dist;
      double divide1 = Cn1_Fn1;
      double du_dn1 = (du_dc1 - du_dt1 * Cn1_Ft1) / divide1;
      double dv_dn1 = (dv_dc1 - dv_dt1 * Cn1_Ft1) / divide1;
      double dun_dn1 = -du_dn1 * xn - dv_dn1 * yn;
      double dut_dn1 = du_dn1 * yn - dv_dn1 * xn;
      double dun_dt1 = -du_dt1 * xn - dv_dt1 * yn;
      double dut_dt1 = du_dt1 * yn - dv_dt1 * xn;
      double mu_1 = tr.face(T[L], T[Rr]);
      double div_1 = dut_dt1 + dun_dn1;
      double u_face_1 = 0, x_face_1 = 1;
      if (c.axisymmetric) {
        x_face_1 = (X[Rr] + X[L]) / 2;
        u_face_1 = (u[Rr] + u[L]) / 2;
        div_1 = dut_dt1 + dun_dn1 + u_face_1 / x_face_1;
      }
      double tau_11 = mu_1 / Re_infty * (2 * dun_dn1 - (2.0 / 3) * div_1);
      double tau_12 = mu_1 / Re_infty * (dun_dt1 + dut_dn1);
      if (c.axisymmetric) tth_1[f] = mu_1 / Re_infty * (2 * u_face_1 / x_face_1 - (2.0 / 3) * div_1);
      tau_1x[f] = -(tau_11 * xn - tau_12 * yn);
      tau_1y[f] = -(tau_11 * yn + tau_12 * xn);
      double inv_rho_1 = 1 / (s.rho[L] + s.rho[Rr]);
      double u_1 = (s.rho_u[L] + s.rho_u[Rr]) * inv_rho_1;
      double v_1 = (s.rho_v[L] + s.rho_v[Rr]) * inv_rho_1;
      w1[f] = u_1 * tau_1x[f] + v_1 * tau_1y[f];
      double k_lr = tr.face(T[L], T[Rr]) * gamma_star_fs / Re_infty / Pr_fs;
      double dT_dc1 = -(T[Rr] - T[L]) / cld;
      double dT_dt1 = (T_c[d.cni(i, j + 1)] - T_c[d.cni(i, j)]) / lr_dist;
      double dT_dn1 = (dT_dc1 - dT_dt1 * Cn1_Ft1) / divide1;
      q_n1[f] = k_lr * dT_dn1;
    }
  // ---- bt faces (index 2): Nchi x (Neta+1), between ghosted (i+1, j) and (i+1, j+1)
  const int NBT = nchi * (neta + 1);
  vec tau_2x(NBT), tau_2y(NBT), w2(NBT), q_n2(NBT), tth_2(NBT);
  for (int j = 1; j <= neta + 1; ++j)
    for (int i = 1; i <= nchi; ++i) {
      int f = d.bti(i, j);
      int B = d.gi(i + 1, j), Tt = d.gi(i + 1, j + 1);
      double xn = m.bt_xn[f], yn = m.bt_yn[f];
      double cbd = std::sqrt(sq(Y[Tt] - Y[B]) + sq(X[Tt] - X[B]));
      double bt_dist = std::sqrt(sq(xc[d.cni(i + 1, j)] - xc[d.cni(i, j)]) + sq(yc[d.cni(i + 1, j)] - yc[d.cni(i, j)]));
      double c2_x = (X[Tt] - X[B]) / cbd;
      double c2_y = (Y[Tt] - Y[B]) / cbd;
      double Cn2_Fn2 = c2_x * xn + c2_y * yn;
      double Cn2_Ft2 = c2_x * yn - c2_y * xn;
      double du_dc2 = (u[Tt] - u[B]) / cbd;
      double dv_dc2 = (v[Tt] - v[B]) / cbd;
      double du_dt2 = -(u_c[d.cni(i + 1, j)] - u_c[d.cni(i, j)]) / bt_dist;
      double dv_dt2 = -(v_c[d.cni(i + 1, j)] - v_c[d.cni(i, j)]) / bt_dist;
      double divide = -Cn2_Fn2;
      double du_dn2 = (Cn2_Ft2 * du_dt2 - du_dc2) / divide;
      double dv_dn2 = (Cn2_Ft2 * dv_dt2 - dv_dc2) / divide;
      double dut_dt2 = du_dt2 * yn - dv_dt2 * xn;
      double dun_dt2 = du_dt2 * xn + dv_dt2 * yn;
      double dut_dn2 = du_dn2 * yn - dv_dn2 * xn;
      double dun_dn2 = du_dn2 * xn + dv_dn2 * yn;
      double mu_2 = tr.face(T[B], T[Tt]);
      double div_2 = dut_dt2 + dun_dn2;
      double u_face_2 = 0, x_face_2 = 1;
      if (c.axisymmetric) {
        x_face_2 = (X[Tt] + X[B]) / 2;
        u_face_2 = (u[Tt] + u[B]) / 2;
        div_2 = dut_dt2 + dun_dn2 + u_face_2 / x_face_2;
      }
      double tau_22 = mu_2 / Re_infty * (2 * dun_dn2 - (2.0 / 3) * div_2);
      double tau_21 = mu_2 / Re_infty * (dut_dn2 + dun_dt2);
      if (c.axisymmetric) tth_2[f] = mu_2 / Re_infty * (2 * u_face_2 / x_face_2 - (2.0 / 3) * div_2);
      tau_2x[f] = (tau_22 * xn + tau_21 * yn);
      tau_2y[f] = (tau_22 * yn - tau_21 * xn);
      double inv_rho_2 = 1 / (s.rho[B] + s.rho[Tt]);
      double u_2 = (s.rho_u[B] + s.rho_u[Tt]) * inv_rho_2;
      double v_2 = (s.rho_v[B] + s.rho_v[Tt]) * inv_rho_2;
      w2[f] = u_2 * tau_2x[f] + v_2 * tau_2y[f];
      double k_bt = tr.face(T[B], T[Tt]) * gamma_star_fs / Re_infty / Pr_fs;
      double dT_dc2 = (T[Tt] - T[B]) / cbd;
      double dT_dt2 = -(T_c[d.cni(i + 1, j)] - T_c[d.cni(i, j)]) / bt_dist;
      double dT_dn2 = (Cn2_Ft2 * dT_dt2 - dT_dc2) / divide;
      q_n2[f] = k_bt * dT_dn2;
    }
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi; ++i) {
      int k = d.ci(i, j);
      int fw = d.lri(i, j), fe = d.lri(i + 1, j), fs = d.bti(i, j), fn = d.bti(i, j + 1);
      double aw = m.lr_a[fw], ae = m.lr_a[fe], as = m.bt_a[fs], an = m.bt_a[fn];
      double vol = m.vol[k];
      double rho_u_temp = (tau_1x[fw] * aw - tau_1x[fe] * ae) + (tau_2x[fn] * an - tau_2x[fs] * as);
      s.flux_rho_u[k] += rho_u_temp / vol;
      if (c.axisymmetric) {
        // VISCOUS_FLUX_3D.jl:154-177: hoop stress averaged to the cell, radius = x
        double tth = (tth_1[fw] + tth_1[fe] + tth_2[fs] + tth_2[fn]) / 4;
        double x_cell = X[d.gi(i + 1, j + 1)];
        s.flux_rho_u[k] -= tth / x_cell;
      }
      double rho_v_temp = (tau_1y[fw] * aw - tau_1y[fe] * ae) + (tau_2y[fn] * an - tau_2y[fs] * as);
      s.flux_rho_v[k] += rho_v_temp / vol;
      double rho_E_temp = (w1[fw] * aw - w1[fe] * ae) + (w2[fn] * an - w2[fs] * as);
      s.flux_rho_E[k] += rho_E_temp / vol;
      double rho_E_temp2 = (q_n2[fn] * an - q_n2[fs] * as) - (q_n1[fe] * ae - q_n1[fw] * aw);
      s.flux_rho_E[k] += rho_E_temp2 / vol;
    }
}

// utils/Operators/PDE.jl:1-47 + NON_LINEAR_DYNAMICS_NO_DISCONTINUITY.jl:1-28.
void non_linear_dynamics(const orc_config& c, const Mesh& m, State& s) {
  update_thermo(c, s);
  update_sound_speed(c, s);
  if (c.shock_enabled) update_shock_bc(c, m, s);
  apply_boundary_conditions(c, m, s);
  inviscid_fluxes(c, m, s);
  viscous_flux(c, m, s);
  if (c.shock_enabled && c.shock_feedback) {
    const size_t N = (size_t)c.nchi * c.neta;
    for (size_t k = 0; k < N; ++k) {
      s.flux_rho[k] *= s.flow[k];
      s.flux_rho_u[k] *= s.flow[k];
      s.flux_rho_v[k] *= s.flow[k];
      s.flux_rho_E[k] *= s.flow[k];
    }
  }
}

// utils/Time_marching/CFL_TIMESTEP.jl:41-138.
double cfl_timestep(const orc_config& c, const Mesh& m, const State& s) {
  const Dims d{c.nchi, c.neta};
  const int nchi = c.nchi, neta = c.neta;
  const int G = (nchi + 2) * (neta + 2);
  double cmax = 0;
  for (int k = 0; k < G; ++k) cmax = std::max(cmax, std::fabs(s.a[k]));
  const double *R = s.rho.data(), *U = s.rho_u.data(), *V = s.rho_v.data();
  auto lam_lr = [&](int i, int j) {  // lr face (i, j)
    int L = d.gi(i, j + 1), Rr = d.gi(i + 1, j + 1), f = d.lri(i, j);
    double rho_sum = R[L] + R[Rr];
    double uf = (U[L] + U[Rr]) / rho_sum, vf = (V[L] + V[Rr]) / rho_sum;
    double Vn = std::fabs(uf * m.lr_xn[f] + vf * m.lr_yn[f]);
    return (Vn + cmax) * m.lr_a[f];
  };
  auto lam_bt = [&](int i, int j) {
    int B = d.gi(i + 1, j), Tt = d.gi(i + 1, j + 1), f = d.bti(i, j);
    double rho_sum = R[B] + R[Tt];
    double uf = (U[B] + U[Tt]) / rho_sum, vf = (V[B] + V[Tt]) / rho_sum;
    double Vn = std::fabs(uf * m.bt_xn[f] + vf * m.bt_yn[f]);
    return (Vn + cmax) * m.bt_a[f];
  };
  double max_lam = -std::numeric_limits<double>::infinity();
  double max_u = -std::numeric_limits<double>::infinity(), max_rho = max_u, max_E = max_u;
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi; ++i) {
      int k = d.ci(i, j), g = d.gi(i + 1, j + 1);
      double lam_xi = std::max(lam_lr(i, j), lam_lr(i + 1, j));
      double lam_eta = std::max(lam_bt(i, j), lam_bt(i, j + 1));
      double lam_c = lam_xi + lam_eta;
      double A_xi = 0.5 * (m.lr_a[d.lri(i, j)] + m.lr_a[d.lri(i + 1, j)]);
      double A_eta = 0.5 * (m.bt_a[d.bti(i, j)] + m.bt_a[d.bti(i, j + 1)]);
      // Re_flow = Re / mu* (UPDATE_CHEMISTRY_EQUILIBRIUM.jl:99-101); mu* = 1 for CPG
      double Re_flow = c.Re;
      if (c.viscosity_model == 1) {
        double e = (s.rho_E[g] - (s.rho_u[g] * s.rho_u[g] + s.rho_v[g] * s.rho_v[g]) / R[g] / 2) / R[g];
        double Ts = e / (c.cv / c.energy_factor);
        Re_flow = c.Re / (Ts * std::sqrt(Ts) * (1 + c.sutherland_S) / (Ts + c.sutherland_S));
      }
      double nu_eff = std::max(4.0 / 3.0, c.gamma / c.Pr) / (R[g] * Re_flow);
      double lam_v = 2 * nu_eff * (A_xi * A_xi + A_eta * A_eta) / m.vol[k];
      double flowk = c.shock_enabled ? s.flow[k] : 1.0;
      double lov = (lam_c + lam_v) * flowk / m.vol[k];
      max_lam = std::max(max_lam, lov);
      double mu_ = (std::fabs(s.flux_rho_v[k]) + std::fabs(s.flux_rho_u[k])) / R[g];
      double mr = std::fabs(s.flux_rho[k] / R[g]);
      double mE = std::fabs(s.flux_rho_E[k] / s.rho_E[g]);
      if (c.shock_enabled) { mu_ = mu_ * flowk; mr = std::fabs(s.flux_rho[k] / R[g] * flowk); mE = std::fabs(s.flux_rho_E[k] / s.rho_E[g] * flowk); }
      max_u = std::max(max_u, mu_);
      max_rho = std::max(max_rho, mr);
      max_E = std::max(max_E, mE);
    }
  double dt1 = c.CFL / max_lam;
  double dt2 = c.CFL / std::max(max_u, std::max(max_rho, max_E));
  return std::min(dt1, std::min(dt2, c.max_dt));
}

// utils/Time_marching/INTEGRATION.jl:36-90 (interior update, masked when shock
// fitting is on, then MOVE_SHOCK).
void integration(const orc_config& c, State& s, const State& ds, double w) {
  const Dims d{c.nchi, c.neta};
  for (int j = 1; j <= c.neta; ++j)
    for (int i = 1; i <= c.nchi; ++i) {
      int k = d.ci(i, j), g = d.gi(i + 1, j + 1);
      if (c.shock_enabled) {
        double f = s.flow[k];
        s.rho[g] = s.rho[g] + w * ds.flux_rho[k] * f;
        s.rho_u[g] = s.rho_u[g] + w * ds.flux_rho_u[k] * f;
        s.rho_v[g] = s.rho_v[g] + w * ds.flux_rho_v[k] * f;
        s.rho_E[g] = s.rho_E[g] + w * ds.flux_rho_E[k] * f;
      } else {
        s.rho[g] = s.rho[g] + w * ds.flux_rho[k];
        s.rho_u[g] = s.rho_u[g] + w * ds.flux_rho_u[k];
        s.rho_v[g] = s.rho_v[g] + w * ds.flux_rho_v[k];
        s.rho_E[g] = s.rho_E[g] + w * ds.flux_rho_E[k];
      }
    }
  if (c.shock_enabled) move_shock(c, s, ds, w);
}

// utils/Time_marching/ADVECT_FLOW_EXPLICIT.jl:36-81. rk_variant 0 reproduces the
// Julia path, where `INTEGRATION(solution_0, temp, ·)` mutates solution_0 in place
// so each stage input accumulates the previous stage (Y3 = Y2 + dt/2 k2,
// Y4 = Y3 + dt k3). rk_variant 1 is classical RK4 (the MATLAB twin's value
// semantics): every stage input is y_n + c_k dt k_{k-1}.
void advect_flow_explicit(const orc_config& c, const Mesh& m, State& s) {
  update_flow_cells(c, m, s);
  double dt = cfl_timestep(c, m, s);
  s.dt = dt;
  if (c.rk_variant == 0) {
    State sol0 = s;
    non_linear_dynamics(c, m, sol0);
    integration(c, s, sol0, dt / 6);
    integration(c, sol0, sol0, dt / 2);
    non_linear_dynamics(c, m, sol0);
    integration(c, s, sol0, dt / 3);
    integration(c, sol0, sol0, dt / 2);
    non_linear_dynamics(c, m, sol0);
    integration(c, s, sol0, dt / 3);
    integration(c, sol0, sol0, dt);
    non_linear_dynamics(c, m, sol0);
    integration(c, s, sol0, dt / 6);
  } else {
    const State y0 = s;
    State Y = y0;
    non_linear_dynamics(c, m, Y);
    integration(c, s, Y, dt / 6);
    const double cw[3] = {dt / 2, dt / 2, dt};
    const double aw[3] = {dt / 3, dt / 3, dt / 6};
    for (int st = 0; st < 3; ++st) {
      State Z = y0;
      integration(c, Z, Y, cw[st]);
      Y = Z;
      non_linear_dynamics(c, m, Y);
      integration(c, s, Y, aw[st]);
    }
  }
  update_thermo(c, s);
  if (c.shock_enabled) update_shock_bc(c, m, s);
  apply_boundary_conditions(c, m, s);
  if (c.shock_enabled) update_field_upstream(c, m, s);
  min_rho(c, s);
  s.t = s.t + s.dt;
}

// ---------------------------------------------------------------------------
// Stencil-block Jacobian. Storage (shared with the GPU path): for output cell m
// (chi-fastest index), neighbour slot q = (b+1)*3 + (a+1) for the input cell at
// offset (a, b) in (chi, eta), block entry [vout][vin]:
//   coef[((m * 9 + q) * 4 + vout) * 4 + vin] = L[(m, vout), (n = m + (a, b), vin)].
// The reference assembles exactly these entries (GET_OUTPUT_INDEXING_A11,
// LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:306-788): each input cell n gets its
// 3x3 neighbourhood of outputs, with wrap-around in chi (eta) when both chi (eta)
// boundaries are periodic.

// utils/Stability_analysis/Modal_stability_analysis/LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:42-288
// (A11 block; perturb_shock = false).
void linearize_equations(const orc_config& c, const Mesh& m, const State& s, double* coef) {
  const int nchi = c.nchi, neta = c.neta;
  const Dims d{nchi, neta};
  const size_t N = (size_t)nchi * neta;
  std::memset(coef, 0, sizeof(double) * N * 144);
  State base = s;
  non_linear_dynamics(c, m, base);
  const double eps = c.perturbation_magnitude;
  const bool per_chi = c.bc_chi0 == ORC_BC_PERIODIC && c.bc_chi1 == ORC_BC_PERIODIC;
  const bool per_eta = c.bc_eta0 == ORC_BC_PERIODIC && c.bc_eta1 == ORC_BC_PERIODIC;
  for (int var = 0; var < 4; ++var) {
    for (int index = 1; index <= 9; ++index) {
      // GET_PERTURBATION_MATRIX (:959-983)
      int start_i = (index % 3 == 0) ? 3 : index % 3;
      int start_j = (index + 2) / 3;
      State sp = s;
      vec* tgt = var == 0 ? &sp.rho : var == 1 ? &sp.rho_u : var == 2 ? &sp.rho_v : &sp.rho_E;
      const vec& src = var == 0 ? s.rho : var == 1 ? s.rho_u : var == 2 ? s.rho_v : s.rho_E;
      for (int j = 1; j <= neta; ++j)
        for (int i = 1; i <= nchi; ++i) {
          double pert = ((i - start_i) % 3 == 0 && i >= start_i && (j - start_j) % 3 == 0 && j >= start_j) ? 1.0 : 0.0;
          int g = d.gi(i + 1, j + 1);
          if (c.shock_enabled)
            (*tgt)[g] = src[g] + s.flow[d.ci(i, j)] * pert * eps;
          else
            (*tgt)[g] = src[g] + pert * eps;
        }
      non_linear_dynamics(c, m, sp);
      // REMOVE_BASE_OUTPUT (:935-946)
      const vec* fp[4] = {&sp.flux_rho, &sp.flux_rho_u, &sp.flux_rho_v, &sp.flux_rho_E};
      const vec* fb[4] = {&base.flux_rho, &base.flux_rho_u, &base.flux_rho_v, &base.flux_rho_E};
      for (int jn = start_j; jn <= neta; jn += 3)
        for (int in = start_i; in <= nchi; in += 3) {
          for (int b = -1; b <= 1; ++b)
            for (int a = -1; a <= 1; ++a) {
              int io = in + a, jo = jn + b;
              bool wi = io < 1 || io > nchi, wj = jo < 1 || jo > neta;
              // the reference wraps one direction at a time; a doubly wrapped corner is never set
              if ((wi && !per_chi) || (wj && !per_eta) || (wi && wj)) continue;
              if (wi) io = io < 1 ? io + nchi : io - nchi;
              if (wj) jo = jo < 1 ? jo + neta : jo - neta;
              int mo = d.ci(io, jo);
              // input offset seen from the output cell: n = m + (-a, -b)
              int q = (-b + 1) * 3 + (-a + 1);
              for (int vo = 0; vo < 4; ++vo) {
                double val = ((*fp[vo])[mo] - (*fb[vo])[mo]) / eps;
                coef[(((size_t)mo * 9 + q) * 4 + vo) * 4 + var] = val;
              }
            }
        }
    }
  }
}

// utils/Stability_analysis/Modal_stability_analysis/LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-274
// (perturb_shock = true), on the prepared state s (its beta from the last UPDATE_SHOCK_BC).
//   rows[i] = sc_i (shock["cell_indices"]).
//   a21_full: the reference's A21 columns as assembled. Per-point strategy when
//     spline_param != 1 (:143-205): one residual per cell (i, sc_i - j), j = 1, 2, per
//     variable; its column holds the change of every point's speed,
//     a21_full[((v * 2 + j - 1) * Nchi + i) * Nchi + idx] (GET_OUTPUT_INDEXING_A21, :800-820).
//     All-at-once strategy otherwise (:207-258): one residual per (v, j) raising the cell
//     (i, sc_i - j) of every column; only the entries idx = i are assembled
//     (GET_OUTPUT_INDEXING_A21_ALL, :829-850).
//   a12[(v * Nchi + i) * Nchi + p], a22[i * Nchi + p]: one residual per shock point p moved by
//     PERTURB_SHOCK (:906-913); the flux of cell (i, sc_i - 1) and every point's speed
//     (GET_OUTPUT_INDEXING_A12_A22, :854-903).
// Every difference is REMOVE_BASE_OUTPUT's (f(x + eps e) - f(x)) / eps (:935-946).
void linearize_shock_blocks(const orc_config& c, const Mesh& m, const State& s, int* rows, double* a21_full,
                            double* a12, double* a22) {
  const int nchi = c.nchi;
  const Dims d{nchi, c.neta};
  const double eps = c.perturbation_magnitude;
  State base = s;
  non_linear_dynamics(c, m, base);
  for (int i = 0; i < nchi; ++i) rows[i] = s.cell_idx[i];
  std::memset(a21_full, 0, sizeof(double) * 8 * (size_t)nchi * nchi);
  auto var_of = [](State& st, int v) -> vec& {
    return v == 0 ? st.rho : v == 1 ? st.rho_u : v == 2 ? st.rho_v : st.rho_E;
  };
  auto speed_diff = [&](const State& sp, int idx) { return (sp.rel_vel[idx] - base.rel_vel[idx]) / eps; };
  for (int v = 0; v < 4; ++v)
    for (int j = 1; j <= 2; ++j) {
      if (c.spline_param != 1) {
        for (int i = 1; i <= nchi; ++i) {
          State sp = s;
          var_of(sp, v)[d.gi(i + 1, s.cell_idx[i - 1] - j + 1)] += eps;
          non_linear_dynamics(c, m, sp);
          double* col = a21_full + ((size_t)(v * 2 + j - 1) * nchi + (i - 1)) * nchi;
          for (int idx = 0; idx < nchi; ++idx) col[idx] = speed_diff(sp, idx);
        }
      } else {
        State sp = s;
        for (int i = 1; i <= nchi; ++i) var_of(sp, v)[d.gi(i + 1, s.cell_idx[i - 1] - j + 1)] += eps;
        non_linear_dynamics(c, m, sp);
        for (int idx = 0; idx < nchi; ++idx)
          a21_full[((size_t)(v * 2 + j - 1) * nchi + idx) * nchi + idx] = speed_diff(sp, idx);
      }
    }
  const double phi = std::atan2(c.rho_v_0, c.rho_u_0);
  for (int p = 0; p < nchi; ++p) {
    State sp = s;
    const double ang = s.beta[p] - M_PI / 2 - phi;
    sp.pts_x[p] += eps * std::cos(ang);
    sp.pts_y[p] += eps * std::sin(ang);
    non_linear_dynamics(c, m, sp);
    const vec* fp[4] = {&sp.flux_rho, &sp.flux_rho_u, &sp.flux_rho_v, &sp.flux_rho_E};
    const vec* fb[4] = {&base.flux_rho, &base.flux_rho_u, &base.flux_rho_v, &base.flux_rho_E};
    for (int i = 1; i <= nchi; ++i) {
      const int k = d.ci(i, s.cell_idx[i - 1] - 1);
      for (int v = 0; v < 4; ++v)
        a12[((size_t)v * nchi + (i - 1)) * nchi + p] = ((*fp[v])[k] - (*fb[v])[k]) / eps;
      a22[(size_t)(i - 1) * nchi + p] = speed_diff(sp, i - 1);
    }
  }
}

// utils/Stability_analysis/Freestream_receptivity/LINEARIZE_B.jl:40-296: the response of the
// residual to the per-column upstream state, column-wise finite differences with 3 colours
// (LINEARIZE_B.jl:49-170) and GET_BLOCK's left / middle / right neighbours (:186-253).
// rows[m] = sc_m; bq[((m*3 + d+1)*4 + vout)*4 + vin] and bs[(m*3 + d+1)*4 + vin] for the
// input column n = m + d (0-based), as include/hymor.h documents for hymor_b_get.
void linearize_b(const orc_config& c, const Mesh& m, const State& s0, int* rows, double* bq, double* bs) {
  const int nchi = c.nchi;
  const Dims d{nchi, c.neta};
  const double eps = c.perturbation_magnitude;
  State s = s0;
  s.up_cols.assign(4 * (size_t)nchi, 0.0);
  const double fs[4] = {c.rho_0, c.rho_u_0, c.rho_v_0, c.rho_E_0};
  for (int v = 0; v < 4; ++v)
    for (int i = 0; i < nchi; ++i) s.up_cols[(size_t)v * nchi + i] = fs[v];
  orc_config cz = c;  // the disturbance amplitude is set to zero (:45)
  for (int v = 0; v < 4; ++v) cz.dist_amp[v] = 0;
  State base = s;
  non_linear_dynamics(cz, m, base);
  for (int i = 0; i < nchi; ++i) rows[i] = s.cell_idx[i];
  std::memset(bq, 0, sizeof(double) * 48 * nchi);
  std::memset(bs, 0, sizeof(double) * 12 * nchi);
  for (int var = 0; var < 4; ++var)
    for (int iter = 1; iter <= 3; ++iter) {
      State sp = s;
      for (int i = iter; i <= nchi; i += 3) sp.up_cols[(size_t)var * nchi + i - 1] += eps * 1.0;
      non_linear_dynamics(cz, m, sp);
      // GET_BLOCK's (output column pert_m, input column pert_n) pairs, 1-based
      auto block = [&](const std::vector<int>& pm, const std::vector<int>& pn) {
        for (size_t k = 0; k < pm.size(); ++k) {
          const int mo = pm[k] - 1, ni = pn[k] - 1, dd = ni - mo;
          const int cell = d.ci(pm[k], s.cell_idx[mo] - 1);
          const vec* fp[4] = {&sp.flux_rho, &sp.flux_rho_u, &sp.flux_rho_v, &sp.flux_rho_E};
          const vec* fb[4] = {&base.flux_rho, &base.flux_rho_u, &base.flux_rho_v, &base.flux_rho_E};
          for (int vo = 0; vo < 4; ++vo)
            bq[((mo * 3 + dd + 1) * 4 + vo) * 4 + var] = ((*fp[vo])[cell] - (*fb[vo])[cell]) / eps;
          bs[(mo * 3 + dd + 1) * 4 + var] = (sp.rel_vel[mo] - base.rel_vel[mo]) / eps;
        }
      };
      std::vector<int> pm, pn;
      for (int x = (iter == 1 ? iter + 2 : iter - 1); x <= nchi - 1; x += 3) { pm.push_back(x); pn.push_back(x + 1); }
      block(pm, pn);
      pm.clear(); pn.clear();
      for (int x = iter; x <= nchi; x += 3) { pm.push_back(x); pn.push_back(x); }
      block(pm, pn);
      pm.clear(); pn.clear();
      for (int x = iter + 1; x <= nchi; x += 3) { pm.push_back(x); pn.push_back(x - 1); }
      block(pm, pn);
    }
}

// The shock-block part of y = A x on vectors [q (4N); r (Nchi)], after stencil_matvec has
// written y's first 4N entries; a21 compact (Nchi x 8, entry (j - 1) * 4 + v).
void shock_matvec(const orc_config& c, const int* rows, const double* a21, const double* a12, const double* a22,
                  const double* x, double* y, int transpose) {
  const int nchi = c.nchi;
  const size_t N = (size_t)nchi * c.neta;
  const double* xr = x + 4 * N;
  double* yr = y + 4 * N;
  auto cell = [&](int i, int row1) { return (size_t)i + (size_t)(row1 - 1) * nchi; };  // 0-based i, 1-based row
  if (!transpose) {
    for (int i = 0; i < nchi; ++i) {
      for (int v = 0; v < 4; ++v) {
        double acc = 0;
        for (int p = 0; p < nchi; ++p) acc += a12[((size_t)v * nchi + i) * nchi + p] * xr[p];
        y[v * N + cell(i, rows[i] - 1)] += acc;
      }
      double acc = 0;
      for (int j = 1; j <= 2; ++j)
        for (int v = 0; v < 4; ++v) acc += a21[i * 8 + (j - 1) * 4 + v] * x[v * N + cell(i, rows[i] - j)];
      for (int p = 0; p < nchi; ++p) acc += a22[(size_t)i * nchi + p] * xr[p];
      yr[i] = acc;
    }
  } else {
    for (int p = 0; p < nchi; ++p) {
      double acc = 0;
      for (int v = 0; v < 4; ++v)
        for (int i = 0; i < nchi; ++i) acc += a12[((size_t)v * nchi + i) * nchi + p] * x[v * N + cell(i, rows[i] - 1)];
      for (int i = 0; i < nchi; ++i) acc += a22[(size_t)i * nchi + p] * xr[i];
      yr[p] = acc;
    }
    for (int i = 0; i < nchi; ++i)
      for (int j = 1; j <= 2; ++j)
        for (int v = 0; v < 4; ++v) y[v * N + cell(i, rows[i] - j)] += a21[i * 8 + (j - 1) * 4 + v] * xr[i];
  }
}

// y = L x (transpose = 0) or y = Lᵀ x (transpose = 1) with the stencil blocks;
// vectors ordered [rho; rho_u; rho_v; rho_E], each Nchi*Neta chi-fastest
// (CHECK_LINEARIZATION_L.jl:52).
void stencil_matvec(const orc_config& c, const double* coef, const double* x, double* y, int transpose) {
  const int nchi = c.nchi, neta = c.neta;
  const size_t N = (size_t)nchi * neta;
  const bool per_chi = c.bc_chi0 == ORC_BC_PERIODIC && c.bc_chi1 == ORC_BC_PERIODIC;
  const bool per_eta = c.bc_eta0 == ORC_BC_PERIODIC && c.bc_eta1 == ORC_BC_PERIODIC;
  // Each output entry is summed by the one thread that owns its cell. Forward: output
  // cell m sums its 9 neighbour blocks (b, a ascending). Transpose: output cell n sums the
  // blocks of the cells m = n - (a, b) whose stencil reaches n (b, a descending, the order
  // in which a scatter over m ascending would add them).
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi; ++i) {
      const size_t me = (size_t)(i - 1) + (size_t)(j - 1) * nchi;
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      for (int bb = 0; bb < 3; ++bb)
        for (int aa = 0; aa < 3; ++aa) {
          const int b = transpose ? 1 - bb : bb - 1;
          const int a = transpose ? 1 - aa : aa - 1;
          // forward: the neighbour (i + a, j + b); transpose: the cell (i - a, j - b)
          int in = transpose ? i - a : i + a, jn = transpose ? j - b : j + b;
          bool wi = in < 1 || in > nchi, wj = jn < 1 || jn > neta;
          if ((wi && !per_chi) || (wj && !per_eta) || (wi && wj)) continue;
          if (wi) in = in < 1 ? in + nchi : in - nchi;
          if (wj) jn = jn < 1 ? jn + neta : jn - neta;
          const size_t other = (size_t)(in - 1) + (size_t)(jn - 1) * nchi;
          const int q = (b + 1) * 3 + (a + 1);
          if (!transpose) {
            const double* B = coef + (me * 9 + q) * 16;
            for (int vo = 0; vo < 4; ++vo)
              for (int vi = 0; vi < 4; ++vi) acc[vo] += B[vo * 4 + vi] * x[vi * N + other];
          } else {
            const double* B = coef + (other * 9 + q) * 16;
            for (int vo = 0; vo < 4; ++vo)
              for (int vi = 0; vi < 4; ++vi) acc[vi] += B[vo * 4 + vi] * x[vo * N + other];
          }
        }
      for (int v = 0; v < 4; ++v) y[v * N + me] = acc[v];
    }
}

}  // namespace

// ===========================================================================
// C API (ctypes).

extern "C" {

typedef struct Ctx orc_ctx;

orc_ctx* orc_create(const orc_config* cfg, const orc_mesh* mesh) {
  Ctx* c = new Ctx();
  c->c = *cfg;
  Mesh& m = c->m;
  const int nchi = cfg->nchi, neta = cfg->neta;
  m.nchi = nchi;
  m.neta = neta;
  auto cp = [](const double* p, size_t n) { return p ? vec(p, p + n) : vec(n, 0.0); };
  const size_t NLR = (size_t)(nchi + 1) * neta, NBT = (size_t)nchi * (neta + 1), N = (size_t)nchi * neta,
               G = (size_t)(nchi + 2) * (neta + 2), NC = (size_t)(nchi + 1) * (neta + 1);
  m.lr_xn = cp(mesh->lr_xn, NLR);
  m.lr_yn = cp(mesh->lr_yn, NLR);
  m.lr_a = cp(mesh->lr_a, NLR);
  m.bt_xn = cp(mesh->bt_xn, NBT);
  m.bt_yn = cp(mesh->bt_yn, NBT);
  m.bt_a = cp(mesh->bt_a, NBT);
  m.vol = cp(mesh->vol, N);
  m.x_ext = cp(mesh->x_ext, G);
  m.y_ext = cp(mesh->y_ext, G);
  m.x_corner = cp(mesh->x_corner, NC);
  m.y_corner = cp(mesh->y_corner, NC);
  m.chi1 = cp(mesh->chi1, nchi);
  m.fb_area = cp(mesh->fb_area, N);
  m.fb_yn_front = mesh->fb_yn_front;
  m.fb_yn_back = mesh->fb_yn_back;
  m.x.resize(N);
  m.y.resize(N);
  const Dims d{nchi, neta};
  for (int j = 1; j <= neta; ++j)
    for (int i = 1; i <= nchi; ++i) {
      m.x[d.ci(i, j)] = m.x_ext[d.gi(i + 1, j + 1)];
      m.y[d.ci(i, j)] = m.y_ext[d.gi(i + 1, j + 1)];
    }
  State& s = c->s;
  s.rho.assign(G, 0.0);
  s.rho_u.assign(G, 0.0);
  s.rho_v.assign(G, 0.0);
  s.rho_E.assign(G, 0.0);
  s.p.assign(G, 0.0);
  s.T.assign(G, 0.0);
  s.a.assign(G, 0.0);
  s.pts_x.assign(nchi, 0.0);
  s.pts_y.assign(nchi, 0.0);
  s.pts_chi.assign(nchi, 0.0);
  s.pts_eta.assign(nchi, 0.0);
  s.cell_idx.assign(nchi, 1);
  s.flow.assign(N, 1.0);
  s.beta.assign(nchi, 0.0);
  s.speed_x.assign(nchi, 0.0);
  s.speed_y.assign(nchi, 0.0);
  s.rel_vel.assign(nchi, 0.0);
  s.flux_rho.assign(N, 0.0);
  s.flux_rho_u.assign(N, 0.0);
  s.flux_rho_v.assign(N, 0.0);
  s.flux_rho_E.assign(N, 0.0);
#ifdef _OPENMP
  c->nthreads = omp_get_max_threads();
#endif
  return c;
}

void orc_destroy(orc_ctx* c) { delete c; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// q: 4 ghosted arrays back to back [rho, rho_u, rho_v, rho_E]; shock arrays Nchi;
// cell_idx 1-based (flow cells follow from it: flow[i, j] = j < cell_idx[i]).
void orc_set_state(orc_ctx* c, const double* q, const double* pts_x, const double* pts_y,
                   const double* pts_chi, const double* pts_eta, const int32_t* cell_idx, double t,
                   const double* a_ghosted) {
  State& s = c->s;
  const int nchi = c->c.nchi, neta = c->c.neta;
  const size_t G = (size_t)(nchi + 2) * (neta + 2);
  std::memcpy(s.rho.data(), q, G * 8);
  std::memcpy(s.rho_u.data(), q + G, G * 8);
  std::memcpy(s.rho_v.data(), q + 2 * G, G * 8);
  std::memcpy(s.rho_E.data(), q + 3 * G, G * 8);
  if (pts_x) std::memcpy(s.pts_x.data(), pts_x, nchi * 8);
  if (pts_y) std::memcpy(s.pts_y.data(), pts_y, nchi * 8);
  if (pts_chi) std::memcpy(s.pts_chi.data(), pts_chi, nchi * 8);
  if (pts_eta) std::memcpy(s.pts_eta.data(), pts_eta, nchi * 8);
  const Dims d{nchi, neta};
  for (int i = 1; i <= nchi; ++i) {
    int sc = cell_idx ? cell_idx[i - 1] : neta + 1;
    s.cell_idx[i - 1] = sc;
    for (int j = 1; j <= neta; ++j) s.flow[d.ci(i, j)] = (c->c.shock_enabled && j >= sc) ? 0.0 : 1.0;
  }
  if (a_ghosted) {
    std::memcpy(s.a.data(), a_ghosted, G * 8);
  } else {
    update_thermo(c->c, s);
    update_sound_speed(c->c, s);
  }
  s.t = t;
}

void orc_get_state(orc_ctx* c, double* q, double* pts_x, double* pts_y, double* pts_chi,
                   double* pts_eta, int32_t* cell_idx, double* t, double* dt) {
  State& s = c->s;
  const int nchi = c->c.nchi, neta = c->c.neta;
  const size_t G = (size_t)(nchi + 2) * (neta + 2);
  if (q) {
    std::memcpy(q, s.rho.data(), G * 8);
    std::memcpy(q + G, s.rho_u.data(), G * 8);
    std::memcpy(q + 2 * G, s.rho_v.data(), G * 8);
    std::memcpy(q + 3 * G, s.rho_E.data(), G * 8);
  }
  if (pts_x) std::memcpy(pts_x, s.pts_x.data(), nchi * 8);
  if (pts_y) std::memcpy(pts_y, s.pts_y.data(), nchi * 8);
  if (pts_chi) std::memcpy(pts_chi, s.pts_chi.data(), nchi * 8);
  if (pts_eta) std::memcpy(pts_eta, s.pts_eta.data(), nchi * 8);
  if (cell_idx)
    for (int i = 0; i < nchi; ++i) cell_idx[i] = s.cell_idx[i];
  if (t) *t = s.t;
  if (dt) *dt = s.dt;
}

// Derived fields after the last operation: p, T, a (ghosted each), beta, speed_x, speed_y.
void orc_get_derived(orc_ctx* c, double* p, double* T, double* a, double* beta, double* speed_x,
                     double* speed_y) {
  State& s = c->s;
  const size_t G = (size_t)(c->c.nchi + 2) * (c->c.neta + 2);
  const int nchi = c->c.nchi;
  if (p) std::memcpy(p, s.p.data(), G * 8);
  if (T) std::memcpy(T, s.T.data(), G * 8);
  if (a) std::memcpy(a, s.a.data(), G * 8);
  if (beta && s.beta.size() == (size_t)nchi) std::memcpy(beta, s.beta.data(), nchi * 8);
  if (speed_x && s.speed_x.size() == (size_t)nchi) std::memcpy(speed_x, s.speed_x.data(), nchi * 8);
  if (speed_y && s.speed_y.size() == (size_t)nchi) std::memcpy(speed_y, s.speed_y.data(), nchi * 8);
}

// NON_LINEAR_DYNAMICS_NO_DISCONTINUITY on the context state, in place (the state
// is mutated exactly as the reference mutates `s`); flux = 4 x Nchi*Neta.
static void copy_flux_out(orc_ctx* c, double* flux) {
  const size_t N = (size_t)c->c.nchi * c->c.neta;
  if (flux) {
    std::memcpy(flux, c->s.flux_rho.data(), N * 8);
    std::memcpy(flux + N, c->s.flux_rho_u.data(), N * 8);
    std::memcpy(flux + 2 * N, c->s.flux_rho_v.data(), N * 8);
    std::memcpy(flux + 3 * N, c->s.flux_rho_E.data(), N * 8);
  }
}

// The entry points that run the shock chain return 0, or -1 with orc_last_error() set
// when the reference would have raised (a shocked row out of range).
static thread_local std::string g_orc_error;
// s["shock"]["relative_increase_velocity"] of the last shock update (Nchi).
void orc_get_rel_vel(orc_ctx* c, double* rel) {
  for (int i = 0; i < c->c.nchi; ++i) rel[i] = i < (int)c->s.rel_vel.size() ? c->s.rel_vel[i] : 0.0;
}

const char* orc_last_error() { return g_orc_error.c_str(); }
#define ORC_GUARD(body)                     \
  try {                                     \
    body;                                   \
  } catch (const std::exception& e) {       \
    g_orc_error = e.what();                 \
    return -1;                              \
  }                                         \
  return 0

int orc_residual(orc_ctx* c, double* flux) {
  ORC_GUARD(non_linear_dynamics(c->c, c->m, c->s); copy_flux_out(c, flux));
}


// Sets the Dict's persistent flux arrays (read by CFL_TIMESTEP's dt2 term).
void orc_set_flux(orc_ctx* c, const double* flux) {
  const size_t N = (size_t)c->c.nchi * c->c.neta;
  std::memcpy(c->s.flux_rho.data(), flux, N * 8);
  std::memcpy(c->s.flux_rho_u.data(), flux + N, N * 8);
  std::memcpy(c->s.flux_rho_v.data(), flux + 2 * N, N * 8);
  std::memcpy(c->s.flux_rho_E.data(), flux + 3 * N, N * 8);
}

int orc_update_flow_cells(orc_ctx* c) { ORC_GUARD(update_flow_cells(c->c, c->m, c->s)); }
int orc_update_shock_bc(orc_ctx* c) {
  ORC_GUARD(update_thermo(c->c, c->s); update_shock_bc(c->c, c->m, c->s));
}
double orc_cfl_timestep(orc_ctx* c) { return cfl_timestep(c->c, c->m, c->s); }

// `nsteps` calls of ADVECT_FLOW (explicit RK4).
int orc_advect(orc_ctx* c, int nsteps) {
  ORC_GUARD(for (int k = 0; k < nsteps; ++k) advect_flow_explicit(c->c, c->m, c->s));
}

void orc_counters(orc_ctx* c, int32_t* rho_limited, int32_t* rh_warnings) {
  if (rho_limited) *rho_limited = c->s.rho_limited;
  if (rh_warnings) *rh_warnings = c->s.rh_warnings;
}

// Smoothing spline (exported for the scipy cross-check): fit (xs, ys, λ), then
// evaluate value and derivative at t (with Linear() extrapolation).
void orc_spline(int n, const double* xs, const double* ys, double lambda, int m, const double* t,
                double* val, double* der) {
  SmoothingSpline sp;
  sp.fit(n, xs, ys, lambda);
  for (int k = 0; k < m; ++k) {
    if (val) val[k] = sp.eval(t[k]);
    if (der) der[k] = sp.deriv(t[k]);
  }
}

void orc_element_space(const orc_config* cfg, int n, const double* x, const double* y, double* chi,
                       double* eta) {
  go_to_element_space(*cfg, n, x, y, chi, eta);
}

// LINEARIZE_L.jl:34-69 preparation (flow cells, shock BC, thermo, BCs; no remesh)
// followed by the coloured finite-difference assembly into stencil blocks
// (Nchi*Neta*144 doubles).
static void linearize_prepared(orc_ctx* c, double* coef) {
  if (c->c.shock_enabled) {
    update_flow_cells(c->c, c->m, c->s);
    update_thermo(c->c, c->s);
    update_shock_bc(c->c, c->m, c->s);
  }
  update_thermo(c->c, c->s);
  update_sound_speed(c->c, c->s);
  apply_boundary_conditions(c->c, c->m, c->s);
  linearize_equations(c->c, c->m, c->s, coef);
}
int orc_linearize(orc_ctx* c, double* coef) { ORC_GUARD(linearize_prepared(c, coef)); }

// Assembly only, on the current state (no preparation).
void orc_jacobian(orc_ctx* c, double* coef) { linearize_equations(c->c, c->m, c->s, coef); }

void orc_matvec(const orc_config* cfg, const double* coef, const double* x, double* y, int transpose) {
  stencil_matvec(*cfg, coef, x, y, transpose);
}

// LINEARIZE_B of the prepared state (run orc_linearize first).
int orc_linearize_b(orc_ctx* c, int32_t* rows, double* bq, double* bs) {
  ORC_GUARD(linearize_b(c->c, c->m, c->s, rows, bq, bs));
}

// Per-column upstream state of the context (4 x Nchi; NULL removes it), for residuals with
// a prescribed upstream state (CHECK_LINEARIZATION_B).
void orc_set_upstream(orc_ctx* c, const double* cols) {
  if (!cols) c->s.up_cols.clear();
  else c->s.up_cols.assign(cols, cols + 4 * (size_t)c->c.nchi);
}

// Shock-position blocks of the prepared state (run orc_linearize first; see
// linearize_shock_blocks for the layouts).
int orc_shock_blocks(orc_ctx* c, int32_t* rows, double* a21_full, double* a12, double* a22) {
  ORC_GUARD(linearize_shock_blocks(c->c, c->m, c->s, rows, a21_full, a12, a22));
}

// y = A x on the extended vectors (4N + Nchi), a21 compact (Nchi x 8).
void orc_matvec_ext(const orc_config* cfg, const double* coef, const int32_t* rows, const double* a21,
                    const double* a12, const double* a22, const double* x, double* y, int transpose) {
  stencil_matvec(*cfg, coef, x, y, transpose);
  shock_matvec(*cfg, rows, a21, a12, a22, x, y, transpose);
}

// POWER_METHOD! with the extended operator: term = (A dt) v (A dt scaled entry by entry, as
// CuSparseMatrixCSC(A * dt)), v = term, vout += v / j!; v = vout after each step.
void orc_expm_ext(const orc_config* cfg, const double* coef, const int32_t* rows, const double* a21,
                  const double* a12, const double* a22, double dt, int nsteps, int order, const double* x,
                  double* y, int transpose) {
  const size_t nchi = cfg->nchi;
  const size_t n = (size_t)4 * cfg->nchi * cfg->neta + nchi;
  const size_t nc = (size_t)cfg->nchi * cfg->neta * 144;
  vec cdt(nc), b21(8 * nchi), b12(4 * nchi * nchi), b22(nchi * nchi);
  for (size_t k = 0; k < nc; ++k) cdt[k] = coef[k] * dt;
  for (size_t k = 0; k < b21.size(); ++k) b21[k] = a21[k] * dt;
  for (size_t k = 0; k < b12.size(); ++k) b12[k] = a12[k] * dt;
  for (size_t k = 0; k < b22.size(); ++k) b22[k] = a22[k] * dt;
  vec v(x, x + n), vout(x, x + n), term(n);
  for (int st = 0; st < nsteps; ++st) {
    long long fact = 1;
    for (int j = 1; j <= order; ++j) {
      stencil_matvec(*cfg, cdt.data(), v.data(), term.data(), transpose);
      shock_matvec(*cfg, rows, b21.data(), b12.data(), b22.data(), v.data(), term.data(), transpose);
      v.swap(term);
      fact = j * fact;
      double r = 1.0 / (double)fact;
#pragma omp parallel for schedule(static)
      for (long k = 0; k < (long)n; ++k) vout[k] += v[k] * r;
    }
    v = vout;
  }
  std::memcpy(y, vout.data(), n * 8);
}

// POWER_METHOD! (ARNOLDI_POWER_GPU.jl:64-82): x <- (Σ_{j<=order} (A dt)^j / j!)^nsteps x,
// with the reference's accumulation order; transpose applies (A dt)ᵀ.
void orc_expm(const orc_config* cfg, const double* coef, double dt, int nsteps, int order,
              const double* x, double* y, int transpose) {
  const size_t n = (size_t)4 * cfg->nchi * cfg->neta;
  vec v(x, x + n), vout(x, x + n), term(n);
  // coef * dt, as CuSparseMatrixCSC(A * dt) (EIGENVALUES.jl:139)
  const size_t nc = (size_t)cfg->nchi * cfg->neta * 144;
  vec cdt(nc);
  for (size_t k = 0; k < nc; ++k) cdt[k] = coef[k] * dt;
  for (int st = 0; st < nsteps; ++st) {
    long long fact = 1;
    for (int j = 1; j <= order; ++j) {
      stencil_matvec(*cfg, cdt.data(), v.data(), term.data(), transpose);
      v.swap(term);
      fact = j * fact;
      double r = 1.0 / (double)fact;
#pragma omp parallel for schedule(static)
      for (long k = 0; k < (long)n; ++k) vout[k] += v[k] * r;
    }
    v = vout;
  }
  std::memcpy(y, vout.data(), n * 8);
}

}  // extern "C"
