// Residual, shock fitting, boundary conditions and time-marching kernels (sm_103a).
//
// One RK4 step (ADVECT_FLOW_EXPLICIT, utils/Time_marching/ADVECT_FLOW_EXPLICIT.jl:36-81)
// is one CUDA graph of these kernels over five streams (api.cu, enqueue_step):
//
//   k_flow_cells        UPDATE_FLOW_CELLS on S (a warp per chi column)
//   k_classify_tiles    the step's flux tile lists (interior / shock and boundary)
//   k_cmax_screen, k_cmax_exact, k_cfl_screen, k_cfl_exact   CFL_TIMESTEP through an FP32
//                       screen and an exact FP64 pass, dt on the device (k_sound_cmax,
//                       k_cfl_faces, k_cfl, k_cfl_final: the FP64 reduction over every cell)
//   k_update_thermo     the stage copy and stage updates of Y and S, p and T
//   k_spline_rows, k_spline_fit   the smoothing-spline fit of the shock points (one CTA)
//   k_shock_columns     R-H jump, extrapolation, MOVE_SHOCK (three warps per 32 columns)
//   k_move_shock        MOVE_SHOCK of the first stage, once dt is known (one CTA)
//   k_bc_edges          ghost-cell boundary conditions (chi edges, then eta edges)
//   k_flux              the FV residual of a stage, in two launches (interior tiles, then
//                       the shock-band and boundary tiles)
//   k_fill_minrho       UPDATE_FIELD_UPSTREAM + MIN_RHO on S, t += dt
//
// The flux kernel dominates. It is FP64-bound on GB300 (the DFMA rate is about 1.7 per
// clock per SM): geometry-only factors are precomputed per face (common.cuh), every face
// flux is evaluated once per tile, the viscous terms of the RK step in float-float on the
// FP32 pipe (ff.cuh), and divisions are replaced by reciprocal multiplies (frcp).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "ff.cuh"
#include "kernels.h"

namespace hymor {

namespace {

constexpr int TX = 31;           // cells per tile along chi (TX + 1 = 32 lr faces per row)
constexpr int TY = 8;            // cells per tile along eta
constexpr int HX = TX + 2;       // halo columns
constexpr int CX = TX + 1;       // corner columns
// Tile geometry of a 31 x TYV-cell flux tile (TYV warps, one per tile row). With TMA the
// halo rows are staged 36 doubles wide (kTmaBoxX: the 33 halo columns from an even first
// column, the 16-byte rule of a TMA box's x coordinate) and each staged plane starts on a
// 128-byte boundary.
constexpr int kTmaBoxX = 36;
template <int TYV, bool TMA = false>
struct TileGeo {
  static constexpr int NH = HX * (TYV + 2);        // halo cells
  static constexpr int HP = TMA ? kTmaBoxX : HX;   // halo row pitch in shared memory
  static constexpr int PS = TMA ? (HP * (TYV + 2) + 15) / 16 * 16 : NH;  // halo plane stride
  static constexpr int NCOR = CX * (TYV + 1);      // corners
  static constexpr int NBTF = TX * (TYV + 1);      // bt faces
  static constexpr int THREADS = 32 * TYV;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Waits for the mbarrier phase `parity` to complete, for at most ~2^22 polls. Returns
// whether it completed.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// ceiling of the flux kernels' dynamic shared memory (above the 48 KB default)
constexpr size_t kFluxMaxSmem = 120 * 1024;

// x > 0 (NaN excluded) on the integer pipe: the bit patterns of +0 .. +inf are ordered
// as unsigned integers, and every NaN or negative pattern lies above +inf.
__device__ __forceinline__ bool positive(double x) {
  return (unsigned long long)__double_as_longlong(x) - 1ull < 0x7ff0000000000000ull;
}

__device__ __forceinline__ bool flow_at(const int* cell_idx, bool shock, int i, int j1) {
  // j1: 1-based interior row; flow cells are rows below the shocked row
  return !shock || j1 < cell_idx[i];
}

// ---------------------------------------------------------------------------
// Stage update + thermodynamic state (INTEGRATION.jl:53-71 followed by
// UPDATE_THERMODYNAMIC_PROPERTIES.jl:22-31, CPG: cv* = 1).
struct UpdArgs {
  Cons S, Y, Yc;
  const double* F0;
  const double* F1;
  const double* F2;
  const double* F3;
  double *p, *T;
  const int* cell_idx;
  const double* scal;
  unsigned* err;
  double* aY;        // sound speed of the lines next to outflow_NRCBC edges (LODI input)
  double cY, cS, gm1;
  int nchi, neta, mode, shock;
  int nrcbc;         // bit e set: edge e (chi0, chi1, eta0, eta1) is outflow_NRCBC
};

__global__ void __launch_bounds__(256) k_update_thermo(UpdArgs a) {
  const int NI = a.nchi + 2, NJ = a.neta + 2;
  const long G = (long)NI * NJ;
  // the stage weights once per block: an FP64 instruction costs the SM partition's FP64 pipe
  // the same whatever its active lanes
  __shared__ double wsh[2];
  if (threadIdx.x == 0) {
    const double dt = a.scal[kDt];
    wsh[0] = a.cY * dt;
    wsh[1] = a.cS * dt;
  }
  __syncthreads();
  const double wY = wsh[0], wS = wsh[1];
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < G; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)k % (unsigned)NI), j = (int)((unsigned)k / (unsigned)NI);
    const bool interior = i >= 1 && i <= a.nchi && j >= 1 && j <= a.neta;
    // Upstream of the shock band (interior rows >= sc + 3) nothing changes the stage array
    // or the solution between the step's first update and its end (the flux is masked
    // there and only the step-start / step-end fills write it, with Y = S), so p and T
    // would be recomputed from the same values: the later updates skip those cells.
    if ((a.mode == 1 || a.mode == 2) && a.shock && interior && j >= a.cell_idx[i - 1] + 3) continue;
    double r, u, v, e;
    const Cons& tgt = (a.mode == 2 || a.mode == 3) ? a.S : a.Y;
    if (a.mode == 0) {
      r = a.S.rho[k]; u = a.S.ru[k]; v = a.S.rv[k]; e = a.S.rE[k];
      a.Y.rho[k] = r; a.Y.ru[k] = u; a.Y.rv[k] = v; a.Y.rE[k] = e;
    } else {
      r = tgt.rho[k]; u = tgt.ru[k]; v = tgt.rv[k]; e = tgt.rE[k];
      if (interior && (a.mode == 1 || a.mode == 2 || a.mode == 5)) {
        const long c = (long)(i - 1) + (long)(j - 1) * a.nchi;
        if (flow_at(a.cell_idx, a.shock, i - 1, j)) {
          const double f0 = a.F0[c], f1 = a.F1[c], f2 = a.F2[c], f3 = a.F3[c];
          // S (accumulator) += wS * k
          a.S.rho[k] = fma(wS, f0, a.S.rho[k]);
          a.S.ru[k] = fma(wS, f1, a.S.ru[k]);
          a.S.rv[k] = fma(wS, f2, a.S.rv[k]);
          a.S.rE[k] = fma(wS, f3, a.S.rE[k]);
          if (a.mode == 1) {  // Y (stage) += wY * k
            r = fma(wY, f0, r); u = fma(wY, f1, u); v = fma(wY, f2, v); e = fma(wY, f3, e);
            a.Y.rho[k] = r; a.Y.ru[k] = u; a.Y.rv[k] = v; a.Y.rE[k] = e;
          } else if (a.mode == 2) {
            r = a.S.rho[k]; u = a.S.ru[k]; v = a.S.rv[k]; e = a.S.rE[k];
          }
        }
      }
    }
    // e = (rho_E - (rho_u^2 + rho_v^2) / rho / 2) / rho ; p = rho e (gamma - 1) ; T = e
    const double ir = frcp(r);
    const double ke = fma(u, u, v * v) * ir;
    const double eint = fma(-0.5, ke, e);
    const double p = eint * a.gm1;
    const double T = eint * ir;
    a.p[k] = p;
    a.T[k] = T;
    if (a.nrcbc) {
      // UPDATE_SOUND_SPEED.jl:31-36 for the cells the LODI outflow condition reads
      const bool nb = ((a.nrcbc & 1) && i == 1) || ((a.nrcbc & 2) && i == NI - 2) ||
                      ((a.nrcbc & 4) && j == 1) || ((a.nrcbc & 8) && j == NJ - 2);
      if (nb) a.aY[k] = sqrt((a.gm1 + 1) * p / r);
    }
    if (interior && !(positive(r) && positive(p))) atomicOr(&a.err[kErrFlags], kBitNumeric);
  }
}

// ---------------------------------------------------------------------------
// Shock fitting + boundary conditions, one CTA.

// Element-space coordinates (utils/Mesh/GO_TO_ELEMENT_SPACE.jl:28-140).
__device__ void element_space(const hymor_config& c, double x, double y, double& chi, double& eta) {
  if (c.mapping == HYMOR_MAP_CIRCLE) {
    const double angle_min = -c.circle_angle_extra, angle_max = M_PI / 2;
    // mod(t, 2 pi) for t = atan2(-x, y) + pi/2 in (-pi/2, 3 pi/2] (Julia's mod: result in [0, 2 pi))
    const double t = atan2(-x, y) + M_PI / 2;
    const double mm = t < 0 ? t + 2 * M_PI : (t >= 2 * M_PI ? t - 2 * M_PI : t);
    const double angle = mm - M_PI / 2;
    const double ch = (angle_max - angle) / (angle_max - angle_min);
    const double r = sqrt(x * x + y * y);
    const double dmax = c.dRs + (c.dRe - c.dRs) * (ch * ch);
    chi = ch;
    eta = (r - c.R) / dmax;
  } else if (c.mapping == HYMOR_MAP_BLUNT_CONE) {
    const double Lm = c.L, Rm = c.R, th = c.theta, ib = c.initial_beta;
    const double s_Straight = ((Lm - Rm) + Rm * cos(th)) / sin(th);
    const double s_Curve = 2 * th * Rm;
    const double s_tot = s_Curve + 2 * s_Straight;
    const double s_Str_sh = ((Lm - Rm) + Rm * cos(ib)) / sin(ib);
    const double s_Crv_sh = ib * Rm;
    const double s_tot_sh = 2 * s_Crv_sh + 2 * s_Str_sh;
    const double slope = sin(th - ib);
    const double x_body = y, y_body = -x;
    const double tang = (y_body - (Lm - Rm)) / x_body;
    double eta_phys, chi_arc;
    if ((tang < tan(M_PI / 2 - th)) && (x_body > 0)) {
      eta_phys = y_body * cos(th) + x_body * sin(th) - Rm - (Lm - Rm) * cos(th);
      const double lambda = (x_body / cos(th) - (eta_phys * sin(th) + Rm * sin(th)) / cos(th)) / s_tot;
      chi_arc = s_Straight / s_tot - lambda;
    } else if ((-tan(M_PI / 2 - th) < tang) && (x_body < 0)) {
      eta_phys = y_body * cos(th) - x_body * sin(th) - Rm - (Lm - Rm) * cos(th);
      const double lambda = (-x_body / cos(th) - (eta_phys * sin(th) + Rm * sin(th)) / cos(th)) / s_tot;
      chi_arc = (s_Straight + s_Curve) / s_tot + lambda;
    } else {
      const double angle = atan2((y_body + Rm - Lm), x_body);
      eta_phys = x_body / cos(angle) - Rm;
      chi_arc = (angle - M_PI / 2 + th) / (2 * th * s_tot / s_Curve) + s_Straight / s_tot;
    }
    chi = 1 - 2 * chi_arc;
    const double dmax = (chi_arc < s_Str_sh / s_tot_sh) ? c.dRs + (s_Str_sh - chi_arc * s_tot_sh) * slope : c.dRs;
    eta = eta_phys / dmax;
  } else if (c.mapping == HYMOR_MAP_CHANNEL) {
    const double p = c.eta_refinement_power;
    chi = (x * cos(c.channel_angle) + y * sin(c.channel_angle)) / c.Lx;
    const double er = (-x * sin(c.channel_angle) + y * cos(c.channel_angle)) / c.Ly;
    eta = er <= 0.5 ? pow(er / pow(2.0, p - 1), 1 / p) : 1 - pow((1 - er) / pow(2.0, p - 1), 1 / p);
  } else {
    chi = 1 - y / c.Lx;
    const double dmax = c.dRs + (c.dRe - c.dRs) * (1 - chi);
    eta = -x / dmax;
  }
}

// g = y - lam Q gamma (one point per thread); ih[k] = 1 / (x[k+1] - x[k])
__device__ double spline_g(int n, const double* ih, const double* ys, const double* gam, double lam, int r) {
  double qg = 0;
  if (r - 1 >= 1 && r - 1 <= n - 2) qg += ih[r - 1] * gam[r - 1];
  if (r >= 1 && r <= n - 2) qg += (-ih[r - 1] - ih[r]) * gam[r];
  if (r + 1 >= 1 && r + 1 <= n - 2) qg += ih[r] * gam[r + 1];
  return ys[r] - lam * qg;
}

// Freestream state seen by shock point i (COMPUTE_UPSTREAM_CONDITIONS.jl:31-112): the
// (disturbed) freestream, or with cols (4 x Nchi: rho, rho_u, rho_v, rho_E per column) the
// prescribed per-column upstream state of `rho_0_upstream_p` (:87-91).
__device__ void upstream(const hymor_config& c, double t, double px, double py, bool first, double& p_inf,
                         double& u_inf, double& v_inf, double& rho_inf, const double* cols = nullptr, int i = 0) {
  double rho, ru, rv, rE;
  if (cols) {
    rho = cols[i];
    ru = cols[c.nchi + i];
    rv = cols[2 * c.nchi + i];
    rE = cols[3 * c.nchi + i];
  } else {
    const double u_y = c.rho_v_0 / c.rho_0, u_x = c.rho_u_0 / c.rho_0;
    const double pert = cos(2.0 * M_PI * c.dist_ky * (py - u_y * t)) * sin(2.0 * M_PI * c.dist_kx * (px - u_x * t));
    rho = c.rho_0 + pert * c.dist_amp[0];
    ru = c.rho_u_0 + pert * c.dist_amp[1];
    rv = c.rho_v_0 + pert * c.dist_amp[2];
    rE = c.rho_E_0 + pert * c.dist_amp[3];
  }
  if (c.axisymmetric && first) rv = 0;
  v_inf = rv / rho;
  u_inf = ru / rho;
  const double um = sqrt(v_inf * v_inf + u_inf * u_inf);
  const double e_inf = (rE - rho * (um * um) * 0.5) / rho;
  p_inf = e_inf * rho * (c.gamma - 1.0);
  rho_inf = rho;
}

// Ghost-cell boundary condition of one edge at position k (0-based along the
// ghosted edge), APPLY_BOUNDARY_CONDITIONS.jl:1-828.
struct EdgeCtx {
  int edge, bc, NI, NJ, nchi, neta;
};

__device__ __forceinline__ int at(const EdgeCtx& e, int depth, int k) {
  if (e.edge == 0) return gidx(depth, k, e.nchi);
  if (e.edge == 1) return gidx(e.NI - 1 - depth, k, e.nchi);
  if (e.edge == 2) return gidx(k, depth, e.nchi);
  return gidx(k, e.NJ - 1 - depth, e.nchi);
}
__device__ __forceinline__ int at_per(const EdgeCtx& e, int k) {
  if (e.edge == 0) return gidx(e.NI - 2, k, e.nchi);
  if (e.edge == 1) return gidx(1, k, e.nchi);
  if (e.edge == 2) return gidx(k, e.NJ - 2, e.nchi);
  return gidx(k, 1, e.nchi);
}

__device__ void edge_normal(const EdgeCtx& e, const DevMesh& m, int k, double& nx, double& ny) {
  // k is the 0-based ghosted position (interior positions 1..len-2)
  if (e.edge == 0) { const long f = (long)0 + (long)(k - 1) * (e.nchi + 1); nx = m.lr_xn[f]; ny = m.lr_yn[f]; }
  else if (e.edge == 1) { const long f = (long)e.nchi + (long)(k - 1) * (e.nchi + 1); nx = m.lr_xn[f]; ny = m.lr_yn[f]; }
  else if (e.edge == 2) { const long f = (long)(k - 1); nx = m.bt_xn[f]; ny = m.bt_yn[f]; }
  else { const long f = (long)(k - 1) + (long)e.neta * e.nchi; nx = m.bt_xn[f]; ny = m.bt_yn[f]; }
}

// First pass of one edge: everything but the symmetry end copies. Each case loads the
// values it reads before it stores any: the compiler cannot tell the planes apart, so a
// load after a store would wait for the store's own load to return.
__device__ void edge_bc_point(const hymor_config& c, const EdgeCtx& e, const DevMesh& m, Cons q,
                              double* P, double* Tt, const double* A, int k, int len) {
  const int g = at(e, 0, k), a1 = at(e, 1, k), a2 = at(e, 2, k);
  double* R = q.rho;
  double* U = q.ru;
  double* V = q.rv;
  double* E = q.rE;
  const bool inner = k >= 1 && k <= len - 2;
  switch (e.bc) {
    case HYMOR_BC_INFLOW_SUBSONIC: {
      const double e1 = E[a1], e2 = E[a2], p1 = P[a1], p2 = P[a2];
      R[g] = c.rho_0; U[g] = c.rho_u_0; V[g] = c.rho_v_0; E[g] = 2 * e1 - e2; P[g] = 2 * p1 - p2;
      break;
    }
    case HYMOR_BC_INFLOW_SUPERSONIC:
      R[g] = c.rho_0; U[g] = c.rho_u_0; V[g] = c.rho_v_0; E[g] = c.rho_E_0; P[g] = c.p_0;
      break;
    case HYMOR_BC_NO_SLIP_ADIABATIC: {
      const double r1 = R[a1], u1 = U[a1], v1 = V[a1], e1 = E[a1], e2 = E[a2];
      const double p1 = P[a1], p2 = P[a2], t1 = Tt[a1];
      R[g] = r1; U[g] = -u1; V[g] = -v1; E[g] = 2 * e1 - e2; P[g] = 2 * p1 - p2; Tt[g] = t1;
      break;
    }
    case HYMOR_BC_NO_SLIP_ISOTHERMAL: {
      const double r1 = R[a1], u1 = U[a1], v1 = V[a1], e1 = E[a1], e2 = E[a2];
      const double p1 = P[a1], p2 = P[a2], t1 = Tt[a1];
      const double Tw = (e.edge <= 1) ? c.Tw_chi0 : (e.edge == 2 ? c.Tw_eta0 : c.Tw_eta1);
      const double T_w = Tw * c.cv / c.energy_factor;
      R[g] = r1; U[g] = -u1; V[g] = -v1; E[g] = 2 * e1 - e2; P[g] = 2 * p1 - p2;
      Tt[g] = 2 * T_w - t1;
      break;
    }
    case HYMOR_BC_OUTFLOW_SUBSONIC: {
      const double r1 = R[a1], r2 = R[a2], e1 = E[a1], e2 = E[a2], u1 = U[a1], u2 = U[a2];
      const double v1 = V[a1], v2 = V[a2], p1 = P[a1], t1 = Tt[a1];
      R[g] = 2 * r1 - r2; E[g] = 2 * e1 - e2; U[g] = 2 * u1 - u2; V[g] = 2 * v1 - v2; P[g] = p1;
      if (e.edge != 1) Tt[g] = t1;
      break;
    }
    case HYMOR_BC_OUTFLOW_SUPERSONIC: {
      const double r1 = R[a1], r2 = R[a2], e1 = E[a1], e2 = E[a2], u1 = U[a1], u2 = U[a2];
      const double v1 = V[a1], v2 = V[a2], p1 = P[a1], p2 = P[a2], t1 = Tt[a1];
      R[g] = 2 * r1 - r2; E[g] = 2 * e1 - e2; U[g] = 2 * u1 - u2; V[g] = 2 * v1 - v2; P[g] = 2 * p1 - p2;
      Tt[g] = t1;
      break;
    }
    case HYMOR_BC_OUTFLOW_SUPERSONIC_1ST: {
      const double u1 = U[a1], v1 = V[a1], r1 = R[a1], e1 = E[a1], p1 = P[a1], t1 = Tt[a1];
      U[g] = u1; V[g] = v1; R[g] = r1; E[g] = e1; P[g] = p1; Tt[g] = t1;
      break;
    }
    case HYMOR_BC_OUTFLOW_NRCBC: {
      const double r1 = R[a1], r2 = R[a2], u1 = U[a1], u2 = U[a2], v1 = V[a1], v2 = V[a2];
      const double e1 = E[a1], e2 = E[a2], p1 = P[a1], p2 = P[a2], t1 = Tt[a1];
      const double rg = 2 * r1 - r2, ug = 2 * u1 - u2, vg = 2 * v1 - v2;
      double eg = 2 * e1 - e2, pg = 2 * p1 - p2;
      if (inner) {
        double nx, ny;
        edge_normal(e, m, k, nx, ny);
        const double a = A[a1];
        const double rho_int = r1;
        const double irg = frcp(rg);
        double ung = (ug * nx + vg * ny) * irg;
        double uni = (u1 * nx + v1 * ny) * frcp(rho_int);
        if (e.edge == 0 || e.edge == 2) { ung = -ung; uni = -uni; }
        if (ung < a) {
          const double p_lodi = p1 + rho_int * a * (ung - uni);
          pg = p_lodi;
          const double rho_e = pg * (1.0 / (c.gamma - 1));
          eg = rho_e + 0.5 * (ug * ug + vg * vg) * irg;
        }
      }
      R[g] = rg; U[g] = ug; V[g] = vg; E[g] = eg; P[g] = pg; Tt[g] = t1;
      break;
    }
    case HYMOR_BC_PERIODIC: {
      const int s = at_per(e, k);
      const double us = U[s], vs = V[s], rs = R[s], es = E[s], ps = P[s], ts = Tt[s];
      U[g] = us; V[g] = vs; R[g] = rs; E[g] = es; P[g] = ps; Tt[g] = ts;
      break;
    }
    case HYMOR_BC_SYMMETRY: {
      const double r1 = R[a1], p1 = P[a1], e1 = E[a1], t1 = Tt[a1];
      if (inner) {
        const double u1 = U[a1], v1 = V[a1];
        double nx, ny;
        edge_normal(e, m, k, nx, ny);
        const double fv = u1 * nx + v1 * ny;
        U[g] = u1 - 2 * fv * nx;
        V[g] = v1 - 2 * fv * ny;
      }
      R[g] = r1; P[g] = p1; E[g] = e1; Tt[g] = t1;
      break;
    }
    default:
      break;
  }
}

// ---------------------------------------------------------------------------
// Shock fitting split over the GPU:
//   k_spline_fit     one CTA: the serial banded factorisation of the smoothing
//                    spline (the only O(Nchi) recurrence), both ordinates at once
//   k_shock_columns  one thread per chi column: resample, element space, beta,
//                    Rankine-Hugoniot jump, extrapolation, MOVE_SHOCK (or k_move_shock
//                    after it, once the time step is known)
//   k_bc_edges       the two boundary phases (chi edges, then eta edges, whose corners
//                    read the chi ghosts), one launch each, one thread per edge point
// Spline workspace (units of n = Nchi doubles): 0 knots, 1-2 ordinates x/y, 3-4
// second derivatives x/y, 5-6 fitted values x/y, 7-11 per-row d0 d1 d2 rhs_x rhs_y,
// 12-14 FP64 Cholesky factors of the fallback solve, 15 interval reciprocals
// 1/(x[k+1] - x[k]).

// 1/sqrt(a): hardware seed (rsqrt.approx.ftz.f64) refined by two Newton-Raphson
// steps y <- y (3 - a y^2) / 2 (quadratic convergence, ~2^-80 before rounding).
__device__ __forceinline__ double frsqrt(double a) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
  double h = 0.5 * a;
  y = y * fma(-h * y, y, 1.5);
  y = y * fma(-h * y, y, 1.5);
  return y;
}

struct SplineArgs {
  ShockPts pts, pS;
  double* ws;
  double lam;
  int n, copy_pts;
};

// Per-row bands of A = R + lam Q^T Q, right-hand sides Q^T y and interval reciprocals,
// one thread per row (the rows are independent), after copying the shock points of S
// into the stage array at stage 1.
__global__ void __launch_bounds__(128) k_spline_rows(SplineArgs A) {
  const int n = A.n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* xs = A.ws;
  double* yx = xs + n;
  double* yy = yx + n;
  double* d0 = A.ws + 7 * n;
  double* d1 = d0 + n;
  double* d2 = d1 + n;
  double* rx = d2 + n;
  double* ry = rx + n;
  double* ih = A.ws + 15 * n;  // 1 / (x[k+1] - x[k])
  const ShockPts& src = A.copy_pts ? A.pS : A.pts;
  const double lam = A.lam;
  auto X = [&](int k) { return src.chi[k]; };
  xs[i] = src.chi[i];
  yx[i] = src.x[i];
  yy[i] = src.y[i];
  if (A.copy_pts) {
    A.pts.x[i] = A.pS.x[i]; A.pts.y[i] = A.pS.y[i];
    A.pts.chi[i] = A.pS.chi[i]; A.pts.eta[i] = A.pS.eta[i];
  }
  if (i + 1 < n) ih[i] = 1.0 / (X(i + 1) - X(i));
  const int m = n - 2;
  const int jj = i;
  if (jj < m) {
    const int j = jj + 1;
    const double hm = X(j) - X(j - 1), h0 = X(j + 1) - X(j);
    const double qm = 1.0 / hm, qp = 1.0 / h0, q0 = -qm - qp;
    d0[jj] = (hm + h0) / 3 + lam * (qm * qm + q0 * q0 + qp * qp);
    double e1 = 0, e2 = 0;
    if (jj + 1 < m) {
      const double h1 = X(j + 2) - X(j + 1);
      const double qm1 = 1.0 / h0, qp1 = 1.0 / h1, q01 = -qm1 - qp1;
      e1 = h0 / 6 + lam * (q0 * qm1 + qp * q01);
    }
    if (jj + 2 < m) e2 = lam * (qp * (1.0 / (X(j + 2) - X(j + 1))));
    d1[jj] = e1;
    d2[jj] = e2;
    rx[jj] = qm * src.x[j - 1] + q0 * src.x[j] + qp * src.x[j + 1];
    ry[jj] = qm * src.y[j - 1] + q0 * src.y[j] + qp * src.y[j + 1];
  }
}

// Solves A gamma = Q^T y for the x and y ordinates (one CTA). GB300 runs a dependent
// FP64 instruction in ~64 cycles and an FP32 one in ~4.5, so the inherently serial
// banded Cholesky factorisation and the two triangular sweeps run in FP32, and
// mixed-precision iterative refinement (FP64 residual r = b - A x, FP32 correction
// solve, x += e; Moler, J. ACM 14 (1967) 316-321) brings the solution to FP64
// accuracy. Each refinement step contracts the error by about cond(A) * 2^-24 (the
// observed ratio rho of successive corrections). The loop stops once the remaining
// error rho * |e| either is below 2^-50 of the solution gamma, or moves the fitted
// values g = y - lam Q gamma by less than 2^-56 of max|y| (|Q|_inf <= max 2 (1/h_{k-1} +
// 1/h_k)); with the default smoothing parameter lam |Q| is ~1e-7, so one refinement step
// suffices. When the corrections contract slower than 1/2 (a heavily smoothed fit
// whose condition number defeats the FP32 factors) or have not converged after
// kMaxRefine steps, the fit is redone by a serial FP64 Cholesky solve.
constexpr int kMaxRefine = 8;

constexpr int kChunk = 8;  // rows loaded into registers ahead of each serial sweep block

// 8 consecutive floats through two 16-byte shared-memory accesses (p 16-byte aligned).
__device__ __forceinline__ void ld8(float (&r)[kChunk], const float* __restrict__ p) {
  const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
  r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
}
__device__ __forceinline__ void st8(float* __restrict__ p, const float (&r)[kChunk]) {
  reinterpret_cast<float4*>(p)[0] = make_float4(r[0], r[1], r[2], r[3]);
  reinterpret_cast<float4*>(p)[1] = make_float4(r[4], r[5], r[6], r[7]);
}

// Forward and backward FP32 sweeps of L L^T x = r for one right-hand side, by one warp:
//   forward:  v_j = c_j - a_j v_{j-1} - b_j v_{j-2}, z_j = v_j / l0_j (c_j = r_j / l0_j)
//   backward: x_j = z_j - p_j x_{j+1} - q_j x_{j+2}
// Each is a second-order linear recurrence, i.e. the state S_j = (v_j, v_{j-1}) follows
// the affine map S_j = T_j(S_{j-1}) = (c_j - a_j S_0 - b_j S_1, S_0). Each lane composes
// the maps of its L consecutive rows (L odd, so that the lanes' shared-memory rows fall
// in distinct banks), a Kogge-Stone scan over the 32 lanes composes the segment maps
// (Blelloch, "Prefix sums and their applications", 1990), and each lane then runs its
// rows from the state the scan hands it: ~3 L + 10 dependent operations instead of m.
struct Affine2 {  // S -> M S + g
  float m00, m01, m10, m11, g0, g1;
};
__device__ __forceinline__ void affine_push(Affine2& A, float a, float b, float c) {  // A <- T ∘ A
  const float n00 = fmaf(-a, A.m00, -b * A.m10), n01 = fmaf(-a, A.m01, -b * A.m11);
  const float ng0 = fmaf(-a, A.g0, fmaf(-b, A.g1, c));
  A.m10 = A.m00; A.m11 = A.m01; A.g1 = A.g0;
  A.m00 = n00; A.m01 = n01; A.g0 = ng0;
}
// inclusive scan over the lanes: lane k ends with the composition of the maps of lanes
// 0..k; returns the state entering lane k's segment (lane 0: S = 0)
__device__ __forceinline__ void affine_scan(Affine2& A, int lane, float& s1, float& s2) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const float p00 = __shfl_up_sync(0xffffffffu, A.m00, d), p01 = __shfl_up_sync(0xffffffffu, A.m01, d);
    const float p10 = __shfl_up_sync(0xffffffffu, A.m10, d), p11 = __shfl_up_sync(0xffffffffu, A.m11, d);
    const float q0 = __shfl_up_sync(0xffffffffu, A.g0, d), q1 = __shfl_up_sync(0xffffffffu, A.g1, d);
    if (lane >= d) {  // A <- A ∘ P
      const float r00 = fmaf(A.m00, p00, A.m01 * p10), r01 = fmaf(A.m00, p01, A.m01 * p11);
      const float r10 = fmaf(A.m10, p00, A.m11 * p10), r11 = fmaf(A.m10, p01, A.m11 * p11);
      const float h0 = fmaf(A.m00, q0, fmaf(A.m01, q1, A.g0)), h1 = fmaf(A.m10, q0, fmaf(A.m11, q1, A.g1));
      A.m00 = r00; A.m01 = r01; A.m10 = r10; A.m11 = r11; A.g0 = h0; A.g1 = h1;
    }
  }
  s1 = __shfl_up_sync(0xffffffffu, A.g0, 1);
  s2 = __shfl_up_sync(0xffffffffu, A.g1, 1);
  if (lane == 0) { s1 = 0.f; s2 = 0.f; }
}
__device__ __forceinline__ void tri_solve_warp_f32(int m, const float* __restrict__ fa, const float* __restrict__ fb,
                                                   const float* __restrict__ fil, const float* __restrict__ fp,
                                                   const float* __restrict__ fq, const float* __restrict__ c,
                                                   float* __restrict__ z, float* __restrict__ o) {
  const int lane = threadIdx.x & 31;
  const int L = ((m + 31) >> 5) | 1;
  {  // forward, lane k on rows [k L, (k + 1) L)
    const int lo = min(m, lane * L), hi = min(m, lo + L);
    Affine2 A{1.f, 0.f, 0.f, 1.f, 0.f, 0.f};
    for (int j = lo; j < hi; ++j) affine_push(A, fa[j], fb[j], c[j]);
    float s1, s2;
    affine_scan(A, lane, s1, s2);
    for (int j = lo; j < hi; ++j) {
      const float v = fmaf(-fa[j], s1, fmaf(-fb[j], s2, c[j]));
      z[j] = v * fil[j];
      s2 = s1; s1 = v;
    }
  }
  __syncwarp();
  {  // backward, lane k on rows m - 1 - k L down to m - (k + 1) L
    const int top = m - 1 - lane * L, bot = max(-1, top - L);
    Affine2 A{1.f, 0.f, 0.f, 1.f, 0.f, 0.f};
    for (int j = top; j > bot; --j) affine_push(A, fp[j], fq[j], z[j]);
    float s1, s2;
    affine_scan(A, lane, s1, s2);
    for (int j = top; j > bot; --j) {
      const float v = fmaf(-fp[j], s1, fmaf(-fq[j], s2, z[j]));
      o[j] = v;
      s2 = s1; s1 = v;
    }
  }
}

__device__ __forceinline__ float rcp_approx_f32(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Pivots of the FP32 banded factorisation A ~ L L^T (one thread). With l0_j^2 = a_j,
// l1_j = t_j / l0_j, l2_j = d2_j / l0_j:
//   a_j = d0_j - t_{j-1}^2 / a_{j-1} - d2_{j-2}^2 / a_{j-2},   t_j = d1_j - d2_{j-1} t_{j-1} / a_{j-1}
// so that the serial chain of a row is one reciprocal and one FMA (the square roots are
// taken afterwards, in parallel). The recurrence forgets its start geometrically when A is
// diagonally dominant, so pivot_window first gets each row's pivot in parallel from the
// kPivWindow rows before it, started at a ~ d0, t ~ d1; the serial form runs only when the
// windowed pivots do not satisfy the recurrence to 2^-20.
constexpr int kPivWindow = 32;

__device__ __forceinline__ void pivot_window(int j, const float* __restrict__ fd0, const float* __restrict__ fd1,
                                             const float* __restrict__ fd2, float& a, float& t) {
  const int s = j > kPivWindow ? j - kPivWindow : 0;
  float q1 = 0.f, q2 = 0.f, t1 = 0.f, e1 = 0.f, e2 = 0.f;
  if (s >= 1) { q1 = rcp_approx_f32(fd0[s - 1]); t1 = fd1[s - 1]; e1 = fd2[s - 1]; }
  if (s >= 2) { q2 = rcp_approx_f32(fd0[s - 2]); e2 = fd2[s - 2]; }
  a = 0.f; t = 0.f;
  for (int r = s; r <= j; ++r) {
    a = fmaf(-t1 * t1, q1, fmaf(-e2 * e2, q2, fd0[r]));
    t = fmaf(-e1 * t1, q1, fd1[r]);
    q2 = q1; q1 = rcp_approx_f32(a); t1 = t; e2 = e1; e1 = fd2[r];
  }
}
__device__ __forceinline__ void chol_pivots_f32(int m, const float* __restrict__ fd0, const float* __restrict__ fd1,
                                                const float* __restrict__ fd2, float* __restrict__ pa,
                                                float* __restrict__ pt) {
  float q1 = 0.f, q2 = 0.f, t1 = 0.f, e1 = 0.f, e2 = 0.f;  // 1/a, t and d2 of rows j-1, j-2
  auto row = [&](float d0, float d1, float d2, float& a, float& t) {
    a = fmaf(-t1 * t1, q1, fmaf(-e2 * e2, q2, d0));
    t = fmaf(-e1 * t1, q1, d1);
    q2 = q1; q1 = rcp_approx_f32(a);
    t1 = t; e2 = e1; e1 = d2;
  };
  int j = 0;
  for (; j + kChunk <= m; j += kChunk) {
    float r0[kChunk], r1[kChunk], r2[kChunk], oa[kChunk], ot[kChunk];
    ld8(r0, fd0 + j); ld8(r1, fd1 + j); ld8(r2, fd2 + j);
#pragma unroll
    for (int u = 0; u < kChunk; ++u) row(r0[u], r1[u], r2[u], oa[u], ot[u]);
    st8(pa + j, oa); st8(pt + j, ot);
  }
  for (; j < m; ++j) row(fd0[j], fd1[j], fd2[j], pa[j], pt[j]);
}

// Serial FP64 banded Cholesky solve of A x = r for both ordinates (one thread); the
// factors go to the workspace slots l0inv, l1, l2 and x overwrites the 1-offset
// solution arrays gx_, gy_ (gx_[j + 1] = x_j).
__device__ __noinline__ void chol_solve_f64(int m, const double* __restrict__ d0, const double* __restrict__ d1,
                               const double* __restrict__ d2, const double* __restrict__ rx,
                               const double* __restrict__ ry, double* __restrict__ il0, double* __restrict__ l1,
                               double* __restrict__ l2, double* __restrict__ gx_, double* __restrict__ gy_) {
  double l1p = 0, l2p = 0, l2pp = 0, zx1 = 0, zx2 = 0, zy1 = 0, zy2 = 0;
  for (int j = 0; j < m; ++j) {
    const double a = d0[j] - l1p * l1p - l2pp * l2pp;
    const double il = frsqrt(a);
    const double nl1 = (d1[j] - l2p * l1p) * il;
    const double nl2 = d2[j] * il;
    // forward: l0_j z_j = r_j - l1_{j-1} z_{j-1} - l2_{j-2} z_{j-2}
    const double zx = (rx[j] - l1p * zx1 - l2pp * zx2) * il;
    const double zy = (ry[j] - l1p * zy1 - l2pp * zy2) * il;
    il0[j] = il; l1[j] = nl1; l2[j] = nl2;
    gx_[j + 1] = zx; gy_[j + 1] = zy;
    zx2 = zx1; zx1 = zx; zy2 = zy1; zy1 = zy;
    l2pp = l2p; l2p = nl2; l1p = nl1;
  }
  // backward: l0_j x_j = z_j - l1_j x_{j+1} - l2_j x_{j+2}
  double x1 = 0, x2 = 0, y1 = 0, y2 = 0;
  for (int j = m - 1; j >= 0; --j) {
    const double xv = (gx_[j + 1] - l1[j] * x1 - l2[j] * x2) * il0[j];
    const double yv = (gy_[j + 1] - l1[j] * y1 - l2[j] * y2) * il0[j];
    gx_[j + 1] = xv; gy_[j + 1] = yv;
    x2 = x1; x1 = xv; y2 = y1; y1 = yv;
  }
}

// Block-wide maxima of K non-negative floats (NaN counts as +inf); every thread gets
// them. red holds 33 K floats.
template <int K>
__device__ __forceinline__ void block_max_f32(float (&v)[K], float* red) {
#pragma unroll
  for (int q = 0; q < K; ++q) {
    if (!(v[q] == v[q])) v[q] = __int_as_float(0x7f800000);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] = fmaxf(v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < K; ++q) red[32 * q + wp] = v[q];
  __syncthreads();
  if (wp == 0) {
    const bool in = lane < (int)(blockDim.x >> 5);
#pragma unroll
    for (int q = 0; q < K; ++q) {
      float a = in ? red[32 * q + lane] : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
      if (lane == 0) red[32 * K + q] = a;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = red[32 * K + q];
}

// Padded row stride of the FP32 arrays of k_spline_fit (a multiple of 4 floats, so that
// every array starts on a 16-byte boundary).
__host__ __device__ inline int spline_stride(int n) { return (n - 2 + 3) & ~3; }
constexpr int kSplineArrays = 14;
// 32 warps: the parallel FP64 phases (residual, corrections, fitted values) spread over
// every warp of the SM; the serial parts use one or two warps
constexpr int kSplineThreads = 1024;

__global__ void __launch_bounds__(kSplineThreads) k_spline_fit(SplineArgs A) {
  __shared__ float red[33 * 4];
  extern __shared__ float4 shf4[];
  float* shf = reinterpret_cast<float*>(shf4);
  const int n = A.n, m = n - 2, tid = threadIdx.x, nt = blockDim.x;
  const int mp = spline_stride(n);
  double* xs = A.ws;
  double* yx = xs + n;
  double* yy = yx + n;
  double* cx = yy + n;
  double* cy = cx + n;
  double* gx = cy + n;
  double* gy = gx + n;
  const double* d0 = A.ws + 7 * n;
  const double* d1 = d0 + n;
  const double* d2 = d1 + n;
  const double* rx = d2 + n;
  const double* ry = rx + n;
  float* fil = shf;           // 1 / l0 (FP32)
  float* fl1 = fil + mp;
  float* fl2 = fl1 + mp;
  float* fa = fl2 + mp;       // l1_{j-1} / l0_j
  float* fb = fa + mp;        // l2_{j-2} / l0_j
  float* fp = fb + mp;        // l1_j / l0_j
  float* fq = fp + mp;        // l2_j / l0_j
  float* wx = fq + mp;        // right-hand sides c = r / l0
  float* wy = wx + mp;
  float* fd0 = wy + mp;       // FP32 bands (factorisation input), then forward results
  float* fd1 = fd0 + mp;
  float* fd2 = fd1 + mp;
  float* ex = fd2 + mp;       // corrections
  float* ey = ex + mp;
  const double lam = A.lam;
  for (int i = tid; i < n; i += nt) { cx[i] = 0; cy[i] = 0; }
  if (m <= 0) {
    __syncthreads();
    for (int i = tid; i < n; i += nt) { gx[i] = yx[i]; gy[i] = yy[i]; }
    return;
  }
  const double* ih = A.ws + 15 * n;
  float qloc = 0.f, yloc = 0.f;  // max 2 (1/h_{k-1} + 1/h_k) and max |y| over this thread's rows
  for (int j = tid; j < m; j += nt) {
    fd0[j] = (float)d0[j]; fd1[j] = (float)d1[j]; fd2[j] = (float)d2[j];
    qloc = fmaxf(qloc, 2.f * ((float)ih[j] + (float)ih[j + 1]));
  }
  for (int i = tid; i < n; i += nt) yloc = fmaxf(yloc, fmaxf(fabsf((float)yx[i]), fabsf((float)yy[i])));
  __syncthreads();
  float* pa = fl1;  // pivots a_j = l0_j^2
  float* pt = fl2;  // t_j = l0_j l1_j
  for (int j = tid; j < m; j += nt) pivot_window(j, fd0, fd1, fd2, pa[j], pt[j]);
  __syncthreads();
  int off = 0;
  for (int j = tid; j < m; j += nt) {
    float ar = fd0[j], tr = fd1[j];
    if (j >= 1) { const float q = rcp_approx_f32(pa[j - 1]); ar = fmaf(-pt[j - 1] * pt[j - 1], q, ar); tr = fmaf(-fd2[j - 1] * pt[j - 1], q, tr); }
    if (j >= 2) ar = fmaf(-fd2[j - 2] * fd2[j - 2], rcp_approx_f32(pa[j - 2]), ar);
    if (!(fabsf(pa[j] - ar) <= 0x1p-20f * fabsf(pa[j]) && fabsf(pt[j] - tr) <= 0x1p-20f * (fabsf(tr) + fabsf(fd1[j]))))
      off = 1;
  }
  if (__syncthreads_or(off)) {
    if (tid == 0) chol_pivots_f32(m, fd0, fd1, fd2, pa, pt);
    __syncthreads();
  }
  for (int j = tid; j < m; j += nt) {
    const float il = rsqrtf(pa[j]);
    fil[j] = il;
    fa[j] = j >= 1 ? pt[j - 1] * rsqrtf(pa[j - 1]) * il : 0.f;   // l1_{j-1} / l0_j
    fb[j] = j >= 2 ? fd2[j - 2] * rsqrtf(pa[j - 2]) * il : 0.f;  // l2_{j-2} / l0_j
    fp[j] = pt[j] * il * il;                                     // l1_j / l0_j
    fq[j] = fd2[j] * il * il;                                    // l2_j / l0_j
    wx[j] = (float)rx[j] * il;
    wy[j] = (float)ry[j] * il;
  }
  __syncthreads();
  // fd0/fd1 are free now: forward-sweep scratch
  float* zx = fd0;
  float* zy = fd1;
  bool direct = false;
  float prev = 0.f;
  for (int pass = 0;; ++pass) {
    if (tid < kWarp) tri_solve_warp_f32(m, fa, fb, fil, fp, fq, wx, zx, ex);
    else if (tid < 2 * kWarp) tri_solve_warp_f32(m, fa, fb, fil, fp, fq, wy, zy, ey);
    __syncthreads();
    // x += e (FP64), then the FP64 residual of the next pass
    float mx[4] = {0.f, 0.f, qloc, yloc};  // |e|, |gamma|, |Q| bound, |y|
    for (int j = tid; j < m; j += nt) {
      const double vx = cx[j + 1] + (double)ex[j], vy = cy[j + 1] + (double)ey[j];
      cx[j + 1] = vx; cy[j + 1] = vy;
      mx[0] = fmaxf(mx[0], fmaxf(fabsf(ex[j]), fabsf(ey[j])));
      mx[1] = fmaxf(mx[1], fmaxf(fabsf((float)vx), fabsf((float)vy)));
    }
    block_max_f32<4>(mx, red);
    const float emax = mx[0], xmax = mx[1];
    if (!(emax <= xmax)) { direct = true; break; }  // NaN or a diverging FP32 solve
    if (pass >= 1) {
      const float rho = emax / fmaxf(prev, 1e-37f);
      const float rem = rho * emax;  // error left in gamma
      if (rem <= 0x1p-50f * xmax || emax <= 0x1p-52f * xmax || (float)lam * mx[2] * rem <= 0x1p-56f * mx[3]) break;
      if (rho > 0.5f || pass == kMaxRefine) { direct = true; break; }
    }
    prev = emax;
    for (int j = tid; j < m; j += nt) {
      // (A x)_j = d2_{j-2} x_{j-2} + d1_{j-1} x_{j-1} + d0_j x_j + d1_j x_{j+1} + d2_j x_{j+2}
      double ax = d0[j] * cx[j + 1], ay = d0[j] * cy[j + 1];
      if (j >= 1) { ax = fma(d1[j - 1], cx[j], ax); ay = fma(d1[j - 1], cy[j], ay); }
      if (j >= 2) { ax = fma(d2[j - 2], cx[j - 1], ax); ay = fma(d2[j - 2], cy[j - 1], ay); }
      if (j + 1 < m) { ax = fma(d1[j], cx[j + 2], ax); ay = fma(d1[j], cy[j + 2], ay); }
      if (j + 2 < m) { ax = fma(d2[j], cx[j + 3], ax); ay = fma(d2[j], cy[j + 3], ay); }
      wx[j] = (float)(rx[j] - ax) * fil[j];
      wy[j] = (float)(ry[j] - ay) * fil[j];
    }
    __syncthreads();
  }
  if (direct) {
    if (tid == 0)
      chol_solve_f64(m, d0, d1, d2, rx, ry, A.ws + 12 * n, A.ws + 13 * n, A.ws + 14 * n, cx, cy);
    __syncthreads();
  }
  // fitted values g = y - lam Q gamma
  for (int i = tid; i < n; i += nt) {
    gx[i] = spline_g(n, ih, yx, cx, lam, i);
    gy[i] = spline_g(n, ih, yy, cy, lam, i);
  }
}

struct ColArgs {
  hymor_config cfg;
  Cons tgt;
  double* p;
  ShockPts pts, pS;
  const double* ws;
  const int* cell_idx;
  double *beta, *speed_x, *speed_y, *rel;
  const double* scal;
  unsigned* err;
  DevMesh m;
  double cY, cS;
  const double* up_cols;                  // per-column upstream state (4 x Nchi) or null
  int move, on_S;
  int disturbed;                          // any freestream disturbance amplitude non-zero
  double p_inf, u_inf, v_inf, rho_inf;    // undisturbed freestream (COMPUTE_UPSTREAM_CONDITIONS.jl)
  double vmag, cph, sph;                  // its speed and flow-angle cosine / sine
  // gas constants of the jump relations: (g+1)/(g-1), 1/(g-1), 2/(g-1)
  double gp1_gm1, igm1, two_igm1;
};

// value and slope of the fitted spline at t (Linear() extrapolation outside the knots)
__device__ void spline_at(int n, const double* xs, const double* g, const double* gam, const double* ih, double t,
                          int guess, double& val, double& der) {
  auto in_der = [&](int k, double tt) {
    const double h = xs[k + 1] - xs[k], a = xs[k + 1] - tt, b = tt - xs[k];
    return (g[k + 1] - g[k]) * ih[k] + ((h * h - 3 * a * a) * gam[k] + (3 * b * b - h * h) * gam[k + 1]) * (ih[k] * (1.0 / 6));
  };
  if (t < xs[0]) { der = in_der(0, xs[0]); val = g[0] + der * (t - xs[0]); return; }
  if (t > xs[n - 1]) { der = in_der(n - 2, xs[n - 1]); val = g[n - 1] + der * (t - xs[n - 1]); return; }
  // the knots stay close to the mesh abscissae, so walk from the column's own interval
  int k = guess < 0 ? 0 : (guess > n - 2 ? n - 2 : guess);
  while (k > 0 && xs[k] > t) --k;
  while (k < n - 2 && xs[k + 1] <= t) ++k;
  const double h = xs[k + 1] - xs[k], a = xs[k + 1] - t, b = t - xs[k];
  val = (a * g[k] + b * g[k + 1]) * ih[k] + ((a * a * a - h * h * a) * gam[k] + (b * b * b - h * h * b) * gam[k + 1]) * (ih[k] * (1.0 / 6));
  der = in_der(k, t);
}

// MOVE_SHOCK (MOVE_SHOCK.jl:29-49) of point i by its shock speed (spx, spy): the solution's
// points by the accumulator weight, the stage points (on_S false) by the stage weight
__device__ __forceinline__ void move_shock_point(const hymor_config& c, const ShockPts& pS, const ShockPts& pts,
                                                 bool on_S, double cY, double cS, double dt, double spx,
                                                 double spy, int i) {
  const double wS = cS * dt * c.relaxation, wY = cY * dt * c.relaxation;
  pS.x[i] = pS.x[i] + spx * wS;
  pS.y[i] = pS.y[i] + spy * wS;
  if (!on_S) {
    pts.x[i] = pts.x[i] + spx * wY;
    pts.y[i] = pts.y[i] + spy * wY;
  }
}

// k_shock_columns: 32 columns per block, the work of a column split over three warps in two
// phases (a warp's FP64 instruction takes the sub-partition's FP64 pipe ~70 cycles whatever
// its active lanes, so the serial chain of one column shortens only when other warps take
// part of it):
//   phase 1: warp 0 evaluates the x spline, warp 1 the y spline, warp 2 loads the shocked
//            column's mesh points and states and forms the geometry and the slopes;
//   phase 2: warp 0 maps the point to element space, warp 1 forms beta, the jump, the
//            extrapolation and the shock speed.
// Each quantity has the arithmetic of the one-thread-per-column form.
constexpr int kColCols = 32;
constexpr int kColThreads = 3 * kColCols;

struct ColShared {
  double xv[kColCols], xd[kColCols], yv[kColCols], yd[kColCols];
  // mesh points of rows sc, sc - 1 and their differences, reciprocal distances
  double x0[kColCols], y0[kColCols], x1[kColCols], y1[kColCols];
  double dx01[kColCols], dy01[kColCols], dx12[kColCols], dy12[kColCols], i01[kColCols], i12[kColCols];
  // the states of rows sc - 1 and sc - 2 (rho, rho u, rho v, rho E, p; p of sc - 2 as the
  // extrapolation reads it) and the slopes of p, rho, rho u, rho v, rho E
  double q1[5][kColCols], q2[5][kColCols], sl[5][kColCols];
  int sc[kColCols];
};

__global__ void __launch_bounds__(kColThreads) k_shock_columns(ColArgs A) {
  __shared__ ColShared sh;
  const hymor_config& c = A.cfg;
  const int nchi = c.nchi, neta = c.neta;
  const int lane = threadIdx.x % kColCols, w = threadIdx.x / kColCols;
  const int i = blockIdx.x * kColCols + lane;
  const bool act = i < nchi;
  const double* xs = A.ws;
  const double* cxs = A.ws + 3 * nchi;
  const double* cys = A.ws + 4 * nchi;
  const double* gxs = A.ws + 5 * nchi;
  const double* gys = A.ws + 6 * nchi;
  const double* ih = A.ws + 15 * nchi;
  const int I = i + 1;
  // phase 1. LEAST_SQUARES_SHOCK_POINTS.jl:60-70, COMPUTE_BETA.jl:37-50: the fitted spline
  // and its slope at the column's abscissa
  if (act && w < 2) {
    double v, dv;
    spline_at(nchi, xs, w == 0 ? gxs : gys, w == 0 ? cxs : cys, ih, A.m.chi1[i], i - 1, v, dv);
    (w == 0 ? sh.xv : sh.yv)[lane] = v;
    (w == 0 ? sh.xd : sh.yd)[lane] = dv;
  } else if (act) {
    // UPDATE_SHOCK_JUMP_PROPERTIES.jl:324-522 and EXTRAPOLATE_CELLS_SHOCK.jl:39-176: the
    // shocked cell's column below the shock
    const int sc = A.cell_idx[i];
    sh.sc[lane] = sc;
    if (sc >= 2 && sc <= neta - 1) {
      const double x0 = A.m.x_ext[gidx(I, sc, nchi)], y0 = A.m.y_ext[gidx(I, sc, nchi)];
      const double x1 = A.m.x_ext[gidx(I, sc - 1, nchi)], y1 = A.m.y_ext[gidx(I, sc - 1, nchi)];
      const double x2 = A.m.x_ext[gidx(I, sc - 2, nchi)], y2 = A.m.y_ext[gidx(I, sc - 2, nchi)];
      const double dx01 = x0 - x1, dy01 = y0 - y1, dx12 = x1 - x2, dy12 = y1 - y2;
      const double i12 = frsqrt(dx12 * dx12 + dy12 * dy12);  // 1 / dist12
      sh.x0[lane] = x0; sh.y0[lane] = y0; sh.x1[lane] = x1; sh.y1[lane] = y1;
      sh.dx01[lane] = dx01; sh.dy01[lane] = dy01; sh.dx12[lane] = dx12; sh.dy12[lane] = dy12;
      sh.i01[lane] = frsqrt(dx01 * dx01 + dy01 * dy01);  // 1 / dist01
      sh.i12[lane] = i12;
      const int g1 = gidx(I, sc - 1, nchi), g2 = gidx(I, sc - 2, nchi);
      const double p_1 = A.p[g1];
      double p_2 = A.p[g2];
      if (sc - 2 == 0 && c.bc_eta0 == HYMOR_BC_NO_SLIP_ISOTHERMAL)
        p_2 = 2 * A.p[gidx(I, 1, nchi)] - A.p[gidx(I, 2, nchi)];  // UPDATE_THERMODYNAMIC_PROPERTIES.jl:28-31
      const double* arr[4] = {A.tgt.rho, A.tgt.ru, A.tgt.rv, A.tgt.rE};
      sh.q1[4][lane] = p_1;
      sh.q2[4][lane] = p_2;
      sh.sl[0][lane] = (p_1 - p_2) * i12;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double a1 = arr[v][g1], a2 = arr[v][g2];
        sh.q1[v][lane] = a1;
        sh.q2[v][lane] = a2;
        sh.sl[v + 1][lane] = (a1 - a2) * i12;
      }
    }
  }
  __syncthreads();
  if (!act || w == 2) return;
  const double xv = sh.xv[lane], yv = sh.yv[lane];
  if (w == 0) {
    double ch, et;
    element_space(c, xv, yv, ch, et);
    A.pts.chi[i] = ch;
    A.pts.eta[i] = et;
    return;
  }
  // phase 2, warp 1
  const double xd = sh.xd[lane], yd = sh.yd[lane];
  const double t = A.scal[kT], dt = A.scal[kDt];
  Cons q = A.tgt;
  A.pts.x[i] = xv; A.pts.y[i] = yv;
  double p_inf = A.p_inf, u_inf = A.u_inf, v_inf = A.v_inf, rho_inf = A.rho_inf;
  const bool local_up = A.disturbed || A.up_cols || (c.axisymmetric && i == 0);
  if (local_up) upstream(c, t, xv, yv, i == 0, p_inf, u_inf, v_inf, rho_inf, A.up_cols, i);
  const double cross = xd * v_inf - yd * u_inf;
  const double dot = xd * u_inf + yd * v_inf;
  // beta = atan2(|cross|, |dot|) enters only through its sine and cosine, |cross| / r and |dot| / r
  double sb, cb;
  {
    const double ir = frsqrt(cross * cross + dot * dot);
    sb = fabs(cross) * ir;
    cb = fabs(dot) * ir;
  }
  if (i == 0 && c.bc_chi0 == HYMOR_BC_SYMMETRY) { sb = 1.0; cb = 0.0; }  // beta = pi/2, UPDATE_SHOCK_BC.jl:31-34
  if (A.on_S) {  // s["shock"]["beta"], read by the shock-position linearisation
    A.beta[i] = sb;
    A.beta[nchi + i] = cb;
  }
  const int sc = sh.sc[lane];
  if (sc < 2 || sc > neta - 1) {
    atomicOr(&A.err[kErrFlags], kBitShockRange);
    return;
  }
  const double i01 = sh.i01[lane], i12 = sh.i12[lane];
  const double dist1s = ((xv - sh.x1[lane]) * sh.dx12[lane] + (yv - sh.y1[lane]) * sh.dy12[lane]) * i12;
  const double dist0s = ((xv - sh.x0[lane]) * sh.dx01[lane] + (yv - sh.y0[lane]) * sh.dy01[lane]) * i01;
  const int g0 = gidx(I, sc, nchi);
  const double p_1 = sh.q1[4][lane];
  const double slope_p = sh.sl[0][lane];
  const double p_s = slope_p * dist1s + p_1;
  const double yr = p_s * frcp(p_inf);
  if (yr < 1) atomicAdd(&A.err[kRhWarn], 1u);
  // the shocked and the free gas share gamma (CPG): Acoef = Bcoef = (g+1)/(g-1)
  const double Acoef = A.gp1_gm1, Bcoef = A.gp1_gm1;
  const double rho_s = rho_inf * (yr * Acoef + 1) * frcp(yr + Bcoef);
  const double irho_s = frcp(rho_s);
  const double e_s = p_s * A.igm1 * irho_s;
  // ang_inf = beta - atan2(v_inf, u_inf): sine and cosine by the angle-difference identity
  double vmag = A.vmag, cph = A.cph, sph = A.sph;
  if (local_up) {
    vmag = sqrt(u_inf * u_inf + v_inf * v_inf);
    const double ivm = frcp(vmag);
    cph = u_inf * ivm;
    sph = v_inf * ivm;
  }
  const double sa = sb * cph - cb * sph, ca = cb * cph + sb * sph;
  const double vn_inf = sa * vmag;
  const double temp1 = 2 * yr * A.igm1 - A.two_igm1;
  const double temp2 = yr * Acoef + 1;
  const double temp3 = p_inf * (yr - 1) * frcp(rho_inf);
  const double rel = -vn_inf + sqrt(temp3 * temp2 * frcp(temp1));
  A.rel[i] = rel;
  const double vt_s = ca * vmag;
  const double vn_s = -rel + rho_inf * irho_s * (rel + vn_inf);
  double spx, spy;
  if (!c.shock_eulerian) {
    spx = -rel * sb;
    spy = rel * cb;
  } else {
    const double sx = -rel * sb, sy = rel * cb;
    spx = sx - sy * (cb * frcp(sb));  // tan(pi/2 - beta) = cos(beta) / sin(beta)
    spy = 0.0;
  }
  A.speed_x[i] = spx;
  A.speed_y[i] = spy;
  const double ru_s = rho_s * (vn_s * sb + vt_s * cb);
  const double rv_s = rho_s * (-vn_s * cb + vt_s * sb);
  const double rE_s = e_s * rho_s + (ru_s * ru_s + rv_s * rv_s) * (0.5 * irho_s);
  // the shocked cell's state (rho, rho u, rho v, rho E, p) and its extrapolation to sc + 1, sc + 2
  double v0[5];
  v0[0] = -sh.sl[1][lane] * dist0s + rho_s;
  v0[1] = -sh.sl[2][lane] * dist0s + ru_s;
  v0[2] = -sh.sl[3][lane] * dist0s + rv_s;
  v0[3] = -sh.sl[4][lane] * dist0s + rE_s;
  v0[4] = -slope_p * dist0s + p_s;
  double* arr[5] = {q.rho, q.ru, q.rv, q.rE, A.p};
  const int i1 = gidx(I, sc + 1, nchi), i2 = gidx(I, sc + 2, nchi);
#pragma unroll
  for (int v = 0; v < 5; ++v) arr[v][g0] = v0[v];
  if (c.shock_interp == 1) {
#pragma unroll
    for (int v = 0; v < 5; ++v) { arr[v][i1] = v0[v]; arr[v][i2] = v0[v]; }
  } else if (c.shock_interp == 2) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double e1 = 2 * v0[v] - sh.q1[v][lane];
      arr[v][i1] = e1;
      if (v < 4) arr[v][i2] = 2 * e1 - v0[v];
    }
  } else {
    // 3 a - 3 b + c with each operation rounded (no fused multiply-add), the reference's
    // association
    auto cubic = [](double a, double b, double c) {
      return __dadd_rn(__dsub_rn(__dmul_rn(3.0, a), __dmul_rn(3.0, b)), c);
    };
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double e1 = cubic(v0[v], sh.q1[v][lane], sh.q2[v][lane]);
      arr[v][i1] = e1;
      if (v < 4) arr[v][i2] = cubic(e1, v0[v], sh.q1[v][lane]);
    }
  }
  // MOVE_SHOCK; the symmetry copy pts_x[1] -> pts_x[0] runs in k_bc_edges
  if (A.move) move_shock_point(c, A.pS, A.pts, A.on_S, A.cY, A.cS, dt, spx, spy, i);
}

// MOVE_SHOCK on its own, after a k_shock_columns launch without it: one CTA moves every
// point by the speeds that launch stored, then makes the symmetry copy pts_x[1] -> pts_x[0].
// It lets the jump and boundary kernels of a step's first stage run before the time step
// is known (only the move needs dt).
struct MoveArgs {
  hymor_config cfg;
  ShockPts pts, pS;
  const double *speed_x, *speed_y, *scal;
  double cY, cS;
  int on_S, fix;
};

__global__ void __launch_bounds__(1024) k_move_shock(MoveArgs A) {
  const int n = A.cfg.nchi;
  const double dt = A.scal[kDt];
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    move_shock_point(A.cfg, A.pS, A.pts, A.on_S, A.cY, A.cS, dt, A.speed_x[i], A.speed_y[i], i);
  __syncthreads();
  if (A.fix && threadIdx.x == 0 && n >= 2) {
    A.pS.x[0] = A.pS.x[1];
    if (!A.on_S) A.pts.x[0] = A.pts.x[1];
  }
}

struct BcArgs {
  hymor_config cfg;
  Cons q;
  double *p, *T;
  const double* a_bc;
  DevMesh m;
  ShockPts pts, pS;
  int phase;     // 0: chi edges, 1: eta edges
  int fix_pts;   // MOVE_SHOCK symmetry copy (phase 0, thread 0)
  int on_S;
};

// point t of the two edges of one phase (0: chi edges, 1: eta edges)
__device__ __forceinline__ void bc_edge_point(const BcArgs& A, int phase, int t) {
  const hymor_config& c = A.cfg;
  const int nchi = c.nchi, neta = c.neta, NI = nchi + 2, NJ = neta + 2;
  const int len = phase == 0 ? NJ : NI;
  const int side = t / len, k = t % len;
  const int edge = 2 * phase + side;
  const int bc = edge == 0 ? c.bc_chi0 : edge == 1 ? c.bc_chi1 : edge == 2 ? c.bc_eta0 : c.bc_eta1;
  if (bc == HYMOR_BC_SHOCK) return;
  EdgeCtx e{edge, bc, NI, NJ, nchi, neta};
  edge_bc_point(c, e, A.m, A.q, A.p, A.T, A.a_bc, k, len);
  if (bc == HYMOR_BC_SYMMETRY) {
    // ends of the ghost line copy their neighbours along the line
    if (k == 1) { A.q.ru[at(e, 0, 0)] = A.q.ru[at(e, 0, 1)]; A.q.rv[at(e, 0, 0)] = A.q.rv[at(e, 0, 1)]; }
    if (k == len - 2) {
      A.q.ru[at(e, 0, len - 1)] = A.q.ru[at(e, 0, len - 2)];
      A.q.rv[at(e, 0, len - 1)] = A.q.rv[at(e, 0, len - 2)];
    }
  }
}

// One boundary phase, one thread per edge point: the chi edges, then (second launch) the
// eta edges, whose corners read the chi ghosts.
__global__ void __launch_bounds__(256) k_bc_edges(BcArgs A) {
  const int len = A.phase == 0 ? A.cfg.neta + 2 : A.cfg.nchi + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (A.fix_pts && t == 0 && A.phase == 0 && A.cfg.nchi >= 2) {
    A.pS.x[0] = A.pS.x[1];
    if (!A.on_S) A.pts.x[0] = A.pts.x[1];
  }
  if (t < 2 * len) bc_edge_point(A, A.phase, t);
}

// ---------------------------------------------------------------------------
// Residual: FLUX_MASS/MOMENTUM/TOTAL_ENERGY + VISCOUS_FLUX (and the *_3D forms),
// fused and face-centric, one 31 x TYV-cell tile per CTA.
struct FluxArgs {
  const double *rho, *ru, *rv, *rE, *p, *T;
  double *o0, *o1, *o2, *o3;
  const int* cell_idx;
  DevMesh m;
  // The gradient planes carry 2 mu*/Re, so the face kernel forms twice the viscous
  // traction (then multiplied by the stored A/2) and, with kpr = gamma / Pr, twice the
  // heat flux k gamma / (Re Pr) dT/dn (CPG: mu* = k* = 1; Sutherland: both times mu_f).
  double kpr;
  double suthS, Tinf_inv;
  float2 kprf, c23f;       // kpr and 2/3 as float-float (the float-float viscous variant)
  unsigned* err;           // device error word (TMA wait timeouts)
  int nchi, neta;
  int mask;                // shock fitting with feedback: zero flux at j >= sc
  int shock;
  int tile_class;          // -1 all tiles; 0 tiles reading nothing the shock/BC kernels write; 1 the others
  // compact tile list of one class (k_classify_tiles): block b processes tile list[b]
  // when b < *count; null: the grid is the tile grid
  const int* list;
  const int* count;
  int tiles_x;
};

// Tile classes of the RK step, once per step (the shocked rows are fixed within a step):
// 0 = the halo (ghosted columns i0-1 .. i0+TX, rows j0 .. j0+TY+1) avoids every ghost cell
// and stays below the shocked rows sc .. sc+2 of its columns, so its flux does not wait
// for the shock/boundary kernels; 1 = the others; tiles wholly at or above the shocked
// rows (zero flux under the NON_LINEAR_DYNAMICS mask, never read by the stage update)
// are left out. lists: [count0, count1, class 0 tiles (cap0), class 1 tiles]. split: each
// tile is listed as its two halves, tiles of the tiling with ty / 2 rows, in its class (a
// half wholly above the shocked rows left out like a tile).
__global__ void k_classify_tiles(const int* __restrict__ cell_idx, int* lists, int nchi, int neta, int tiles_x,
                                 int ntiles, int shock, int mask, int ty, int split, int cap0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const int i0 = (t % tiles_x) * TX, j0 = (t / tiles_x) * ty;
  int sc = 0x7fffffff;
  if (mask) {
    sc = 0;
    for (int c = i0; c < i0 + TX && c < nchi; ++c) sc = max(sc, cell_idx[c]);
    if (j0 + 1 >= sc) return;
  }
  bool inner = i0 >= 1 && i0 + TX + 1 <= nchi && j0 >= 1 && j0 + ty + 1 <= neta;
  if (shock) {
    int scmin = 0x7fffffff;
    for (int c = i0 - 1; c <= i0 + TX; ++c)
      if (c >= 0 && c < nchi) scmin = min(scmin, cell_idx[c]);
    inner = inner && (j0 + ty + 1 < scmin);
  }
  const int cls = inner ? 0 : 1;
  int* list = lists + 2 + cls * cap0;
  if (split) {
    const int h = 2 * (t / tiles_x) * tiles_x + t % tiles_x;  // the lower half's index
    const bool upper = j0 + ty / 2 + 1 < sc && j0 + ty / 2 < neta;
    const int k = atomicAdd(&lists[cls], upper ? 2 : 1);
    list[k] = h;
    if (upper) list[k + 1] = h + tiles_x;
  } else {
    list[atomicAdd(&lists[cls], 1)] = t;
  }
}

// One 31 x TYV-cell tile (bx, by) of the residual, TYV warps (one per tile row); every
// thread of the block takes part.
// The viscous part of one face in float-float arithmetic (the FP64 form, with its
// derivation, is in flux_tile): u, v, T of the two cells A (left / bottom) and B (right /
// top) and the corner sums at the face's two ends (lo, hi), the face's float-float planes
// (nx, ny, s g1, s g2/4, s/(4 len)). LR: an lr face (sg = 1), else a bt face (sg = -1).
// Returns twice the traction (tx, ty), twice the heat flux qn, and for the axisymmetric
// hoop stress -2/3 div + 2 u_f / x_f (the caller scales it by mu_f / 2), all float-float.
template <bool LR, bool AXI>
__device__ __forceinline__ void visc_face_ff(const ff* fu, const ff* fv, const ff* fT, int A, int B, const ff* fuc,
                                             const ff* fvc, const ff* fTc, int lo, int hi, const float2* pl, long NF,
                                             long f, double rxd, float2 kprf, float2 c23f, ff& txf, ff& tyf, ff& qf,
                                             ff& hoop) {
  const ff nx = *reinterpret_cast<const ff*>(pl + f), ny = *reinterpret_cast<const ff*>(pl + NF + f);
  const ff g1 = *reinterpret_cast<const ff*>(pl + 2 * NF + f), g2 = *reinterpret_cast<const ff*>(pl + 3 * NF + f);
  const ff il = *reinterpret_cast<const ff*>(pl + 4 * NF + f);
  const ff dUc = ff_sub(fuc[hi], fuc[lo]), dVc = ff_sub(fvc[hi], fvc[lo]), dTc = ff_sub(fTc[hi], fTc[lo]);
  const ff du_dn = ff_add(ff_mul(g1, ff_sub(fu[B], fu[A])), ff_mul(g2, dUc));
  const ff dv_dn = ff_add(ff_mul(g1, ff_sub(fv[B], fv[A])), ff_mul(g2, dVc));
  const ff dT_dn = ff_add(ff_mul(g1, ff_sub(fT[B], fT[A])), ff_mul(g2, dTc));
  ff du_dt = ff_mul(dUc, il), dv_dt = ff_mul(dVc, il);
  if (!LR) {
    du_dt = ff_neg(du_dt);
    dv_dt = ff_neg(dv_dt);
  }
  const ff Dn = ff_add(ff_mul(du_dn, nx), ff_mul(dv_dn, ny));
  const ff En = ff_add(ff_mul(du_dt, nx), ff_mul(dv_dt, ny));
  const ff Et = ff_sub(ff_mul(du_dt, ny), ff_mul(dv_dt, nx));
  ff div = LR ? ff_sub(Et, Dn) : ff_add(Et, Dn);
  ff uf{0.f, 0.f}, rx{0.f, 0.f};
  if (AXI) {
    rx = ff_from_double(rxd);
    uf = ff_scale2(ff_add(fu[B], fu[A]), 0.5f);
    div = ff_add(div, ff_mul(uf, rx));
  }
  const ff c23 = *reinterpret_cast<const ff*>(&c23f);
  const ff al = ff_add(ff_mul(LR ? c23 : ff_neg(c23), div), Dn);
  const ff Ey = ff_mul(En, ny), Ex = ff_mul(En, nx);
  txf = ff_add(ff_mul(al, nx), LR ? ff_sub(du_dn, Ey) : ff_add(du_dn, Ey));
  tyf = ff_add(ff_mul(al, ny), LR ? ff_add(dv_dn, Ex) : ff_sub(dv_dn, Ex));
  qf = ff_mul(*reinterpret_cast<const ff*>(&kprf), dT_dn);
  if (AXI) hoop = ff_add(ff_mul(ff_neg(c23), div), ff_mul(ff_scale2(uf, 2.f), rx));
}

// The flux of one face with the viscous terms in float-float (the RK step's form). A, B:
// the halo cells left / right (lr face, LR) or bottom / top (bt face); lo, hi: the corner
// sums at its ends; gA: the FP64 planes nx A/2, ny A/2; pl: the float-float planes (the
// five of visc_face_ff, then A/2). Writes the four fluxes (stride fs) of the FP64 form in
// flux_tile, i.e. (Vn (S) + p n + s t) A/2 with s = 1 (lr) or -1 (bt) and the energy's
// s (w + qn) A/2, and for the axisymmetric the hoop term mu_f hoop / 2. The inviscid parts
// are FP64 with the area folded into n; the traction, the heat flux and the work term
// w = (S_u tx + S_v ty) / S_rho are scaled by s A/2 (and mu_f) in float-float and join the
// FP64 sums through one addition each.
template <bool LR, bool AXI, bool SUTH>
__device__ __forceinline__ void face_flux_ff(const FluxArgs& a, const double* s_r, const double* s_ru,
                                             const double* s_rv, const double* s_rE, const double* s_p, const ff* fu,
                                             const ff* fv, const ff* fT, const ff* fuc, const ff* fvc, const ff* fTc,
                                             int A, int B, int lo, int hi, const double* gA, const float2* pl, long NF,
                                             long f, double rxd, double* out, int fs, double* hoop_out) {
  const double Sr = s_r[A] + s_r[B], Su = s_ru[A] + s_ru[B], Sv = s_rv[A] + s_rv[B];
  const double SE = s_rE[A] + s_rE[B], Sp = s_p[A] + s_p[B];
  const double ir = frcp(Sr);
  const double nxA = gA[f], nyA = gA[NF + f];
  const double m2A = fma(Su, nxA, Sv * nyA);  // (S_u nx + S_v ny) A/2
  const double VnA = m2A * ir;
  ff txf, tyf, qf, hpf;
  visc_face_ff<LR, AXI>(fu, fv, fT, A, B, fuc, fvc, fTc, lo, hi, pl, NF, f, rxd, a.kprf, a.c23f, txf, tyf, qf, hpf);
  ff fac = *reinterpret_cast<const ff*>(pl + 5 * NF + f);
  if (!LR) fac = ff_neg(fac);
  ff muf{1.f, 0.f};
  if (SUTH) {  // Sutherland at the face temperature
    const double Ts = (ff_to_double(fT[A]) + ff_to_double(fT[B])) * 0.5 * a.Tinf_inv;
    muf = ff_from_double(Ts * sqrt(Ts) * (1 + a.suthS) * frcp(Ts + a.suthS));
    fac = ff_mul(fac, muf);
  }
  const ff txA = ff_mul(txf, fac), tyA = ff_mul(tyf, fac);
  const ff wA = ff_mul(ff_add(ff_mul(ff_from_double(Su), txA), ff_mul(ff_from_double(Sv), tyA)), ff_from_double(ir));
  const ff wqA = ff_add(wA, ff_mul(qf, fac));
  out[0] = m2A;
  out[fs] = fma(Su, VnA, fma(Sp, nxA, ff_to_double(txA)));
  out[2 * fs] = fma(Sv, VnA, fma(Sp, nyA, ff_to_double(tyA)));
  out[3 * fs] = fma(SE + Sp, VnA, ff_to_double(wqA));
  if (AXI) *hoop_out = ff_to_double(ff_scale2(SUTH ? ff_mul(hpf, muf) : hpf, 0.5f));
}

// Returns false when a TMA wait gave up (the block then stops).
template <bool AXI, bool SUTH, int TYV, bool FFV, bool TMA>
__device__ __forceinline__ bool flux_tile(const FluxArgs& a, const FluxMaps& tm, int bx, int by, double* sm,
                                          uint64_t* bar, unsigned& phase) {
  using G = TileGeo<TYV, TMA>;
  // halo planes; with TMA the first six are the staged copies of the ghosted planes
  double* s_r = sm;
  double* s_ru = s_r + G::PS;
  double* s_rv = s_ru + G::PS;
  double* s_rE = s_rv + G::PS;
  double* s_p = s_rE + G::PS;
  double* s_T = s_p + G::PS;
  double* s_u = s_T + G::PS;   // u = rho_u / rho
  double* s_v = s_u + G::PS;
  double* s_uc = s_v + G::PS;
  double* s_vc = s_uc + G::NCOR;
  double* s_Tc = s_vc + G::NCOR;
  // the lr faces stay in registers (a row's faces are one warp's lanes: a cell's east face
  // is the next lane's west face); the bottom/top faces cross warps and go through here
  double* f_bt = s_Tc + G::NCOR;                // 4 x G::NBTF
  double* t_bt = f_bt + 4 * G::NBTF;            // AXI hoop stress on bt faces
  // the float-float variant keeps u, v, T and the corner sums as float-float pairs in the
  // same shared slots (8 bytes per entry either way)
  ff* fu = reinterpret_cast<ff*>(s_u);
  ff* fv = reinterpret_cast<ff*>(s_v);
  ff* fT = reinterpret_cast<ff*>(s_T);
  ff* fuc = reinterpret_cast<ff*>(s_uc);
  ff* fvc = reinterpret_cast<ff*>(s_vc);
  ff* fTc = reinterpret_cast<ff*>(s_Tc);

  const int nchi = a.nchi, neta = a.neta;
  const int i0 = bx * TX, j0 = by * TYV;  // first interior cell (0-based)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // shared index of halo cell (hx, hy) = ghosted (i0 + hx, j0 + hy); with TMA the staged rows
  // start at the even column i0 - (i0 & 1)
  const int xo = TMA ? (i0 & 1) : 0;
  auto hid = [&](int hx, int hy) { return hx + xo + hy * G::HP; };

  if (a.tile_class >= 0 && !a.list) {
    // the halo (ghosted columns i0..i0+TX+1, rows j0..j0+TYV+1) avoids every ghost cell and
    // stays below the shocked rows sc..sc+2 of its columns -> independent of shock/BC work
    bool inner = i0 >= 1 && i0 + TX + 1 <= nchi && j0 >= 1 && j0 + TYV + 1 <= neta;
    if (a.shock) {
      int scmin = 0x7fffffff;
      for (int c = lane; c < TX + 2; c += 32) {
        const int col = i0 - 1 + c;  // interior column of halo column
        if (col >= 0 && col < nchi) scmin = min(scmin, a.cell_idx[col]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) scmin = min(scmin, __shfl_xor_sync(0xffffffffu, scmin, o));
      inner = inner && (j0 + TYV + 1 < scmin);
    }
    if (inner != (a.tile_class == 0)) return true;
  }

  // whole tile at or above the shocked rows: flux is zero (NON_LINEAR_DYNAMICS mask)
  if (a.mask) {
    int sc = 0;
    if (lane < TX && i0 + lane < nchi) sc = a.cell_idx[i0 + lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sc = max(sc, __shfl_xor_sync(0xffffffffu, sc, o));
    if (j0 + 1 >= sc) {
      const int ci = i0 + lane, cj = j0 + warp;
      if (lane < TX && ci < nchi && cj < neta) {
        const long c = (long)ci + (long)cj * nchi;
        a.o0[c] = 0; a.o1[c] = 0; a.o2[c] = 0; a.o3[c] = 0;
      }
      return true;
    }
  }

  if (TMA) {
    // (1a) the six halo planes by TMA: boxes of 36 x (TYV + 2) doubles from the even column
    // i0 - xo and row j0 (cells past the ghost layer read as zero and are never used)
    if (tid == 0) {
      const unsigned b = smem_u32(bar);
      // earlier generic-proxy reads of these buffers come before the async-proxy writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                   "r"((unsigned)(6 * G::HP * (TYV + 2) * sizeof(double)))
                   : "memory");
      double* dst[6] = {s_r, s_ru, s_rv, s_rE, s_p, s_T};
#pragma unroll
      for (int q = 0; q < 6; ++q)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
            "[%4];" ::"r"(smem_u32(dst[q])),
            "l"(&tm.m[q]), "r"(i0 - xo), "r"(j0), "r"(b)
            : "memory");
    }
    const bool ok = mbar_wait(smem_u32(bar), phase);
    phase ^= 1u;
    if (!__syncthreads_and(ok)) {
      if (tid == 0) atomicOr(a.err, kBitTimeout);
      return false;
    }
  }
  // (1) halo cells: ghosted (i0 + hx, j0 + hy)
  for (int h0 = tid; h0 < G::NH; h0 += G::THREADS) {
    const int hx = h0 % HX, hy = h0 / HX;
    const int h = hid(hx, hy);
    const int gi = i0 + hx, gj = j0 + hy;
    if (gi <= nchi + 1 && gj <= neta + 1) {
      double r, ru, rv, T;
      if (TMA) {
        r = s_r[h]; ru = s_ru[h]; rv = s_rv[h]; T = s_T[h];
      } else {
        const long g = (long)gi + (long)gj * (nchi + 2);
        r = a.rho[g]; ru = a.ru[g]; rv = a.rv[g];
        s_r[h] = r; s_ru[h] = ru; s_rv[h] = rv; s_rE[h] = a.rE[g];
        s_p[h] = a.p[g];
        T = a.T[g];
      }
      if (FFV) {  // u, v as float-float quotients: no FP64 work per halo cell
        const ff iv = ff_rcp(ff_from_double(r));
        fu[h] = ff_mul(ff_from_double(ru), iv);
        fv[h] = ff_mul(ff_from_double(rv), iv);
        fT[h] = ff_from_double(T);
      } else {
        const double ir = frcp(r);
        s_u[h] = ru * ir; s_v[h] = rv * ir;
        s_T[h] = T;
      }
    }
  }
  __syncthreads();
  // (2) corner averages (VISCOUS_FLUX.jl:67-70, 184-185)
  for (int cidx = tid; cidx < G::NCOR; cidx += G::THREADS) {
    const int cx = cidx % CX, cy = cidx / CX;
    if (i0 + cx <= nchi && j0 + cy <= neta) {
      const int h00 = hid(cx, cy), h10 = h00 + 1, h01 = h00 + G::HP, h11 = h01 + 1;
      // four times the corner averages: the 1/4 is folded into the g2/h2 and 1/len planes
      if (FFV) {
        fuc[cidx] = ff_add(ff_add(fu[h00], fu[h10]), ff_add(fu[h01], fu[h11]));
        fvc[cidx] = ff_add(ff_add(fv[h00], fv[h10]), ff_add(fv[h01], fv[h11]));
        fTc[cidx] = ff_add(ff_add(fT[h00], fT[h10]), ff_add(fT[h01], fT[h11]));
      } else {
        s_uc[cidx] = s_u[h00] + s_u[h10] + s_u[h01] + s_u[h11];
        s_vc[cidx] = s_v[h00] + s_v[h10] + s_v[h01] + s_v[h11];
        s_Tc[cidx] = s_T[h00] + s_T[h10] + s_T[h01] + s_T[h11];
      }
    }
  }
  __syncthreads();
  const long NLR = (long)(nchi + 1) * neta, NBT = (long)nchi * (neta + 1);
  // (3a) lr faces: warp = tile row fy, lane = fx (32 faces per row), into registers
  double fl[4] = {0.0, 0.0, 0.0, 0.0}, tl = 0.0;
  {
    const int fx = lane, fy = warp;
    const int gi = i0 + fx, gj = j0 + fy;  // face (gi, gj) 0-based: between ghosted (gi, gj+1), (gi+1, gj+1)
    if (FFV && gi <= nchi && gj < neta) {
      const long f = (long)gi + (long)gj * (nchi + 1);
      const int L = hid(fx, fy + 1);
      face_flux_ff<true, AXI, SUTH>(a, s_r, s_ru, s_rv, s_rE, s_p, fu, fv, fT, fuc, fvc, fTc, L, L + 1,
                                    fx + fy * CX, fx + fy * CX + CX, a.m.lra, a.m.lrf, NLR, f,
                                    AXI ? a.m.rx_lr[f] : 0.0, fl, 1, &tl);
    } else if (gi <= nchi && gj < neta) {
      const long f = (long)gi + (long)gj * (nchi + 1);
      const double nx = a.m.lrg[f], ny = a.m.lrg[NLR + f], Ah = a.m.lrg[2 * NLR + f];
      const int L = hid(fx, fy + 1), R = L + 1;
      const int clo = fx + fy * CX, chi_ = clo + CX;
      const double Sr = s_r[L] + s_r[R], Su = s_ru[L] + s_ru[R], Sv = s_rv[L] + s_rv[R];
      const double SE = s_rE[L] + s_rE[R], Sp = s_p[L] + s_p[R];
      const double ir = frcp(Sr);
      const double m2 = fma(Su, nx, Sv * ny);
      const double Vn = m2 * ir;
      double tx, ty, qn, hoop = 0, mu_f = 1;
      {
        const double g1 = a.m.lrg[3 * NLR + f], g2 = a.m.lrg[4 * NLR + f], il = a.m.lrg[5 * NLR + f];
        // viscous (VISCOUS_FLUX.jl:98-133)
        const double dUc = s_uc[chi_] - s_uc[clo], dVc = s_vc[chi_] - s_vc[clo], dTc = s_Tc[chi_] - s_Tc[clo];
        const double du_dn = fma(g1, s_u[R] - s_u[L], g2 * dUc);
        const double dv_dn = fma(g1, s_v[R] - s_v[L], g2 * dVc);
        const double dT_dn = fma(g1, s_T[R] - s_T[L], g2 * dTc);
        const double du_dt = dUc * il, dv_dt = dVc * il;
        // With D = (du_dn, dv_dn), E = (du_dt, dv_dt), n and t = (ny, -nx) the face frame of
        // VISCOUS_FLUX.jl:98-133 has dun_dn = -D.n, dut_dn = D.t, dun_dt = -E.n, dut_dt = E.t,
        // and the traction t = -tau11 n + tau12 t with tau11 = mu (2 dun_dn - 2/3 div),
        // tau12 = mu (dun_dt + dut_dn) is, expanding D in the (n, t) basis,
        //   t = mu (D + (D.n + 2/3 div) n - (E.n) t),   div = E.t - D.n (+ u/x axisymmetric)
        const double Dn = fma(du_dn, nx, dv_dn * ny);
        const double En = fma(du_dt, nx, dv_dt * ny);
        const double Et = fma(du_dt, ny, -dv_dt * nx);
        double div = Et - Dn;
        double kpr = a.kpr;  // gamma / Pr: the heat flux from the 2/Re-scaled temperature gradient
        if (SUTH) {  // Sutherland at the face temperature
          const double Ts = (s_T[L] + s_T[R]) * 0.5 * a.Tinf_inv;
          mu_f = Ts * sqrt(Ts) * (1 + a.suthS) * frcp(Ts + a.suthS);
          kpr *= mu_f;
        }
        double uf = 0, rx = 0;
        if (AXI) {
          rx = a.m.rx_lr[f];
          uf = (s_u[R] + s_u[L]) * 0.5;
          div = fma(uf, rx, div);
        }
        // twice the traction, the work and the heat flux: (2 t) (A/2) = t A
        const double al = fma(2.0 / 3.0, div, Dn);
        tx = fma(al, nx, fma(-En, ny, du_dn));
        ty = fma(al, ny, fma(En, nx, dv_dn));
        if (SUTH) { tx *= mu_f; ty *= mu_f; }
        qn = kpr * dT_dn;
        if (AXI) hoop = fma(-2.0 / 3.0, div, 2 * uf * rx);
      }
      const double w = fma(Su, tx, Sv * ty) * ir;
      fl[0] = m2 * Ah;
      fl[1] = fma(Su, Vn, fma(Sp, nx, tx)) * Ah;
      fl[2] = fma(Sv, Vn, fma(Sp, ny, ty)) * Ah;
      fl[3] = fma(SE + Sp, Vn, w + qn) * Ah;
      if (AXI) tl = (0.5 * mu_f) * hoop;
    }
  }
  // west minus east face of the lane's cell (the last lane's value is unused: TX = 31)
  double dl[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) dl[k] = fl[k] - __shfl_down_sync(0xffffffffu, fl[k], 1);
  const double tls = AXI ? tl + __shfl_down_sync(0xffffffffu, tl, 1) : 0.0;
  // (3b) bt faces: TX x (TYV + 1)
  for (int b = tid; b < (TX + 1) * (TYV + 1); b += G::THREADS) {
    const int fx = b & 31, fy = b >> 5;
    if (fx >= TX) continue;
    const int gi = i0 + fx, gj = j0 + fy;  // face (gi, gj): between ghosted (gi+1, gj), (gi+1, gj+1)
    const int o = fx + fy * TX;
    if (FFV && gi < nchi && gj <= neta) {
      const long f = (long)gi + (long)gj * nchi;
      const int B = hid(fx + 1, fy);
      face_flux_ff<false, AXI, SUTH>(a, s_r, s_ru, s_rv, s_rE, s_p, fu, fv, fT, fuc, fvc, fTc, B, B + G::HP,
                                     fx + fy * CX, fx + fy * CX + 1, a.m.bta, a.m.btf, NBT, f,
                                     AXI ? a.m.rx_bt[f] : 0.0, f_bt + o, G::NBTF, t_bt + o);
    } else if (gi < nchi && gj <= neta) {
      const long f = (long)gi + (long)gj * nchi;
      const double nx = a.m.btg[f], ny = a.m.btg[NBT + f], Ah = a.m.btg[2 * NBT + f];
      const int B = hid(fx + 1, fy), Tt = B + G::HP;
      const int clo = fx + fy * CX, chi_ = clo + 1;
      const double Sr = s_r[B] + s_r[Tt], Su = s_ru[B] + s_ru[Tt], Sv = s_rv[B] + s_rv[Tt];
      const double SE = s_rE[B] + s_rE[Tt], Sp = s_p[B] + s_p[Tt];
      const double ir = frcp(Sr);
      const double m2 = fma(Su, nx, Sv * ny);
      const double Vn = m2 * ir;
      double tx, ty, qn, hoop = 0, mu_f = 1;
      {
        const double h1 = a.m.btg[3 * NBT + f], h2 = a.m.btg[4 * NBT + f], il = a.m.btg[5 * NBT + f];
        const double dUc = s_uc[chi_] - s_uc[clo], dVc = s_vc[chi_] - s_vc[clo], dTc = s_Tc[chi_] - s_Tc[clo];
        const double du_dn = fma(h1, s_u[Tt] - s_u[B], h2 * dUc);
        const double dv_dn = fma(h1, s_v[Tt] - s_v[B], h2 * dVc);
        const double dT_dn = fma(h1, s_T[Tt] - s_T[B], h2 * dTc);
        const double du_dt = -dUc * il, dv_dt = -dVc * il;
        // bt frame: dun_dn = D.n, dut_dn = D.t, dun_dt = E.n, dut_dt = E.t, traction
        // tau22 n + tau21 t = mu (D + (D.n - 2/3 div) n + (E.n) t), div = E.t + D.n
        const double Dn = fma(du_dn, nx, dv_dn * ny);
        const double En = fma(du_dt, nx, dv_dt * ny);
        const double Et = fma(du_dt, ny, -dv_dt * nx);
        double div = Et + Dn;
        double kpr = a.kpr;
        if (SUTH) {
          const double Ts = (s_T[B] + s_T[Tt]) * 0.5 * a.Tinf_inv;
          mu_f = Ts * sqrt(Ts) * (1 + a.suthS) * frcp(Ts + a.suthS);
          kpr *= mu_f;
        }
        double uf = 0, rx = 0;
        if (AXI) {
          rx = a.m.rx_bt[f];
          uf = (s_u[Tt] + s_u[B]) * 0.5;
          div = fma(uf, rx, div);
        }
        const double al = fma(-2.0 / 3.0, div, Dn);
        tx = fma(al, nx, fma(En, ny, du_dn));
        ty = fma(al, ny, fma(-En, nx, dv_dn));
        if (SUTH) { tx *= mu_f; ty *= mu_f; }
        qn = kpr * dT_dn;
        if (AXI) hoop = fma(-2.0 / 3.0, div, 2 * uf * rx);
      }
      const double w = fma(Su, tx, Sv * ty) * ir;
      f_bt[o] = m2 * Ah;
      f_bt[G::NBTF + o] = fma(Su, Vn, fma(Sp, nx, -tx)) * Ah;
      f_bt[2 * G::NBTF + o] = fma(Sv, Vn, fma(Sp, ny, -ty)) * Ah;
      f_bt[3 * G::NBTF + o] = fma(SE + Sp, Vn, -(w + qn)) * Ah;
      if (AXI) t_bt[o] = (0.5 * mu_f) * hoop;
    }
  }
  __syncthreads();
  // (4) cells: warp = tile row, lane = column
  {
    const int cx = lane, cy = warp;
    const int ci = i0 + cx, cj = j0 + cy;
    if (cx < TX && ci < nchi && cj < neta) {
      const long c = (long)ci + (long)cj * nchi;
      double r0 = 0, r1 = 0, r2 = 0, r3 = 0;
      const bool active = !a.mask || (cj + 1 < a.cell_idx[ci]);
      if (active) {
        const int s = cx + cy * TX, n = s + TX;
        const double rv = a.m.rvol[c];
        r0 = (dl[0] + f_bt[s] - f_bt[n]) * rv;
        r1 = (dl[1] + f_bt[G::NBTF + s] - f_bt[G::NBTF + n]) * rv;
        double v2 = dl[2] + f_bt[2 * G::NBTF + s] - f_bt[2 * G::NBTF + n];
        if (AXI) {
          // FLUX_MOMENTUM_3D.jl:120-122: front/back pressure with sign(y) of the cell centre
          const double pc = s_p[hid(cx + 1, cy + 1)];
          const double ycell = a.m.y_ext[(long)(ci + 1) + (long)(cj + 1) * (nchi + 2)];
          v2 += (pc * a.m.fb_yn_front - pc * a.m.fb_yn_back) * a.m.fb_area[c] * jsign(ycell);
          // VISCOUS_FLUX_3D.jl:154-177: hoop stress, radius = x of the cell centre
          const double tth = (tls + t_bt[s] + t_bt[n]) * 0.25;
          const double xcell = a.m.x_ext[(long)(ci + 1) + (long)(cj + 1) * (nchi + 2)];
          r1 -= tth * frcp(xcell);
        }
        r2 = v2 * rv;
        r3 = (dl[3] + f_bt[3 * G::NBTF + s] - f_bt[3 * G::NBTF + n]) * rv;
      }
      a.o0[c] = r0; a.o1[c] = r1; a.o2[c] = r2; a.o3[c] = r3;
    }
  }
  return true;
}

// The 2-D constant-viscosity 31 x 4 kernel is held to 56 registers for nine resident blocks
// per SM (its shared memory allows ten), so that the persistent interior grid of the split
// tiling keeps eight beside a spare slot; the others to 64.
template <bool AXI, bool SUTH, int TYV>
constexpr int flux_min_blocks() { return TYV == 4 && !AXI && !SUTH ? 9 : 32 / TYV; }

// Tile grid (no list), or a persistent grid striding over the compact tile list of a class.
template <bool AXI, bool SUTH, int TYV, bool FFV, bool TMA>
__global__ void __launch_bounds__(32 * TYV, flux_min_blocks<AXI, SUTH, TYV>())
    k_flux(FluxArgs a, const __grid_constant__ FluxMaps tm) {
  extern __shared__ double sm_raw[];
  __shared__ uint64_t bar;  // completion of the halo TMA transfers of a tile
  // TMA destinations start on a 128-byte boundary (128 bytes of slack in the launch's size)
  double* sm = TMA ? reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(sm_raw) + 127) & ~uintptr_t(127)) : sm_raw;
  unsigned phase = 0;
  if (TMA) {
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
  }
  if (!a.list) {
    flux_tile<AXI, SUTH, TYV, FFV, TMA>(a, tm, blockIdx.x, blockIdx.y, sm, &bar, phase);
    return;
  }
  const int n = *a.count;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int t = a.list[k];
    if (!flux_tile<AXI, SUTH, TYV, FFV, TMA>(a, tm, t % a.tiles_x, t / a.tiles_x, sm, &bar, phase)) return;
    __syncthreads();  // the next tile reuses the shared arrays
  }
}

template <bool AXI, bool SUTH, int TYV = TY, bool TMA = false>
size_t flux_smem() {
  using G = TileGeo<TYV, TMA>;
  return sizeof(double) * (8 * G::PS + 3 * G::NCOR + 4 * G::NBTF + (AXI ? G::NBTF : 0)) +
         (TMA ? 128 : 0);
}

// ---------------------------------------------------------------------------
// UPDATE_FLOW_CELLS on S: DETECT_CELLS_SHOCKED (DETECT_CELLS_SHOCKED.jl:50-65),
// UPDATE_FIELD_UPSTREAM (UPDATE_FIELD_UPSTREAM.jl:93-109), EXTRAPOLATE_CELLS_SHOCK.
// x as a float with its mantissa truncated to 23 bits, from the bit pattern; zero below the
// float normal range; sets bad beyond it (and for infinities and NaN).
__device__ __forceinline__ float trunc_float(double x, bool& bad) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const unsigned e = (hw >> 20) & 0x7ffu;
  bad |= e >= 1151u;
  const unsigned fb = (hw & 0x80000000u) | ((e - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  return e > 896u ? __uint_as_float(fb) : 0.0f;
}

// EXTRAPOLATE_CELLS_SHOCK above the shocked cell sc of column i: rows sc + 1, sc + 2 of
// variable v (the 3rd-order form with each operation rounded, the reference's association)
__device__ void extrapolate_column(const hymor_config& c, Cons q, int i, int sc, int v) {
  const int nchi = c.nchi, I = i + 1;
  const int g0 = gidx(I, sc, nchi), i1 = gidx(I, sc + 1, nchi), i2 = gidx(I, sc + 2, nchi);
  const int im1 = gidx(I, sc - 1, nchi), im2 = gidx(I, sc - 2, nchi);
  double* a = v == 0 ? q.rho : (v == 1 ? q.ru : (v == 2 ? q.rv : q.rE));
  if (c.shock_interp == 1) {
    a[i1] = a[g0];
    a[i2] = a[g0];
  } else if (c.shock_interp == 2) {
    const double e1 = 2 * a[g0] - a[im1];
    a[i1] = e1;
    a[i2] = 2 * e1 - a[g0];
  } else {
    auto cubic = [](double x, double y, double z) {
      return __dadd_rn(__dsub_rn(__dmul_rn(3.0, x), __dmul_rn(3.0, y)), z);
    };
    const double e1 = cubic(a[g0], a[im1], a[im2]);
    a[i1] = e1;
    a[i2] = cubic(e1, a[g0], a[im1]);
  }
}

struct FlowArgs {
  hymor_config cfg;
  DevMesh m;
  Cons S;
  ShockPts pS;
  int* cell_idx;
  const double* scal;
  unsigned* err;
  int disturbed;  // any freestream disturbance amplitude non-zero (set on the host)
};

// The nearest cell centre of a column is found by an FP32 screen: every row's squared
// distance in FP32 from the truncated coordinates, with a bound E on its error against the
// exact value, and the FP64 distance (rounded like the reference's unfused dx^2 + dy^2) only
// for the rows whose interval [d - E, d + E] reaches below the smallest d + E. Every row
// attaining the FP64 minimum is among them, so the nearest row and its ties are those of the
// full FP64 scan. Rows whose coordinates are not finite floats are always evaluated in FP64.
struct NearScreen {
  float px, py;
  bool bad;
};

// lower (lo) and upper (hi) bounds of the squared distance of the row's centre (x, y)
__device__ __forceinline__ void near_bounds(const NearScreen& s, double x, double y, float& lo, float& hi) {
  bool bad = s.bad;
  const float xf = trunc_float(x, bad), yf = trunc_float(y, bad);
  const float dx = s.px - xf, dy = s.py - yf;
  const float d = dx * dx + dy * dy;
  // |dx - (X - C)| <= 2^-23 (|X| + |C|) + 2^-24 |x - c| (truncation and the subtraction),
  // taken twice over, plus the float normal range's floor
  const float ex = 0x1p-22f * (fabsf(s.px) + fabsf(xf)) + 0x1p-23f * fabsf(dx) + 0x1p-125f;
  const float ey = 0x1p-22f * (fabsf(s.py) + fabsf(yf)) + 0x1p-23f * fabsf(dy) + 0x1p-125f;
  const float e = 2.0f * ((2.0f * fabsf(dx) + ex) * ex + (2.0f * fabsf(dy) + ey) * ey + 0x1p-21f * d) + 0x1p-120f;
  lo = d - e;
  hi = d + e;
  if (bad || !(hi <= 3.0e38f)) { lo = 0.0f; hi = __int_as_float(0x7f800000); }  // always evaluated
}

// one warp per column (two per block, so that the columns spread over every SM)
__global__ void __launch_bounds__(64) k_flow_cells(FlowArgs A) {
  const hymor_config& c = A.cfg;
  const int nchi = c.nchi, neta = c.neta, NJ = neta + 2;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= nchi) return;
  const double px = A.pS.x[i], py = A.pS.y[i];
  // nearest cell centre along the column; ties go to the smallest row, like the
  // reference's sequential scan with a strict comparison (the transposed centres make the
  // loads coalesced)
  const double* xc = A.m.xt + (long)(i + 1) * NJ;
  const double* yc = A.m.yt + (long)(i + 1) * NJ;
  NearScreen scr;
  scr.bad = false;
  scr.px = trunc_float(px, scr.bad);
  scr.py = trunc_float(py, scr.bad);
  float top = __int_as_float(0x7f800000);
#pragma unroll 4
  for (int j = 1 + lane; j <= neta; j += 32) {
    float lo, hi;
    near_bounds(scr, xc[j], yc[j], lo, hi);
    top = fminf(top, hi);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) top = fminf(top, __shfl_xor_sync(0xffffffffu, top, o));
  // the FP64 distances of the candidates; non-negative doubles order as their bit patterns
  unsigned long long best = 0x7ff0000000000000ull;  // +inf
  int bj = 0x7fffffff;
#pragma unroll 4
  for (int j = 1 + lane; j <= neta; j += 32) {
    const double x = xc[j], y = yc[j];
    float lo, hi;
    near_bounds(scr, x, y, lo, hi);
    if (lo <= top) {
      const double dx = px - x, dy = py - y;
      const double d = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      const unsigned long long db = (unsigned long long)__double_as_longlong(d);
      if (db < best) { best = db; bj = j; }  // NaN (above +inf) never wins, like d < best
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (ob < best || (ob == best && oj < bj)) { best = ob; bj = oj; }
  }
  if (bj == 0x7fffffff) bj = 1;
  if (lane == 0) A.cell_idx[i] = bj;
  if (bj < 2 || bj > neta - 1) {
    if (lane == 0) atomicOr(&A.err[kErrFlags], kBitShockRange);
    return;
  }
  // UPDATE_FIELD_UPSTREAM: ghosted rows >= sc + 2 of this column
  const double t = A.scal[kT];
  const bool dist = A.disturbed;
  double u_y = 0, u_x = 0;
  if (dist) { u_y = c.rho_v_0 / c.rho_0; u_x = c.rho_u_0 / c.rho_0; }
  for (int jg = bj + 2 + lane; jg < NJ; jg += 32) {
    const long k = gidx(i + 1, jg, nchi);
    if (dist) {
      const double pert =
          cos(2.0 * M_PI * c.dist_ky * (A.m.y_ext[k] - u_y * t)) * sin(2.0 * M_PI * c.dist_kx * (A.m.x_ext[k] - u_x * t));
      A.S.rho[k] = c.rho_0 + pert * c.dist_amp[0];
      A.S.ru[k] = c.rho_u_0 + pert * c.dist_amp[1];
      A.S.rv[k] = c.rho_v_0 + pert * c.dist_amp[2];
      A.S.rE[k] = c.rho_E_0 + pert * c.dist_amp[3];
    } else {
      A.S.rho[k] = c.rho_0; A.S.ru[k] = c.rho_u_0; A.S.rv[k] = c.rho_v_0; A.S.rE[k] = c.rho_E_0;
    }
  }
  __syncwarp();
  if (lane < 4) extrapolate_column(c, A.S, i, bj, lane);
}

// Sound speed of S, max |a| over every ghosted cell (CFL_TIMESTEP.jl:80).
//   mode 0: max over the stored sound speed
//   mode 1: recompute a = sqrt(gamma p / rho) everywhere, and its max
//   mode 2: the max only, as sqrt(max gamma p / rho) (sqrt is monotone and correctly
//           rounded, so this is the max of the square roots exactly), storing a only on
//           the lines the outflow_NRCBC condition reads; the last block takes the root
struct SoundArgs {
  Cons S;
  double* aS;
  double* scal;
  unsigned* ticket;  // blocks done (mode 2), reset by the last one
  double gamma;
  int nchi, neta, mode, isothermal_eta0, nrcbc;
};

// gamma p / rho of ghosted cell k = (i, j) of S; the isothermal wall's ghost row takes the
// pressure extrapolated from the first two rows (UPDATE_THERMODYNAMIC_PROPERTIES.jl:28-31)
__device__ __forceinline__ double cell_c2(const SoundArgs& A, long k, int i, int j) {
  const double gm1 = A.gamma - 1;
  auto pres_r = [&](long q, double ir) {
    const double u = A.S.ru[q], v = A.S.rv[q], e = A.S.rE[q];
    return fma(-0.5, fma(u, u, v * v) * ir, e) * gm1;
  };
  auto pres = [&](long q) { return pres_r(q, frcp(A.S.rho[q])); };
  double p;
  const double ir = frcp(A.S.rho[k]);
  if (j == 0 && A.isothermal_eta0)
    p = 2 * pres(gidx(i, 1, A.nchi)) - pres(gidx(i, 2, A.nchi));
  else
    p = pres_r(k, ir);
  return A.gamma * p * ir;
}

__global__ void __launch_bounds__(256) k_sound_cmax(SoundArgs A) {
  const int NI = A.nchi + 2, NJ = A.neta + 2;
  const long G = (long)NI * NJ;
  double mx = 0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < G; k += (long)gridDim.x * blockDim.x) {
    if (A.mode == 0) {
      mx = fmax(mx, fabs(A.aS[k]));
      continue;
    }
    const int i = (int)((unsigned)k % (unsigned)NI), j = (int)((unsigned)k / (unsigned)NI);
    const double c2 = cell_c2(A, k, i, j);
    if (A.mode == 1) {
      const double a = sqrt(c2);
      A.aS[k] = a;
      mx = fmax(mx, fabs(a));
    } else {
      const bool nb = ((A.nrcbc & 1) && i == 1) || ((A.nrcbc & 2) && i == NI - 2) ||
                      ((A.nrcbc & 4) && j == 1) || ((A.nrcbc & 8) && j == NJ - 2);
      if (nb) A.aS[k] = sqrt(c2);
      mx = fmax(mx, c2);
    }
  }
  mx = warp_max(mx);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_max(v);
    if (threadIdx.x == 0) {
      atomic_max_nonneg(&A.scal[kCmax], v);
      if (A.mode == 2) {
        __threadfence();
        if (atomicAdd(A.ticket, 1u) == gridDim.x - 1) {  // every block's maximum is in
          unsigned long long* bits = reinterpret_cast<unsigned long long*>(&A.scal[kCmax]);
          const double c2max = __longlong_as_double((long long)atomicAdd(bits, 0ull));
          A.scal[kCmax] = sqrt(c2max);
          *A.ticket = 0;
        }
      }
    }
  }
}

// CFL maxima (CFL_TIMESTEP.jl:80-130) and dt. k_cfl_faces evaluates the convective
// face rate (|V_n| + c) A once per face; k_cfl takes, per cell, the max over opposite
// faces, adds the viscous rate 2 max(4/3, gamma/Pr) (A_xi^2 + A_eta^2) / (rho Re_flow vol)
// (the mesh factor 2 (A_xi^2 + A_eta^2) / vol is precomputed), divides by the volume and
// reduces the maxima of the rates and of the stored-flux terms of dt2.
struct CflArgs {
  Cons S;
  const double* SF0;
  const double* SF1;
  const double* SF2;
  const double* SF3;
  DevMesh m;
  const int* cell_idx;
  double* scal;
  double* lam_lr;   // face rates, lr then bt
  double* lam_bt;
  double gamma, suthS, Tinf_inv;
  int nchi, neta, shock, suth;
  int sf_zero;      // the stored flux is zero everywhere: its dt term is +inf, skip it
};

// Convective rate (|V_n| + c_max) A of the face between ghosted cells L and R of S.
__device__ __forceinline__ double face_rate(const Cons& S, long L, long R, double nx, double ny, double Af,
                                            double cmax) {
  const double rs = S.rho[L] + S.rho[R];
  const double Vn = fabs(fma(S.ru[L] + S.ru[R], nx, (S.rv[L] + S.rv[R]) * ny)) * frcp(rs);
  return (Vn + cmax) * Af;
}

// CFL rate of interior cell c (ghosted g, ir = 1 / rho) from its west, east, south and
// north face rates: the larger of opposite faces, summed, over the volume, plus the viscous
// rate 2 max(4/3, gamma/Pr) (A_xi^2 + A_eta^2) / (rho Re_flow vol^2).
__device__ __forceinline__ double cell_rate(const CflArgs& A, long c, long g, double lw, double le, double ls,
                                            double ln, double ir) {
  const double lam_c = fmax(lw, le) + fmax(ls, ln);
  // viscous rate over the volume: gvis carries max(4/3, gamma/Pr) / Re and 1/vol^2
  double lam_v = A.m.gvis[c] * ir;
  if (A.suth) {  // Re_flow = Re / mu* (UPDATE_CHEMISTRY_EQUILIBRIUM.jl:99-101); mu* = 1 for CPG
    const double e = fma(-0.5, fma(A.S.ru[g], A.S.ru[g], A.S.rv[g] * A.S.rv[g]) * ir, A.S.rE[g]) * ir;
    const double Ts = e * A.Tinf_inv;
    lam_v *= Ts * sqrt(Ts) * (1 + A.suthS) * frcp(Ts + A.suthS);
  }
  return fma(lam_c, A.m.rvol[c], lam_v);
}

__global__ void __launch_bounds__(256) k_cfl_faces(CflArgs A) {
  const int nchi = A.nchi, neta = A.neta;
  const long NLR = (long)(nchi + 1) * neta, NBT = (long)nchi * (neta + 1);
  const double cmax = A.scal[kCmax];
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < NLR + NBT; f += (long)gridDim.x * blockDim.x) {
    long L, R;
    double nx, ny, Af;
    if (f < NLR) {
      const int i = (int)(f % (nchi + 1)), j = (int)(f / (nchi + 1));
      L = gidx(i, j + 1, nchi);
      R = L + 1;
      // the flux kernel's geometry planes (n_x, n_y, A/2), one copy of the face data
      nx = A.m.lrg[f]; ny = A.m.lrg[NLR + f]; Af = 2 * A.m.lrg[2 * NLR + f];
    } else {
      const long g = f - NLR;
      const int i = (int)(g % nchi), j = (int)(g / nchi);
      L = gidx(i + 1, j, nchi);
      R = L + (nchi + 2);
      nx = A.m.btg[g]; ny = A.m.btg[NBT + g]; Af = 2 * A.m.btg[2 * NBT + g];
    }
    const double lam = face_rate(A.S, L, R, nx, ny, Af, cmax);
    if (f < NLR) A.lam_lr[f] = lam; else A.lam_bt[f - NLR] = lam;
  }
}

__global__ void __launch_bounds__(256) k_cfl(CflArgs A) {
  const int nchi = A.nchi, neta = A.neta;
  const long N = (long)nchi * neta;
  double mlam = 0, mflux = 0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)c % (unsigned)nchi), j = (int)((unsigned)c / (unsigned)nchi);
    const bool flow = !A.shock || (j + 1 < A.cell_idx[i]);
    if (flow) {
      const long fw = i + (long)j * (nchi + 1), fs = i + (long)j * nchi;
      const long g = gidx(i + 1, j + 1, nchi);
      const double ir = frcp(A.S.rho[g]);
      mlam = fmax(mlam, cell_rate(A, c, g, A.lam_lr[fw], A.lam_lr[fw + 1], A.lam_bt[fs], A.lam_bt[fs + nchi], ir));
      if (!A.sf_zero) {
        const double t_u = (fabs(A.SF2[c]) + fabs(A.SF1[c])) * ir;
        const double t_r = fabs(A.SF0[c] * ir);
        const double t_E = fabs(A.SF3[c] * frcp(A.S.rE[g]));
        mflux = fmax(mflux, fmax(t_u, fmax(t_r, t_E)));
      }
    }
  }
  mlam = warp_max(mlam);
  mflux = warp_max(mflux);
  __shared__ double r1[32], r2[32];
  if ((threadIdx.x & 31) == 0) { r1[threadIdx.x >> 5] = mlam; r2[threadIdx.x >> 5] = mflux; }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool ok = threadIdx.x < (blockDim.x >> 5);
    double v1 = ok ? r1[threadIdx.x] : 0.0, v2 = ok ? r2[threadIdx.x] : 0.0;
    v1 = warp_max(v1);
    v2 = warp_max(v2);
    if (threadIdx.x == 0) {
      atomic_max_nonneg(&A.scal[kMaxLam], v1);
      atomic_max_nonneg(&A.scal[kMaxFlux], v2);
    }
  }
}

__device__ __forceinline__ double cfl_dt(double max_lam, double max_flux, double CFL, double max_dt) {
  const double dt1 = CFL / max_lam;
  const double dt2 = CFL / max_flux;  // +inf when the stored flux is zero
  return fmin(dt1, fmin(dt2, max_dt));
}

__global__ void k_cfl_final(double* scal, double CFL, double max_dt) {
  scal[kDt] = cfl_dt(scal[kMaxLam], scal[kMaxFlux], CFL, max_dt);
}

// ---------------------------------------------------------------------------
// The RK step's CFL reduction, screened: the same maxima as k_sound_cmax (mode 2) and
// k_cfl_faces + k_cfl, bit for bit, with ~1 % of their FP64 work. A first pass evaluates
// every cell's value in FP32 from its inputs truncated to float through their bit patterns
// (integer pipe: a cvt between f64 and f32 issues on the FP64 pipe) and reduces the FP32
// maximum M; a second pass evaluates in FP64, with the expressions of the full kernels
// (cell_c2, face_rate, cell_rate), only the cells whose FP32 value is at least
// M (1 - 2^-8), and reduces their maximum. The FP32 value of a cell is within a relative
// ~1e-6 x (its cancellation factor) of its FP64 value, so the cell that attains the FP64
// maximum is always among those evaluated, for cancellation factors below ~10^3 (the
// pressure's rho E / (rho e), 1 + gamma (gamma - 1) M^2 / 2 at local Mach number M, is 113
// at M = 20). Cells whose inputs are not finite floats, or whose FP32 value is NaN, are
// always evaluated in FP64. The last block of each second pass takes the root (c_max) or
// forms dt, and resets the FP32 maximum and its block counter for the next step.
constexpr float kScreenKeep = 1.0f - 1.0f / 256;


// block maximum of non-negative floats into *slot (bit patterns order as unsigned integers)
__device__ __forceinline__ void block_max_f32(float v, unsigned* slot) {
  __shared__ float red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    float w = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (threadIdx.x == 0) atomicMax(slot, __float_as_uint(fmaxf(w, 0.0f)));
  }
}

// FP64 block maximum into scal[slot]; true in thread 0 of the block that arrives last at
// *ticket (every block's maximum is then in)
__device__ __forceinline__ bool block_max_f64_last(double v, double* slot, unsigned* ticket) {
  __shared__ double red[32];
  __shared__ bool last;
  v = warp_max(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    w = warp_max(w);
    if (threadIdx.x == 0) {
      atomic_max_nonneg(slot, w);
      __threadfence();
      last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  return last && threadIdx.x == 0;
}

// scr: [0] FP32 max of gamma p / rho, [1] FP32 max of the cell rates, [2], [3] block counters
__global__ void __launch_bounds__(256) k_cmax_screen(SoundArgs A, float* c2f, unsigned* scr) {
  const int NI = A.nchi + 2, NJ = A.neta + 2;
  const long G = (long)NI * NJ;
  const float gm1 = (float)(A.gamma - 1), gam = (float)A.gamma;
  float mx = 0.0f;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < G; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)k % (unsigned)NI), j = (int)((unsigned)k / (unsigned)NI);
    bool bad = false;
    auto pres = [&](long q, float& r) {
      r = trunc_float(A.S.rho[q], bad);
      const float u = trunc_float(A.S.ru[q], bad), v = trunc_float(A.S.rv[q], bad);
      const float e = trunc_float(A.S.rE[q], bad);
      return __fmaf_rn(-0.5f, __fdividef(__fmaf_rn(u, u, v * v), r), e) * gm1;
    };
    float r, p;
    if (j == 0 && A.isothermal_eta0) {
      float r1, r2;
      p = 2.0f * pres(gidx(i, 1, A.nchi), r1) - pres(gidx(i, 2, A.nchi), r2);
      r = trunc_float(A.S.rho[k], bad);
    } else {
      p = pres(k, r);
    }
    float c2 = __fdividef(gam * p, r);
    if (bad) c2 = __int_as_float(0x7f800000);  // evaluated in FP64, kept out of the FP32 maximum
    else mx = fmaxf(mx, c2);
    c2f[k] = c2;
  }
  block_max_f32(mx, &scr[0]);
}

__global__ void __launch_bounds__(256) k_cmax_exact(SoundArgs A, const float* c2f, unsigned* scr) {
  const int NI = A.nchi + 2, NJ = A.neta + 2;
  const long G = (long)NI * NJ;
  const float M = __uint_as_float(scr[0]);
  const float keep = M > 0.0f ? M * kScreenKeep : -__int_as_float(0x7f800000);
  double mx = 0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < G; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)k % (unsigned)NI), j = (int)((unsigned)k / (unsigned)NI);
    const bool nb = ((A.nrcbc & 1) && i == 1) || ((A.nrcbc & 2) && i == NI - 2) ||
                    ((A.nrcbc & 4) && j == 1) || ((A.nrcbc & 8) && j == NJ - 2);
    if (!(c2f[k] < keep) || nb) {
      const double c2 = cell_c2(A, k, i, j);
      if (nb) A.aS[k] = sqrt(c2);
      mx = fmax(mx, c2);
    }
  }
  if (block_max_f64_last(mx, &A.scal[kCmax], &scr[2])) {
    unsigned long long* bits = reinterpret_cast<unsigned long long*>(&A.scal[kCmax]);
    A.scal[kCmax] = sqrt(__longlong_as_double((long long)atomicAdd(bits, 0ull)));
    scr[0] = 0;
    scr[2] = 0;
  }
}

__global__ void __launch_bounds__(256) k_cfl_screen(CflArgs A, float* rf, unsigned* scr) {
  const int nchi = A.nchi, neta = A.neta;
  const long N = (long)nchi * neta, NLR = (long)(nchi + 1) * neta, NBT = (long)nchi * (neta + 1);
  bool bad_c = false;
  const float cmax = trunc_float(A.scal[kCmax], bad_c);
  float mx = 0.0f;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)c % (unsigned)nchi), j = (int)((unsigned)c / (unsigned)nchi);
    if (A.shock && !(j + 1 < A.cell_idx[i])) continue;
    bool bad = bad_c;
    const long g = gidx(i + 1, j + 1, nchi);
    const long nb[5] = {g, g - 1, g + 1, g - (nchi + 2), g + (nchi + 2)};  // cell, W, E, S, N
    float r[5], u[5], v[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      r[q] = trunc_float(A.S.rho[nb[q]], bad);
      u[q] = trunc_float(A.S.ru[nb[q]], bad);
      v[q] = trunc_float(A.S.rv[nb[q]], bad);
    }
    // the planes' high floats: nx, ny (planes 0, 1) and A/2 (plane 5)
    auto rate = [&](const float2* pl, long NF, long f, int a, int b) {
      const float nx = pl[f].x, ny = pl[NF + f].x, Ah = pl[5 * NF + f].x;
      const float Vn = fabsf(__fmaf_rn(u[a] + u[b], nx, (v[a] + v[b]) * ny)) * __fdividef(1.0f, r[a] + r[b]);
      return (Vn + cmax) * (2.0f * Ah);
    };
    const long fw = i + (long)j * (nchi + 1), fs = i + (long)j * nchi;
    const float lw = rate(A.m.lrf, NLR, fw, 1, 0), le = rate(A.m.lrf, NLR, fw + 1, 0, 2);
    const float ls = rate(A.m.btf, NBT, fs, 3, 0), ln = rate(A.m.btf, NBT, fs + nchi, 0, 4);
    const float ir = __fdividef(1.0f, r[0]);
    float lam_v = trunc_float(A.m.gvis[c], bad) * ir;
    if (A.suth) {
      const float e = __fmaf_rn(-0.5f, __fmaf_rn(u[0], u[0], v[0] * v[0]) * ir, trunc_float(A.S.rE[g], bad)) * ir;
      const float Ts = e * (float)A.Tinf_inv, S = (float)A.suthS;
      lam_v *= Ts * sqrtf(Ts) * (1.0f + S) * __fdividef(1.0f, Ts + S);
    }
    float rate_c = __fmaf_rn(fmaxf(lw, le) + fmaxf(ls, ln), trunc_float(A.m.rvol[c], bad), lam_v);
    if (bad) rate_c = __int_as_float(0x7f800000);
    else mx = fmaxf(mx, rate_c);
    rf[c] = rate_c;
  }
  block_max_f32(mx, &scr[1]);
}

__global__ void __launch_bounds__(256) k_cfl_exact(CflArgs A, const float* rf, unsigned* scr, double CFL,
                                                   double max_dt) {
  const int nchi = A.nchi, neta = A.neta;
  const long N = (long)nchi * neta, NLR = (long)(nchi + 1) * neta, NBT = (long)nchi * (neta + 1);
  const float M = __uint_as_float(scr[1]);
  const float keep = M > 0.0f ? M * kScreenKeep : -__int_as_float(0x7f800000);
  const double cmax = A.scal[kCmax];
  double mlam = 0, mflux = 0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)c % (unsigned)nchi), j = (int)((unsigned)c / (unsigned)nchi);
    if (A.shock && !(j + 1 < A.cell_idx[i])) continue;
    const long g = gidx(i + 1, j + 1, nchi);
    const bool eval = !(rf[c] < keep);
    if (!eval && A.sf_zero) continue;
    const double ir = frcp(A.S.rho[g]);
    if (eval) {
      // the face rates of k_cfl_faces: lr face f between ghosted (i, j+1) and (i+1, j+1),
      // bt face f between (i+1, j) and (i+1, j+1)
      const long fw = i + (long)j * (nchi + 1), fs = i + (long)j * nchi;
      auto lr = [&](long f, long L) {
        return face_rate(A.S, L, L + 1, A.m.lrg[f], A.m.lrg[NLR + f], 2 * A.m.lrg[2 * NLR + f], cmax);
      };
      auto bt = [&](long f, long L) {
        return face_rate(A.S, L, L + (nchi + 2), A.m.btg[f], A.m.btg[NBT + f], 2 * A.m.btg[2 * NBT + f], cmax);
      };
      mlam = fmax(mlam, cell_rate(A, c, g, lr(fw, g - 1), lr(fw + 1, g), bt(fs, g - (nchi + 2)),
                                  bt(fs + nchi, g), ir));
    }
    if (!A.sf_zero) {
      const double t_u = (fabs(A.SF2[c]) + fabs(A.SF1[c])) * ir;
      const double t_r = fabs(A.SF0[c] * ir);
      const double t_E = fabs(A.SF3[c] * frcp(A.S.rE[g]));
      mflux = fmax(mflux, fmax(t_u, fmax(t_r, t_E)));
    }
  }
  // the stored-flux maximum first (no counter), then the rates with the block counter
  mflux = warp_max(mflux);
  __shared__ double rfx[32];
  if ((threadIdx.x & 31) == 0) rfx[threadIdx.x >> 5] = mflux;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < (blockDim.x >> 5) ? rfx[threadIdx.x] : 0.0;
    w = warp_max(w);
    if (threadIdx.x == 0) atomic_max_nonneg(&A.scal[kMaxFlux], w);
  }
  if (block_max_f64_last(mlam, &A.scal[kMaxLam], &scr[3])) {
    unsigned long long* lam = reinterpret_cast<unsigned long long*>(&A.scal[kMaxLam]);
    unsigned long long* flx = reinterpret_cast<unsigned long long*>(&A.scal[kMaxFlux]);
    A.scal[kDt] = cfl_dt(__longlong_as_double((long long)atomicAdd(lam, 0ull)),
                         __longlong_as_double((long long)atomicAdd(flx, 0ull)), CFL, max_dt);
    scr[1] = 0;
    scr[3] = 0;
  }
}

// Step end on S: UPDATE_FIELD_UPSTREAM (after APPLY_BOUNDARY_CONDITIONS), MIN_RHO, t += dt.
struct FillArgs {
  hymor_config cfg;
  DevMesh m;
  Cons S;
  const int* cell_idx;
  double* scal;
  unsigned* err;
  unsigned* ticket;  // blocks done; the last one advances t (every block has read t by then)
  int advance;
  int disturbed;     // any freestream disturbance amplitude non-zero (set on the host)
};

// x < m for m > 0 (not NaN) on the integer pipe: true for every negative x and -0, false
// for NaN, else the order of the non-negative bit patterns
__device__ __forceinline__ bool below_positive(double x, double m) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long a = b & 0x7fffffffffffffffull;
  if (a > 0x7ff0000000000000ull) return false;  // NaN
  return (b >> 63) ? true : b < (unsigned long long)__double_as_longlong(m);
}

// a 32 x 8 block of ghosted cells (columns 1 .. Nchi, every row); MINPOS: rho_min > 0, the
// MIN_RHO test on the bit patterns
template <bool MINPOS>
__global__ void __launch_bounds__(256) k_fill_minrho(FillArgs A) {
  const hymor_config& c = A.cfg;
  const int nchi = c.nchi, neta = c.neta, NI = nchi + 2;
  const double t = A.scal[kT];
  const bool dist = A.disturbed;
  // every FP64 instruction costs a full pass of the SM partition's FP64 pipe on GB300, so
  // the convection speeds of the disturbance are only formed when there is one
  double u_y = 0, u_x = 0;
  if (dist) { u_y = c.rho_v_0 / c.rho_0; u_x = c.rho_u_0 / c.rho_0; }
  unsigned limited = 0;
  const int i = blockIdx.x * 32 + (threadIdx.x & 31) + 1, j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i <= nchi && j <= neta + 1) {
    const long k = (long)i + (long)j * NI;
    if (c.shock_enabled && j >= A.cell_idx[i - 1] + 2) {
      if (dist) {
        const double pert =
            cos(2.0 * M_PI * c.dist_ky * (A.m.y_ext[k] - u_y * t)) * sin(2.0 * M_PI * c.dist_kx * (A.m.x_ext[k] - u_x * t));
        A.S.rho[k] = c.rho_0 + pert * c.dist_amp[0];
        A.S.ru[k] = c.rho_u_0 + pert * c.dist_amp[1];
        A.S.rv[k] = c.rho_v_0 + pert * c.dist_amp[2];
        A.S.rE[k] = c.rho_E_0 + pert * c.dist_amp[3];
      } else {  // pert = 0: the sums reduce to the freestream exactly
        A.S.rho[k] = c.rho_0; A.S.ru[k] = c.rho_u_0; A.S.rv[k] = c.rho_v_0; A.S.rE[k] = c.rho_E_0;
      }
    }
    if (j >= 1 && j <= neta) {  // MIN_RHO.jl:16-23
      const double r = A.S.rho[k];
      if (MINPOS ? below_positive(r, c.rho_min) : r < c.rho_min) {
        A.S.rho[k] = c.rho_min;
        ++limited;
      }
    }
  }
  if (limited) atomicAdd(&A.err[kRhoLimited], limited);
  if (A.advance) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(A.ticket, 1u) == gridDim.x * gridDim.y - 1) {
        A.scal[kT] = A.scal[kT] + A.scal[kDt];
        *A.ticket = 0;
      }
    }
  }
}


// Classical RK4 helpers (value-semantics stages of the MATLAB twin).
struct SnapArgs {
  Cons S, Yc;
  ShockPts pS, pYc;
  long G;
  int nchi;
};
__global__ void k_snapshot(SnapArgs A) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < A.G; k += (long)gridDim.x * blockDim.x) {
    A.Yc.rho[k] = A.S.rho[k]; A.Yc.ru[k] = A.S.ru[k]; A.Yc.rv[k] = A.S.rv[k]; A.Yc.rE[k] = A.S.rE[k];
    if (k < A.nchi) {
      A.pYc.x[k] = A.pS.x[k]; A.pYc.y[k] = A.pS.y[k]; A.pYc.chi[k] = A.pS.chi[k]; A.pYc.eta[k] = A.pS.eta[k];
    }
  }
}

struct ClassArgs {
  Cons Y, Yc;
  ShockPts pY, pYc;
  const double* F0;
  const double* F1;
  const double* F2;
  const double* F3;
  const double* speed_x;
  const double* speed_y;
  const int* cell_idx;
  const double* scal;
  double cY, relax;
  int nchi, neta, shock, sym;
};
__global__ void k_classical_stage(ClassArgs A) {
  const int NI = A.nchi + 2;
  const long G = (long)NI * (A.neta + 2);
  const double w = A.cY * A.scal[kDt];
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < G; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)((unsigned)k % (unsigned)NI), j = (int)((unsigned)k / (unsigned)NI);
    double r = A.Yc.rho[k], u = A.Yc.ru[k], v = A.Yc.rv[k], e = A.Yc.rE[k];
    if (i >= 1 && i <= A.nchi && j >= 1 && j <= A.neta && flow_at(A.cell_idx, A.shock, i - 1, j)) {
      const long c = (long)(i - 1) + (long)(j - 1) * A.nchi;
      r = fma(w, A.F0[c], r); u = fma(w, A.F1[c], u); v = fma(w, A.F2[c], v); e = fma(w, A.F3[c], e);
    }
    A.Y.rho[k] = r; A.Y.ru[k] = u; A.Y.rv[k] = v; A.Y.rE[k] = e;
    if (A.shock && k < A.nchi) {
      const double wr = w * A.relax;
      A.pY.x[k] = A.pYc.x[k] + A.speed_x[k] * wr;
      A.pY.y[k] = A.pYc.y[k] + A.speed_y[k] * wr;
      A.pY.chi[k] = A.pYc.chi[k];
      A.pY.eta[k] = A.pYc.eta[k];
    }
  }
}
// symmetry fix of the classical stage points runs after the stage kernel
__global__ void k_sym_fix(ShockPts p) { p.x[0] = p.x[1]; }

// (a context's ghosted grid has at most 2^30 cells, so the grid-stride kernels split a cell
// index into (i, j) by 32-bit unsigned division)
int grid_for(long n, int threads) {
  long b = (n + threads - 1) / threads;
  const long cap = 152L * 16;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

// ===========================================================================
// launchers

void launch_update_thermo(const DevCtx& d, int mode, double cY, double cS, cudaStream_t st) {
  UpdArgs a;
  a.S = d.S;
  a.Y = d.Y;
  a.Yc = d.Yc;
  a.F0 = d.F[0]; a.F1 = d.F[1]; a.F2 = d.F[2]; a.F3 = d.F[3];
  a.p = d.p;
  a.T = d.T;
  a.cell_idx = d.cell_idx;
  a.scal = d.scal;
  a.err = d.err;
  a.cY = cY;
  a.cS = cS;
  a.gm1 = d.cfg.gamma - 1;
  a.nchi = d.nchi;
  a.neta = d.neta;
  a.mode = mode;
  a.shock = d.cfg.shock_enabled;
  a.aY = d.aY;
  a.nrcbc = (d.cfg.bc_chi0 == HYMOR_BC_OUTFLOW_NRCBC) | ((d.cfg.bc_chi1 == HYMOR_BC_OUTFLOW_NRCBC) << 1) |
            ((d.cfg.bc_eta0 == HYMOR_BC_OUTFLOW_NRCBC) << 2) | ((d.cfg.bc_eta1 == HYMOR_BC_OUTFLOW_NRCBC) << 3);
  k_update_thermo<<<grid_for(d.G, 256), 256, 0, st>>>(a);
}

void launch_spline(const DevCtx& d, bool on_S, bool copy_pts, cudaStream_t st) {
  const hymor_config& c = d.cfg;
  if (!c.shock_enabled) return;
  SplineArgs sa;
  sa.pts = on_S ? d.Sp : d.Yp;
  sa.pS = d.Sp;
  sa.ws = d.spl;
  sa.lam = (1 - c.spline_param) / c.spline_param;
  sa.n = d.nchi;
  sa.copy_pts = copy_pts;
  k_spline_rows<<<(d.nchi + 127) / 128, 128, 0, st>>>(sa);
  k_spline_fit<<<1, kSplineThreads, sizeof(float) * kSplineArrays * spline_stride(d.nchi), st>>>(sa);
}

void launch_columns_bc(const DevCtx& d, bool on_S, bool move, double cY, double cS, int a_mode, bool do_shock,
                       bool do_bc, cudaStream_t st) {
  const hymor_config& c = d.cfg;
  const Cons& tgt = on_S ? d.S : d.Y;
  const ShockPts& pts = on_S ? d.Sp : d.Yp;
  const bool shock = c.shock_enabled && do_shock;
  if (shock) {
    ColArgs ca;
    ca.cfg = c;
    ca.tgt = tgt;
    ca.p = d.p;
    ca.pts = pts;
    ca.pS = d.Sp;
    ca.ws = d.spl;
    ca.cell_idx = d.cell_idx;
    ca.beta = d.beta;
    ca.speed_x = d.speed_x;
    ca.speed_y = d.speed_y;
    ca.rel = d.rel;
    ca.scal = d.scal;
    ca.err = d.err;
    ca.m = d.m;
    ca.cY = cY;
    ca.cS = cS;
    ca.up_cols = d.up_cols;
    ca.move = move;
    ca.on_S = on_S;
    ca.disturbed = c.dist_amp[0] != 0 || c.dist_amp[1] != 0 || c.dist_amp[2] != 0 || c.dist_amp[3] != 0;
    {
      const double rho = c.rho_0, ru = c.rho_u_0, rv = c.rho_v_0, rE = c.rho_E_0;
      const double vi = rv / rho, ui = ru / rho;
      const double um = std::sqrt(vi * vi + ui * ui);
      const double e_inf = (rE - rho * (um * um) * 0.5) / rho;
      ca.p_inf = e_inf * rho * (c.gamma - 1.0);
      ca.u_inf = ui;
      ca.v_inf = vi;
      ca.rho_inf = rho;
      ca.vmag = std::sqrt(ui * ui + vi * vi);
      ca.cph = ui * (1.0 / ca.vmag);
      ca.sph = vi * (1.0 / ca.vmag);
    }
    ca.gp1_gm1 = (c.gamma + 1) / (c.gamma - 1);
    ca.igm1 = 1.0 / (c.gamma - 1);
    ca.two_igm1 = 2 / (c.gamma - 1);
    k_shock_columns<<<(d.nchi + kColCols - 1) / kColCols, kColThreads, 0, st>>>(ca);
  }
  const bool fix = shock && move && c.bc_chi0 == HYMOR_BC_SYMMETRY;
  if (do_bc || fix) {
    BcArgs ba;
    ba.cfg = c;
    ba.q = tgt;
    ba.p = d.p;
    ba.T = d.T;
    ba.a_bc = (a_mode == 0) ? d.aY : d.aS;
    ba.m = d.m;
    ba.pts = pts;
    ba.pS = d.Sp;
    ba.on_S = on_S;
    ba.fix_pts = fix;
    if (!do_bc) {
      // only the shock-point symmetry copy
      ba.cfg.bc_chi0 = HYMOR_BC_SHOCK;
      ba.cfg.bc_chi1 = HYMOR_BC_SHOCK;
    }
    ba.phase = 0;
    k_bc_edges<<<(2 * d.NJ + 255) / 256, 256, 0, st>>>(ba);
    if (do_bc) {
      ba.phase = 1;
      ba.fix_pts = 0;
      k_bc_edges<<<(2 * d.NI + 255) / 256, 256, 0, st>>>(ba);
    }
  }
}

void launch_move_shock(const DevCtx& d, bool on_S, double cY, double cS, cudaStream_t st) {
  const hymor_config& c = d.cfg;
  if (!c.shock_enabled) return;
  MoveArgs a;
  a.cfg = c;
  a.pts = on_S ? d.Sp : d.Yp;
  a.pS = d.Sp;
  a.speed_x = d.speed_x;
  a.speed_y = d.speed_y;
  a.scal = d.scal;
  a.cY = cY;
  a.cS = cS;
  a.on_S = on_S;
  a.fix = c.bc_chi0 == HYMOR_BC_SYMMETRY;
  k_move_shock<<<1, 1024, 0, st>>>(a);
}

static void launch_shock_bc_impl(const DevCtx& d, bool on_S, bool copy_pts, bool move, double cY, double cS,
                                 int a_mode, bool do_shock, bool do_bc, cudaStream_t st) {
  if (do_shock) launch_spline(d, on_S, copy_pts, st);
  launch_columns_bc(d, on_S, move, cY, cS, a_mode, do_shock, do_bc, st);
}

void launch_shock_bc(const DevCtx& d, bool on_S, bool copy_pts, bool move, double cY, double cS,
                     int a_mode, cudaStream_t st) {
  launch_shock_bc_impl(d, on_S, copy_pts, move, cY, cS, a_mode, true, true, st);
}

void launch_shock_bc_flags(const DevCtx& d, bool on_S, bool copy_pts, bool do_shock, bool do_bc, int a_mode,
                           cudaStream_t st) {
  launch_shock_bc_impl(d, on_S, copy_pts, false, 0, 0, a_mode, do_shock, do_bc, st);
}

// resident flux blocks per SM of each variant (index flux_variant + 2 axisymmetric + Sutherland)
int g_flux_blocks_per_sm[40];
// 16 TMA + 8 (16-row tiles) + 4 float-float; the 4-row tiles (thread loads only) from 32
constexpr int flux_variant(bool tma, int rows, bool ffv) {
  return rows == TY / 2 ? 32 + ffv * 4 : tma * 16 + (rows == 16) * 8 + ffv * 4;
}

// a double as a float-float pair (high: nearest float, low: the nearest float to the rest)
float2 host_ff(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

// flux_rows 4 is the split tiling: the tiles are classified at 8 rows and run as 31 x 4 halves
// (halo by thread loads), so that a block of the shock/boundary class fits beside the
// persistent interior grid and its tiles spread over twice the blocks; the halo re-read is
// 6/4 of the cells instead of 10/8.
bool flux_split(const DevCtx& d) { return d.flux_rows == TY / 2; }
int flux_rows(const DevCtx& d) { return d.flux_rows == 16 ? 16 : TY; }  // of the classified tiles
int flux_tiles_x(const DevCtx& d) { return (d.nchi + TX - 1) / TX; }
int flux_tiles(const DevCtx& d) { return flux_tiles_x(d) * ((d.neta + flux_rows(d) - 1) / flux_rows(d)); }
int flux_tiles_max(const DevCtx& d) { return flux_tiles_x(d) * ((d.neta + TY / 2 - 1) / (TY / 2)); }
// capacity of the class-0 list (the class-1 list follows it; each holds at most the tiles of
// the tiling it lists)
int flux_list0_cap(const DevCtx& d) { return flux_split(d) ? flux_tiles_max(d) : flux_tiles(d); }

void launch_classify_tiles(const DevCtx& d, cudaStream_t st) {
  const int nt = flux_tiles(d);
  cudaMemsetAsync(d.tiles, 0, 2 * sizeof(int), st);
  k_classify_tiles<<<(nt + 127) / 128, 128, 0, st>>>(d.cell_idx, d.tiles, d.nchi, d.neta, flux_tiles_x(d), nt,
                                                   d.cfg.shock_enabled, d.cfg.shock_enabled && d.cfg.shock_feedback,
                                                   flux_rows(d), flux_split(d), flux_list0_cap(d));
}

template <bool AXI, bool SUTH, bool FFV, int TYV, bool TMA>
void flux_launch_rows(const FluxArgs& a, const FluxMaps& tm, int tile_class, dim3 grid, const DevCtx& d,
                      cudaStream_t st) {
  const size_t smem = flux_smem<AXI, SUTH, TYV, TMA>();
  if (tile_class == 1 && a.list) {
    // the shock/boundary class: a persistent grid of one block per SM over its few tiles (two
    // of the half-height tiles)
    k_flux<AXI, SUTH, TYV, FFV, TMA><<<d.sms * (TYV == TY / 2 ? 2 : 1), 32 * TYV, smem, st>>>(a, tm);
  } else {
    k_flux<AXI, SUTH, TYV, FFV, TMA><<<grid, 32 * TYV, smem, st>>>(a, tm);
  }
}

template <bool AXI, bool SUTH, bool FFV>
void flux_launch(const FluxArgs& a, const FluxMaps& tm, int tile_class, dim3 grid, const DevCtx& d,
                 cudaStream_t st, int rows, bool tma) {
  const bool r16 = rows == 16;
  if (rows == TY / 2) {
    flux_launch_rows<AXI, SUTH, FFV, TY / 2, false>(a, tm, tile_class, grid, d, st);
  } else if (tma) {
    if (r16) flux_launch_rows<AXI, SUTH, FFV, 16, true>(a, tm, tile_class, grid, d, st);
    else flux_launch_rows<AXI, SUTH, FFV, TY, true>(a, tm, tile_class, grid, d, st);
  } else {
    if (r16) flux_launch_rows<AXI, SUTH, FFV, 16, false>(a, tm, tile_class, grid, d, st);
    else flux_launch_rows<AXI, SUTH, FFV, TY, false>(a, tm, tile_class, grid, d, st);
  }
}

void launch_flux_class(const DevCtx& d, bool on_S, double* const out[4], int tile_class, cudaStream_t st,
                       int spare, bool ffv) {
  FluxArgs a;
  a.tile_class = tile_class;
  a.list = nullptr;
  a.count = nullptr;
  a.tiles_x = flux_tiles_x(d);
  const Cons& q = on_S ? d.S : d.Y;
  a.rho = q.rho; a.ru = q.ru; a.rv = q.rv; a.rE = q.rE;
  a.p = d.p;
  a.T = d.T;
  a.o0 = out[0]; a.o1 = out[1]; a.o2 = out[2]; a.o3 = out[3];
  a.cell_idx = d.cell_idx;
  a.m = d.m;
  a.err = d.err;
  // the split tiling's classes: half-height tiles, halo by thread loads
  const bool half = flux_split(d) && tile_class >= 0 && d.tiles;
  const int rows = half ? TY / 2 : flux_rows(d);
  const bool tma = d.tma && !half;
  FluxMaps tm;
  if (tma) {
    const int ri = rows == 16;
    const CUtensorMap* q4 = on_S ? d.tmS[ri] : d.tmY[ri];
    for (int v = 0; v < 4; ++v) tm.m[v] = q4[v];
    tm.m[4] = d.tmP[ri];
    tm.m[5] = d.tmT[ri];
  } else {
    memset(&tm, 0, sizeof tm);
  }
  const hymor_config& c = d.cfg;
  a.kpr = c.gamma / c.Pr;
  a.kprf = host_ff(a.kpr);
  a.c23f = host_ff(2.0 / 3.0);
  a.suthS = c.sutherland_S;
  a.Tinf_inv = c.energy_factor / c.cv;
  a.nchi = d.nchi;
  a.neta = d.neta;
  a.shock = c.shock_enabled;
  a.mask = c.shock_enabled && c.shock_feedback;
  dim3 grid((d.nchi + TX - 1) / TX, (d.neta + rows - 1) / rows);
  const bool axi = c.axisymmetric, suth = c.viscosity_model == 1;
  if (tile_class >= 0 && d.tiles) {
    // the compact list of the class over a persistent grid (the interior tiles at full
    // occupancy)
    a.count = d.tiles + tile_class;
    a.list = d.tiles + 2 + tile_class * flux_list0_cap(d);
    const int b = g_flux_blocks_per_sm[flux_variant(tma, rows, ffv) + axi * 2 + suth];
    grid = dim3((b > spare + 1 ? b - spare : 1) * d.sms, 1);
  }
  if (ffv) {
    if (!axi && !suth) flux_launch<false, false, true>(a, tm, tile_class, grid, d, st, rows, tma);
    else if (axi && !suth) flux_launch<true, false, true>(a, tm, tile_class, grid, d, st, rows, tma);
    else if (!axi && suth) flux_launch<false, true, true>(a, tm, tile_class, grid, d, st, rows, tma);
    else flux_launch<true, true, true>(a, tm, tile_class, grid, d, st, rows, tma);
  } else {
    if (!axi && !suth) flux_launch<false, false, false>(a, tm, tile_class, grid, d, st, rows, tma);
    else if (axi && !suth) flux_launch<true, false, false>(a, tm, tile_class, grid, d, st, rows, tma);
    else if (!axi && suth) flux_launch<false, true, false>(a, tm, tile_class, grid, d, st, rows, tma);
    else flux_launch<true, true, false>(a, tm, tile_class, grid, d, st, rows, tma);
  }
}

void launch_flux(const DevCtx& d, bool on_S, double* const out[4], cudaStream_t st) {
  launch_flux_class(d, on_S, out, -1, st);
}

template <bool FFV, int TYV, bool TMA>
void flux_setup_variant() {
  auto occ = [](auto kern, size_t smem) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 32 * TYV, smem) != cudaSuccess || b < 1) b = 1;
    return b;
  };
  const int base = flux_variant(TMA, TYV, FFV);
  auto one = [&](auto kern, size_t smem, int idx) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFluxMaxSmem);
    g_flux_blocks_per_sm[base + idx] = occ(kern, smem);
  };
  one(k_flux<false, false, TYV, FFV, TMA>, flux_smem<false, false, TYV, TMA>(), 0);
  one(k_flux<false, true, TYV, FFV, TMA>, flux_smem<false, true, TYV, TMA>(), 1);
  one(k_flux<true, false, TYV, FFV, TMA>, flux_smem<true, false, TYV, TMA>(), 2);
  one(k_flux<true, true, TYV, FFV, TMA>, flux_smem<true, true, TYV, TMA>(), 3);
}

void flux_kernel_setup() {
  flux_setup_variant<false, TY, false>();
  flux_setup_variant<true, TY, false>();
  flux_setup_variant<false, 16, false>();
  flux_setup_variant<true, 16, false>();
  flux_setup_variant<false, TY, true>();
  flux_setup_variant<true, TY, true>();
  flux_setup_variant<false, 16, true>();
  flux_setup_variant<true, 16, true>();
  flux_setup_variant<false, TY / 2, false>();
  flux_setup_variant<true, TY / 2, false>();
  cudaFuncSetAttribute(k_spline_fit, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(float) * kSplineArrays * spline_stride(4096));
}

void launch_flow_cells(const DevCtx& d, cudaStream_t st) {
  FlowArgs A;
  A.cfg = d.cfg;
  A.m = d.m;
  A.S = d.S;
  A.pS = d.Sp;
  A.cell_idx = d.cell_idx;
  A.scal = d.scal;
  A.err = d.err;
  const hymor_config& c = d.cfg;
  A.disturbed = c.dist_amp[0] != 0 || c.dist_amp[1] != 0 || c.dist_amp[2] != 0 || c.dist_amp[3] != 0;
  k_flow_cells<<<(d.nchi * 32 + 63) / 64, 64, 0, st>>>(A);
}

void launch_sound_cmax(const DevCtx& d, bool recompute, cudaStream_t st, bool max_only) {
  SoundArgs A;
  A.S = d.S;
  A.aS = d.aS;
  A.scal = d.scal;
  A.ticket = d.ticket;
  A.gamma = d.cfg.gamma;
  A.nchi = d.nchi;
  A.neta = d.neta;
  A.mode = recompute ? (max_only ? 2 : 1) : 0;
  A.nrcbc = (d.cfg.bc_chi0 == HYMOR_BC_OUTFLOW_NRCBC) | ((d.cfg.bc_chi1 == HYMOR_BC_OUTFLOW_NRCBC) << 1) |
            ((d.cfg.bc_eta0 == HYMOR_BC_OUTFLOW_NRCBC) << 2) | ((d.cfg.bc_eta1 == HYMOR_BC_OUTFLOW_NRCBC) << 3);
  A.isothermal_eta0 = d.cfg.bc_eta0 == HYMOR_BC_NO_SLIP_ISOTHERMAL;
  k_sound_cmax<<<grid_for(d.G, 256), 256, 0, st>>>(A);
}

void launch_cfl(const DevCtx& d, cudaStream_t st) {
  CflArgs A;
  A.S = d.S;
  A.SF0 = d.SF[0]; A.SF1 = d.SF[1]; A.SF2 = d.SF[2]; A.SF3 = d.SF[3];
  A.m = d.m;
  A.cell_idx = d.cell_idx;
  A.scal = d.scal;
  A.gamma = d.cfg.gamma;
  A.suthS = d.cfg.sutherland_S;
  A.Tinf_inv = d.cfg.energy_factor / d.cfg.cv;
  A.suth = d.cfg.viscosity_model == 1;
  A.nchi = d.nchi;
  A.neta = d.neta;
  A.shock = d.cfg.shock_enabled;
  A.lam_lr = d.cflw;
  A.lam_bt = d.cflw + d.NLR;
  A.sf_zero = d.sf_zero;
  k_cfl_faces<<<grid_for(d.NLR + d.NBT, 256), 256, 0, st>>>(A);
  k_cfl<<<grid_for(d.N, 256), 256, 0, st>>>(A);
  k_cfl_final<<<1, 1, 0, st>>>(d.scal, d.cfg.CFL, d.cfg.max_dt);
}

// The step's CFL reduction with the FP32 screen (with shock fitting: the sound-speed
// maximum is recomputed from S, as launch_sound_cmax(d, true, st, true) followed by
// launch_cfl(d, st)); the FP32 values go to the face-rate buffer.
void launch_cfl_screened(const DevCtx& d, cudaStream_t st) {
  SoundArgs S;
  S.S = d.S;
  S.aS = d.aS;
  S.scal = d.scal;
  S.ticket = d.ticket;
  S.gamma = d.cfg.gamma;
  S.nchi = d.nchi;
  S.neta = d.neta;
  S.mode = 2;
  S.nrcbc = (d.cfg.bc_chi0 == HYMOR_BC_OUTFLOW_NRCBC) | ((d.cfg.bc_chi1 == HYMOR_BC_OUTFLOW_NRCBC) << 1) |
            ((d.cfg.bc_eta0 == HYMOR_BC_OUTFLOW_NRCBC) << 2) | ((d.cfg.bc_eta1 == HYMOR_BC_OUTFLOW_NRCBC) << 3);
  S.isothermal_eta0 = d.cfg.bc_eta0 == HYMOR_BC_NO_SLIP_ISOTHERMAL;
  CflArgs A;
  A.S = d.S;
  A.SF0 = d.SF[0]; A.SF1 = d.SF[1]; A.SF2 = d.SF[2]; A.SF3 = d.SF[3];
  A.m = d.m;
  A.cell_idx = d.cell_idx;
  A.scal = d.scal;
  A.gamma = d.cfg.gamma;
  A.suthS = d.cfg.sutherland_S;
  A.Tinf_inv = d.cfg.energy_factor / d.cfg.cv;
  A.suth = d.cfg.viscosity_model == 1;
  A.nchi = d.nchi;
  A.neta = d.neta;
  A.shock = d.cfg.shock_enabled;
  A.lam_lr = d.cflw;
  A.lam_bt = d.cflw + d.NLR;
  A.sf_zero = d.sf_zero;
  float* c2f = reinterpret_cast<float*>(d.cflw);  // G floats
  float* rf = c2f + d.G;                          // N floats (G + N floats fit in NLR + NBT doubles)
  unsigned* scr = d.ticket + 2;
  // the second passes read one float per cell and evaluate a few cells: two blocks per SM,
  // so that the blocks' atomics on the two maxima and the counter stay few
  const int exact_grid = std::min(grid_for(d.G, 256), 2 * d.sms);
  k_cmax_screen<<<grid_for(d.G, 256), 256, 0, st>>>(S, c2f, scr);
  k_cmax_exact<<<exact_grid, 256, 0, st>>>(S, c2f, scr);
  k_cfl_screen<<<grid_for(d.N, 256), 256, 0, st>>>(A, rf, scr);
  k_cfl_exact<<<std::min(grid_for(d.N, 256), 2 * d.sms), 256, 0, st>>>(A, rf, scr, d.cfg.CFL, d.cfg.max_dt);
}

void launch_fill_minrho(const DevCtx& d, bool advance_time, cudaStream_t st) {
  FillArgs A;
  A.cfg = d.cfg;
  A.m = d.m;
  A.S = d.S;
  A.cell_idx = d.cell_idx;
  A.scal = d.scal;
  A.err = d.err;
  A.ticket = d.ticket + 1;
  A.advance = advance_time;
  const hymor_config& c = d.cfg;
  A.disturbed = c.dist_amp[0] != 0 || c.dist_amp[1] != 0 || c.dist_amp[2] != 0 || c.dist_amp[3] != 0;
  const dim3 grid((d.nchi + 31) / 32, (d.neta + 2 + 7) / 8);
  if (c.rho_min > 0)
    k_fill_minrho<true><<<grid, 256, 0, st>>>(A);
  else
    k_fill_minrho<false><<<grid, 256, 0, st>>>(A);
}

void launch_snapshot(const DevCtx& d, cudaStream_t st) {
  SnapArgs A{d.S, d.Yc, d.Sp, d.Ycp, d.G, d.nchi};
  k_snapshot<<<grid_for(d.G, 256), 256, 0, st>>>(A);
}

void launch_classical_stage(const DevCtx& d, double cY, cudaStream_t st) {
  ClassArgs A;
  A.Y = d.Y;
  A.Yc = d.Yc;
  A.pY = d.Yp;
  A.pYc = d.Ycp;
  A.F0 = d.F[0]; A.F1 = d.F[1]; A.F2 = d.F[2]; A.F3 = d.F[3];
  A.speed_x = d.speed_x;
  A.speed_y = d.speed_y;
  A.cell_idx = d.cell_idx;
  A.scal = d.scal;
  A.cY = cY;
  A.relax = d.cfg.relaxation;
  A.nchi = d.nchi;
  A.neta = d.neta;
  A.shock = d.cfg.shock_enabled;
  k_classical_stage<<<grid_for(d.G, 256), 256, 0, st>>>(A);
  if (d.cfg.shock_enabled && d.cfg.bc_chi0 == HYMOR_BC_SYMMETRY && d.nchi >= 2) k_sym_fix<<<1, 1, 0, st>>>(d.Yp);
}

}  // namespace hymor
