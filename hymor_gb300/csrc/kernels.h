// Host-side launchers of the libhymor kernels (core.cu, linear.cu).
#pragma once

#include "common.cuh"

namespace hymor {

// Shock-position blocks of the linearised operator (stability_analysis.perturb_shock,
// LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-274). With them the operator acts on
// n = 4 Nchi Neta + Nchi unknowns: [rho; rho_u; rho_v; rho_E; r], r the normal
// displacements of the shock points, and
//   [A11 A12] with A12 writing only the flux rows (i, sc_i - 1) of every column,
//   [A21 A22]      A21 reading only the cells (i, sc_i - 1), (i, sc_i - 2) of column i.
struct ShockJac {
  int on;          // the operator carries the shock unknowns
  int* rows;       // Nchi: 1-based shocked row sc_i of each column at linearisation
  double* a21;     // Nchi x 8, row-major: d speed_i / d q_v(i, sc_i - j) at (j - 1) * 4 + v
  double* a12;     // 4 Nchi x Nchi, row-major, row v Nchi + i: d flux_v(i, sc_i - 1) / d r_p
  double* a22;     // Nchi x Nchi, row-major: d speed_i / d r_p
  double* a12t;    // transposes of a12 (Nchi x 4 Nchi) and a22, read by the transposed operator
  double* a22t;
  double* rel_b;   // Nchi: shock speeds of the base evaluation
  double* dir;     // 2 x Nchi: PERTURB_SHOCK direction (cos ang, sin ang) of each point
};

struct DevCtx {
  hymor_config cfg;
  int nchi, neta, NI, NJ;
  int sms;         // streaming multiprocessors of the device
  long G, N, NLR, NBT;
  DevMesh m;
  Cons S;          // the solution (reference `s`)
  Cons Y;          // the stage solution (reference `solution_0` / `temp`)
  Cons Yc;         // classical-RK4 snapshot of y_n
  double *p, *T;   // ghosted work arrays (thermodynamic state of the array being evaluated)
  double* aS;      // ghosted sound speed of S (persistent like s["var"]["a"])
  double* aY;      // ghosted sound speed of the stage array (edge-adjacent lines only)
  double* F[4];    // stage flux
  double* SF[4];   // persistent flux of S (s["flux"])
  int sf_zero;     // SF is still all zero (nothing has written it since creation)
  ShockPts Sp, Yp, Ycp;  // shock points of S, Y and the classical snapshot
  int* cell_idx;   // 1-based shocked rows (Nchi)
  double* beta;    // 2 x Nchi: sin and cos of the shock angle of the last shock update of S
  double *speed_x, *speed_y, *rel;  // Nchi
  double* spl;     // spline workspace (device, sized for Nchi)
  double* cflw;    // CFL face rates (NLR + NBT)
  double* scal;    // Scalar block
  unsigned* err;   // ErrWord block
  int* tiles;      // flux tile lists of the RK step (launch_classify_tiles)
  unsigned* ticket;  // [0] k_sound_cmax (mode 2) and [1] k_fill_minrho block counters; [2..5] the
                     // screened CFL reduction's FP32 maxima and block counters
  // Jacobian
  double* coef;    // N * 144 stencil blocks (or null)
  float2* coef_ff; // float-float copy of coef for the propagator (or null)
  int coef_version, coef_ff_version;  // writes of coef, and the write coef_ff was split from
  // the cooperative Taylor propagator in float-float (1, the default) or FP64 (0)
  int expm_ff;
  double* jwork;   // linearisation workspace
  ShockJac sj;
  // prescribed per-column upstream state (4 x Nchi) of the shock chain, or null: set only
  // while the upstream-boundary operator B is assembled (rho_0_upstream_p)
  const double* up_cols;
  // upstream-boundary operator B (LINEARIZE_B): per column m, for the input column
  // n = m + d (d = -1, 0, 1), bq[((m*3 + d+1)*4 + vout)*4 + vin] = d flux_vout(m, sc_m - 1) /
  // d upstream_vin(n) and bs[(m*3 + d+1)*4 + vin] = d speed_m / d upstream_vin(n)
  double *bq, *bs;
  double* res_up;  // 4 x Nchi upstream state of hymor_residual (hymor_set_upstream), or null
  int* brows;      // Nchi: the shocked rows sc_m of B's flux rows
  double* bwork;   // 5 x Nchi: the per-column upstream state and the base shock speeds
  // the RK step's flux forms the viscous terms in float-float arithmetic (1, the default)
  // or in FP64 (0); the residual entry point and the Jacobian always use FP64
  int step_ffv;
  // the step's CFL maxima through the FP32 screen (1, the default) or in FP64 over every cell
  int cfl_screen;
  // flux tiling of the RK step (hymor_autotune): tile rows (8 or 16; 4 = the split tiling, the
  // tiles classified at 8 rows and run as 31 x 4 halves by thread loads) and the block slots
  // per SM the persistent interior-tile grid leaves to the side streams
  int flux_rows, flux_spare;
  // TMA descriptors of the ghosted planes for the flux halo, per tile height (8, 16 rows):
  // S and Y conserved planes, p, T. tma: 1 when they are used (they exist when (Nchi + 2) * 8
  // bytes is a multiple of 16, the TMA row-pitch rule); else the flux loads its halo thread
  // by thread.
  CUtensorMap tmS[2][4], tmY[2][4], tmP[2], tmT[2];
  int tma;
};

// Unknowns of the linearised operator: 4N, plus Nchi with the shock blocks.
inline long op_size(const DevCtx& d) { return 4 * d.N + (d.sj.on ? d.nchi : 0); }

// ---- core.cu ----
// mode: 0 = Y <- S (all ghosted cells), thermo(Y); 1 = Y += wY F, S += wS F (interior,
// masked), thermo(Y); 2 = S += wS F, thermo(S); 3 = thermo(S); 4 = thermo(Y).
// Stage weights are read from the device dt: wY = cY * dt, wS = cS * dt.
void launch_update_thermo(const DevCtx& d, int mode, double cY, double cS, cudaStream_t st);
// Shock fitting + boundary conditions on `tgt` (S when on_S, else Y).
//   copy_pts: copy S's shock points into Y first (stage 1)
//   move: apply MOVE_SHOCK to S (weight cS*dt) and Y (weight cY*dt)
//   a_mode: 0 = compute the edge-adjacent sound speed of tgt into aY before the shock
//           update and use it (PDE); 1 = use the persistent aS (ADVECT_FLOW step end)
void launch_shock_bc(const DevCtx& d, bool on_S, bool copy_pts, bool move, double cY, double cS,
                     int a_mode, cudaStream_t st);
// The two halves of launch_shock_bc: the smoothing-spline fit of the shock points
// (depends only on the points) and the per-column jump + boundary conditions.
void launch_spline(const DevCtx& d, bool on_S, bool copy_pts, cudaStream_t st);
void launch_columns_bc(const DevCtx& d, bool on_S, bool move, double cY, double cS, int a_mode, bool do_shock,
                       bool do_bc, cudaStream_t st);
// MOVE_SHOCK after a launch_columns_bc(.., move = false, ..) with the same on_S, cY, cS:
// moves the points by the stored shock speeds and makes the symmetry copy
void launch_move_shock(const DevCtx& d, bool on_S, double cY, double cS, cudaStream_t st);
// Flux (residual) of tgt into out[4] (masked by the flow cells when feedback is on).
void launch_flux(const DevCtx& d, bool on_S, double* const out[4], cudaStream_t st);
// tile_class 0: only tiles whose halo no shock/BC kernel writes; 1: the other tiles.
// With the step's tile lists (d.tiles) each class runs over its compact list, and tiles
// wholly above the shock are not evaluated (their flux is never read by the stage update).
// spare: resident block slots per SM the persistent interior-tile grid leaves to other streams
// ffv: the viscous terms in float-float arithmetic (the RK step), else FP64
void launch_flux_class(const DevCtx& d, bool on_S, double* const out[4], int tile_class, cudaStream_t st,
                       int spare = 0, bool ffv = false);
// Classifies the flux tiles of the current shocked rows into d.tiles.
void launch_classify_tiles(const DevCtx& d, cudaStream_t st);
int flux_tiles(const DevCtx& d);
int flux_tiles_max(const DevCtx& d);  // the tile count of the smallest tile height (list sizes)
// UPDATE_FLOW_CELLS part 1: detect shocked cells, upstream fill, extrapolation (on S).
void launch_flow_cells(const DevCtx& d, cudaStream_t st);
// Sound speed of S (recompute) and max|a| into scal[kCmax]; recompute=false only reduces aS.
// max_only (with recompute): the max, and a only on the lines outflow_NRCBC reads.
void launch_sound_cmax(const DevCtx& d, bool recompute, cudaStream_t st, bool max_only = false);
// CFL maxima and dt (scal[kDt]).
void launch_cfl(const DevCtx& d, cudaStream_t st);
void launch_cfl_screened(const DevCtx& d, cudaStream_t st);
// Step end: upstream fill + MIN_RHO on S, t += dt.
void launch_fill_minrho(const DevCtx& d, bool advance_time, cudaStream_t st);
// Classical RK4: snapshot S -> Yc (cells and shock points); restore Y <- Yc + c*dt*F.
void launch_snapshot(const DevCtx& d, cudaStream_t st);
void launch_classical_stage(const DevCtx& d, double cY, cudaStream_t st);

// ---- linear.cu ----
void launch_matvec(const DevCtx& d, int k, const double* X, double* Y, int transpose, double scale,
                   cudaStream_t st, long ld = 0);
// graph_ok: with the shock blocks, the Taylor steps may be captured once into a CUDA graph
// and replayed (false: every step is launched directly, nothing is instantiated).
void launch_expm(const DevCtx& d, int k, double dt, int nsteps, int order, const double* X,
                 double* Y, int transpose, double* work, cudaStream_t st, bool graph_ok = true);

}  // namespace hymor
