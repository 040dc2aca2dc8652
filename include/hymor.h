/*
 * hymor.h — C ABI of the GB300-native HYMOR hot path (libhymor.so).
 *
 * The reference (AdrianAA00/HYMOR) is Julia; its hot path is the Julia API
 * below, which a Julia host binds with `ccall`. Every entry
 * point returns 0 on success or a negative HYMOR_ERR_* code; hymor_last_error()
 * gives the message. Arrays use the reference layout: column-major with chi (i)
 * fastest; conserved variables are ghosted (Nchi+2) x (Neta+2) and stored back
 * to back as [rho; rho_u; rho_v; rho_E]; fluxes are 4 x Nchi*Neta; linear
 * vectors are [rho; rho_u; rho_v; rho_E] x Nchi*Neta (4N).
 *
 * One context = one GPU, one CUDA stream, one solution. Contexts are not
 * thread-safe: calls on one context must not overlap.
 */
#ifndef HYMOR_H
#define HYMOR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HYMOR_OK 0
#define HYMOR_ERR_INVALID (-1)      /* bad argument / size / configuration          */
#define HYMOR_ERR_CUDA (-2)         /* CUDA runtime error                           */
#define HYMOR_ERR_NUMERIC (-3)      /* NaN / non-positive density or pressure seen  */
#define HYMOR_ERR_SHOCK_RANGE (-4)  /* shocked cell too close to the domain top     */
#define HYMOR_ERR_TIMEOUT (-5)      /* a bounded device wait (TMA transfer) gave up        */
#define HYMOR_ERR_NOT_READY (-6)    /* e.g. matvec before a Jacobian exists         */

/* Boundary conditions (names of utils/Operators/APPLY_BOUNDARY_CONDITIONS.jl). */
enum {
  HYMOR_BC_SYMMETRY = 0,
  HYMOR_BC_NO_SLIP_ADIABATIC = 1,
  HYMOR_BC_NO_SLIP_ISOTHERMAL = 2,
  HYMOR_BC_OUTFLOW_SUPERSONIC = 3,
  HYMOR_BC_OUTFLOW_SUPERSONIC_1ST = 4,
  HYMOR_BC_OUTFLOW_SUBSONIC = 5,
  HYMOR_BC_OUTFLOW_NRCBC = 6,
  HYMOR_BC_INFLOW_SUPERSONIC = 7,
  HYMOR_BC_INFLOW_SUBSONIC = 8,
  HYMOR_BC_PERIODIC = 9,
  HYMOR_BC_SHOCK = 10
};

/* Curvilinear mappings (utils/Mesh/GO_TO_ELEMENT_SPACE.jl). */
enum { HYMOR_MAP_CIRCLE = 0, HYMOR_MAP_BLUNT_CONE = 1, HYMOR_MAP_CHANNEL = 2, HYMOR_MAP_WEDGE = 3 };

/* The fields of the reference's input Dict that the hot path reads. */
typedef struct {
  int32_t nchi, neta;
  int32_t axisymmetric;                 /* PDE_dimension: 0 "2D", 1 "3D-axisymmetric"        */
  int32_t bc_chi0, bc_chi1, bc_eta0, bc_eta1;
  int32_t shock_enabled, shock_feedback;
  int32_t shock_interp;                 /* 1, 2, 3 = "1st", "2nd", "3rd"                     */
  int32_t shock_eulerian;               /* 0 Lagrangian, 1 Eulerian                          */
  int32_t mapping;                      /* HYMOR_MAP_*                                       */
  int32_t rk_variant;                   /* 0 reference Julia stages, 1 classical RK4         */
  int32_t viscosity_model;              /* 0 constant (reference CPG), 1 Sutherland          */
  int32_t perturb_shock;                /* stability_analysis.perturb_shock: the linearised   */
                                        /* operator adds the Nchi shock-position unknowns    */
  double gamma, Pr, Re, Mach;
  double Tw_chi0, Tw_eta0, Tw_eta1;     /* wall temperature / freestream temperature         */
  double cv, energy_factor;             /* freestream cv, energy factor                      */
  double rho_0, rho_u_0, rho_v_0, rho_E_0, p_0;   /* non-dimensional freestream              */
  double dist_kx, dist_ky, dist_amp[4]; /* freestream disturbance                            */
  double relaxation, spline_param;
  double R, dRs, dRe, circle_angle_extra;
  double L, theta, initial_beta;
  double Lx, Ly, channel_angle, eta_refinement_power;
  double rho_min;
  double CFL, max_dt;
  double perturbation_magnitude;        /* finite-difference step of the Jacobian            */
  double sutherland_S;                  /* S / T_inf of the Sutherland law                   */
} hymor_config;

/* Mesh arrays, host pointers in the reference layout (copied to the device). */
typedef struct {
  const double *lr_xn, *lr_yn, *lr_a;   /* (Nchi+1) x Neta                                   */
  const double *bt_xn, *bt_yn, *bt_a;   /* Nchi x (Neta+1)                                   */
  const double *vol;                    /* Nchi x Neta                                       */
  const double *x_ext, *y_ext;          /* (Nchi+2) x (Neta+2)                               */
  const double *x_corner, *y_corner;    /* (Nchi+1) x (Neta+1)                               */
  const double *chi1;                   /* Nchi: mesh["chi"][:, 1]                           */
  const double *fb_area;                /* Nchi x Neta, axisymmetric only (else NULL)        */
  double fb_yn_front, fb_yn_back;
} hymor_mesh;

typedef struct hymor_ctx_s hymor_ctx;

/* Context: copies the mesh, builds the face geometry, allocates device state.
 * Replaces the reference's solution Dict set-up (utils/Initialization/INITIALIZATION.jl:35-61
 * leaves `s["mesh"]`, `s["var"]`, `s["shock"]` ready for the hot path). */
int hymor_ctx_create(const hymor_config* cfg, const hymor_mesh* mesh, hymor_ctx** out);
int hymor_ctx_destroy(hymor_ctx* ctx);
const char* hymor_last_error(const hymor_ctx* ctx);

/* Solution state: q = 4 ghosted arrays; shock points (Nchi each); cell_idx
 * 1-based shocked-cell rows (shock["cell_indices"], flow cells follow as
 * j < cell_idx[i]); t = time; a = ghosted sound speed or NULL (then sqrt(gamma p / rho)
 * of q). Any shock pointer may be NULL when shock fitting is off. */
int hymor_set_state(hymor_ctx* ctx, const double* q, const double* pts_x, const double* pts_y,
                    const double* pts_chi, const double* pts_eta, const int32_t* cell_idx,
                    double t, const double* a);
int hymor_get_state(hymor_ctx* ctx, double* q, double* pts_x, double* pts_y, double* pts_chi,
                    double* pts_eta, int32_t* cell_idx, double* t, double* dt);

/* NON_LINEAR_DYNAMICS_NO_DISCONTINUITY (utils/Operators/NON_LINEAR_DYNAMICS_NO_DISCONTINUITY.jl:1-28,
 * calling PDE, utils/Operators/PDE.jl:1-47) on the context state, which it mutates
 * like the reference mutates `s` (ghost cells, shocked cells, shock points). Writes
 * the context's flux (read by the CFL dt2 term) and, if flux != NULL, copies it out. */
int hymor_residual(hymor_ctx* ctx, double* flux);
/* A prescribed upstream state per column for hymor_residual (the Dict's rho_0_upstream_p
 * with freestream rho_0_p, rho_u_0_p, rho_v_0_p, rho_E_0_p: 4 x Nchi, COMPUTE_UPSTREAM_
 * CONDITIONS.jl:87-91), as CHECK_LINEARIZATION_B uses it; NULL restores the freestream.
 * The RK step never reads it. */
int hymor_set_upstream(hymor_ctx* ctx, const double* cols);
/* Sets the context's persistent flux arrays (the Dict's s["flux"]). */
int hymor_set_flux(hymor_ctx* ctx, const double* flux);

/* Arithmetic of the viscous terms in the RK step's flux (no counterpart in the reference,
 * whose arithmetic is FP64 throughout). mode 1 (the default): the gradients, stresses and heat
 * flux of VISCOUS_FLUX.jl:36-210 in float-float arithmetic (pairs of FP32 values, ~48-bit
 * significands, on the FP32 pipe, which GB300 issues ~70x faster than FP64), joined back into
 * FP64 before they enter the face fluxes; mode 0: FP64. hymor_residual and the Jacobian
 * (hymor_linearize, hymor_linearize_b) always use FP64. The next hymor_step re-captures its
 * graph. */
int hymor_set_step_viscous(hymor_ctx* ctx, int mode);

/* Reduction of the RK step's CFL maxima (CFL_TIMESTEP.jl:80-130; no counterpart in the
 * reference, which evaluates them in FP64). on = 1 (the default): every cell is screened in
 * FP32 and only the cells within 2^-8 of the FP32 maximum are evaluated in FP64, which gives
 * the FP64 maxima, and dt, bit for bit with ~1 % of the FP64 work; on = 0: every cell in
 * FP64. Only the step with shock fitting screens. The next hymor_step re-captures its graph. */
int hymor_set_cfl_screen(hymor_ctx* ctx, int on);

/* Arithmetic of the Taylor propagator's matvecs (POWER_METHOD!, ARNOLDI_POWER_GPU.jl:36-82;
 * no counterpart in the reference, which multiplies in FP64). mode 1 (the default): the
 * propagations that run as one cooperative launch (the stencil operator, Taylor degree >= 2,
 * 16 launches or more) keep their Taylor terms and running sum as float-float pairs and
 * multiply by a float-float copy of the blocks on the FP32 pipe, ~2^-47 per operation (the
 * input and output vectors stay FP64); mode 0: FP64. hymor_matvec_dev, the propagators with
 * the shock-position unknowns and the receptivity operator are FP64 in either mode. The
 * eigen and transient-growth solvers (hymor_eigs, hymor_tg_gain) use the context's mode. */
int hymor_set_expm_arith(hymor_ctx* ctx, int mode);

/* Tile-shape autotuner of the RK step's flux (no counterpart in the reference): times `steps`
 * steps (CUDA events, after a warm-up step) for each flux configuration — the tile halo staged
 * by TMA (cp.async.bulk.tensor) or loaded thread by thread, tiles of 31 x 8 or 31 x 16 cells
 * or the split tiling (rows = 4: the tiles classified at 31 x 8 cells and run as 31 x 4 halves,
 * halo by thread loads), and 0, 1 or 2 block slots per SM that the persistent
 * interior-tile grid leaves to the side streams — each from the same saved state, restores the
 * state, and keeps the fastest. choice[3] = (rows, spare, tma); ms_per_step[18] (or NULL) = the
 * candidates' times, index 9 tma + 3 r + spare with r = 0, 1, 2 for rows 8, 16, 4 (0 where a
 * TMA candidate could not run: Nchi odd). Every
 * configuration gives bit-identical fluxes (each face flux has the same arithmetic whichever
 * tile computes it, and the staged halo holds the same values). hymor_set_flux_tiling sets one
 * directly (default: the split tiling, 1 spare slot, TMA when Nchi is even: with the split
 * tiling only the whole-grid flux of the residual and of the classical RK4 scheme stages its
 * halo by TMA). */
int hymor_autotune(hymor_ctx* ctx, int steps, int32_t* choice, float* ms_per_step);
int hymor_set_flux_tiling(hymor_ctx* ctx, int rows, int spare, int tma);

/* nsteps x ADVECT_FLOW (utils/Time_marching/ADVECT_FLOW.jl:30-39 ->
 * ADVECT_FLOW_EXPLICIT.jl:36-81), all on the device (one CUDA graph per step). */
int hymor_step(hymor_ctx* ctx, int nsteps);
/* ADVECT_FLOW on a host-resident solution, in one call: the state in q (4 x G, as
 * hymor_set_state), the shock points, the shocked rows and t are uploaded, nsteps steps
 * run, and the advanced state, points, rows and t are written back into the same buffers
 * (the Dict mutated in place, ADVECT_FLOW.jl:30-39). One synchronisation per call; errors
 * as hymor_step. Equivalent to hymor_set_state + hymor_step + hymor_get_state. */
int hymor_advect(hymor_ctx* ctx, int nsteps, double* q, double* pts_x, double* pts_y, double* pts_chi,
                 double* pts_eta, int32_t* cell_idx, double* t);
/* UPDATE_FLOW_CELLS (utils/Shock_fitting/UPDATE_FLOW_CELLS.jl:25-37). */
int hymor_update_flow_cells(hymor_ctx* ctx);
/* CFL_TIMESTEP (utils/Time_marching/CFL_TIMESTEP.jl:41-138) on the current state. */
int hymor_cfl_timestep(hymor_ctx* ctx, double* dt);
/* Counters: MIN_RHO activations and Rankine-Hugoniot y < 1 warnings since creation. */
int hymor_counters(hymor_ctx* ctx, int32_t* rho_limited, int32_t* rh_warnings);
/* Number of kernel launches one hymor_step makes (the kernel nodes of its CUDA graph),
 * for launch accounting. No counterpart in the reference. */
int hymor_step_kernels(hymor_ctx* ctx, int32_t* n);
/* Average phases (ms) of the steps profiled since hymor_profile_flux(ctx, 1, ..):
 * ms[0] step start to the first stage update; per stage k, ms[1 + 4k] the stage update,
 * ms[2 + 4k] the flux of the interior tiles, ms[3 + 4k] the start of the flux of the
 * shock/boundary tiles (its own stream) after the start of the interior flux, ms[4 + 4k]
 * that flux; ms[17] the later end of the last stage's two flux launches to the step end.
 * Call before hymor_profile_flux(ctx, 0, ..), which releases the events. No counterpart
 * in the reference. */
int hymor_profile_phases(hymor_ctx* ctx, float* ms);
/* FP64 FMA throughput of the context's GPU in TFLOP/s (independent DFMA chains over
 * every SM, timed with CUDA events), the roofline denominator of the FP64-bound
 * kernels. No counterpart in the reference. */
int hymor_fp64_peak(hymor_ctx* ctx, double* tflops);

/* Device timing on the context stream (CUDA events): start, then stop returns ms. */
int hymor_timer_start(hymor_ctx* ctx);
int hymor_timer_stop(hymor_ctx* ctx, float* ms);
/* Per-kernel device time of the residual (flux) kernel inside the last hymor_step
 * call: total ms and number of launches (measured with CUDA events on the stream). */
int hymor_profile_flux(hymor_ctx* ctx, int enable, float* total_ms, int32_t* launches);
int hymor_synchronize(hymor_ctx* ctx);
/* Benchmark helper (no reference counterpart): nsteps x ADVECT_FLOW, each step preceded,
 * outside its timed window, by a write of flush_bytes to a scratch buffer (evicts the
 * L2 cache). *ms = summed device time of the steps (CUDA events on the context stream). */
int hymor_bench_steps(hymor_ctx* ctx, int nsteps, uint64_t flush_bytes, float* ms);

/* ---- Linearised operator (stencil-block Jacobian) ----
 * Storage per output cell m (chi-fastest), neighbour slot q = (b+1)*3 + (a+1) for the
 * input cell at offset (a, b): coef[((m*9 + q)*4 + vout)*4 + vin] = L[(m,vout),(m+(a,b),vin)]. */

/* LINEARIZE_L (utils/Stability_analysis/Modal_stability_analysis/LINEARIZE_L.jl:34-69 ->
 * LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:42-288): coloured finite-difference Jacobian of the
 * residual on the device, 36 perturbed residuals batched. Keeps the blocks on the device. */
int hymor_linearize(hymor_ctx* ctx);
/* Copy the blocks out (Nchi*Neta*144 doubles) / in. */
int hymor_jacobian_get(hymor_ctx* ctx, double* coef);
int hymor_jacobian_set(hymor_ctx* ctx, const double* coef);

/* Shock-position unknowns (stability_analysis.perturb_shock,
 * LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-274). hymor_linearize with cfg.perturb_shock
 * also assembles, on the device, the blocks that couple the flow to the normal displacements
 * r of the Nchi shock points; the operator then acts on n = 4 Nchi Neta + Nchi unknowns
 * [rho; rho_u; rho_v; rho_E; r] (the reference's 4*Nchi*Neta + Nchi), and every matvec,
 * propagator and vector length below uses that n. With sc_i the 1-based shocked row of
 * column i at linearisation:
 *   rows[i] = sc_i                                                         (Nchi)
 *   a21[i*8 + (j-1)*4 + v] = d speed_i / d q_v(i, sc_i - j), j = 1, 2        (Nchi x 8)
 *   a12[(v*Nchi + i)*Nchi + p] = d flux_v(i, sc_i - 1) / d r_p              (4 Nchi x Nchi)
 *   a22[i*Nchi + p] = d speed_i / d r_p                                      (Nchi x Nchi)
 * (speed = s["shock"]["relative_increase_velocity"]); every other entry of the reference's
 * blocks is zero. Requires 3 <= sc_i <= Neta - 1. */
int hymor_operator_size(hymor_ctx* ctx, int64_t* n);
int hymor_shock_blocks_get(hymor_ctx* ctx, int32_t* rows, double* a21, double* a12, double* a22);
/* Sets the blocks (after a Jacobian exists) and turns the shock unknowns on; rows == NULL
 * turns them off (n = 4 Nchi Neta). */
int hymor_shock_blocks_set(hymor_ctx* ctx, const int32_t* rows, const double* a21, const double* a12,
                           const double* a22);
/* s["shock"]["beta"] of the last shock update of the solution (Nchi angles) and the
 * relative shock speeds of the last shock update (Nchi); either pointer may be NULL. */
int hymor_shock_fields(hymor_ctx* ctx, double* beta, double* rel_vel);

/* Y = L X (transpose 0) or Lᵀ X (transpose 1) for k vectors (n x k, column-major, n =
 * hymor_operator_size), host pointers. Replaces the CuSparse SpMV `mul!(term, A, v)` of
 * Eigenvalues/ARNOLDI_POWER_GPU.jl:73 (and its transpose, TRANSIENT_GROWTH_DOWNSTREAM.jl:75). */
int hymor_matvec(hymor_ctx* ctx, int k, const double* X, double* Y, int transpose);
/* Same on device pointers (no copies). */
int hymor_matvec_dev(hymor_ctx* ctx, int k, const double* dX, double* dY, int transpose);
/* Timing of hymor_matvec_dev (no counterpart in the reference): reps repetitions of one
 * launch over the k vectors (per_vector 0), or of k launches of one vector each
 * (per_vector 1, the one-vector path); *ms = their device time, CUDA events on the
 * context stream. */
int hymor_bench_matvec(hymor_ctx* ctx, int k, const double* dX, double* dY, int transpose, int per_vector,
                       int reps, float* ms);
/* Y = (Σ_{j<=order} (A dt)^j / j!)^nsteps X for k vectors: POWER_METHOD!
 * (Eigenvalues/ARNOLDI_POWER_GPU.jl:64-82); transpose uses (A dt)ᵀ (EXPONENTIAL!,
 * Transient_growth_downstream/CONSTRUCT_C.jl:78-111). Host pointers. */
int hymor_expm_apply(hymor_ctx* ctx, int k, double dt, int nsteps, int order, const double* X,
                     double* Y, int transpose);
int hymor_expm_apply_dev(hymor_ctx* ctx, int k, double dt, int nsteps, int order,
                         const double* dX, double* dY, int transpose);
/* k propagations of different lengths in one batched call: vector c gets nsteps[c] steps
 * of dt[c] (host arrays of k; nsteps non-increasing, so the vectors still advancing are a
 * prefix). Device pointers. The transient-growth horizons of one solve batch (no
 * counterpart in the reference, which propagates one horizon per call). */
int hymor_expm_apply_multi_dev(hymor_ctx* ctx, int k, const double* dts, const int32_t* nsteps, int order,
                               const double* dX, double* dY, int transpose);

/* Allocation-free variant of hymor_expm_apply_dev. It has no counterpart in the reference.
 * For callers that cannot call cudaMalloc during a solve: a service that reserves its whole
 * device-memory budget at start-up and treats any later allocation as a failure, or a host
 * runtime whose own pool allocator owns the device memory. hymor_expm_apply_dev allocates
 * work vectors per call (and, with the shock unknowns, instantiates a CUDA graph of one
 * Taylor step); this variant takes its work vectors from one fixed 24 MiB device array that
 * every GPU loading the library holds until exit, and launches every Taylor step directly.
 * Requires hymor_operator_size * k <= 1048576 (else HYMOR_ERR_INVALID, before any device
 * work). All calls share the array and it keeps the last call's contents (nothing in it
 * needs to start at zero): calls whose GPU work overlaps race, so serialise them. The first
 * call for a context on a device makes that device current and looks up the array's
 * address there: make that first call before any stream capture. */
int hymor_expm_apply_dev_noalloc(hymor_ctx* ctx, int k, double dt, int nsteps, int order,
                                 const double* dX, double* dY, int transpose);

/* ---- Freestream receptivity (utils/Stability_analysis/Freestream_receptivity) ----
 * LINEARIZE_B (LINEARIZE_B.jl:40-296): the upstream-boundary operator B, the response of
 * the residual to a per-column upstream state (rho_0_upstream_p) [rho; rho_u; rho_v; rho_E]
 * (4 x Nchi), assembled on the device with 13 residuals (3 colours of columns per
 * variable). With sc_m the 1-based shocked row of column m at assembly and n = m + d,
 * d = -1, 0, 1:
 *   rows[m] = sc_m,
 *   bq[((m*3 + d+1)*4 + vout)*4 + vin] = d flux_vout(m, sc_m - 1) / d upstream_vin(n),
 *   bs[(m*3 + d+1)*4 + vin] = d speed_m / d upstream_vin(n)   (rows of the shock unknowns).
 * Needs shock fitting and 2 <= sc_m <= Neta - 1; call after hymor_linearize. */
int hymor_linearize_b(hymor_ctx* ctx);
int hymor_b_get(hymor_ctx* ctx, int32_t* rows, double* bq, double* bs);
int hymor_b_set(hymor_ctx* ctx, const int32_t* rows, const double* bq, const double* bs);
/* The extended operator of LINEARIZE_L_ (LINEARIZE_L_.jl:36-71) for nw frequencies w (host
 * array): L_ = [L, B ... B; 0, diag(-i w_k I_{4 Nchi})], n_ = hymor_operator_size + nw*4*Nchi
 * unknowns (hymor_recept_size). Complex vectors are stored as their real part followed by
 * their imaginary part (2 n_ doubles each); k of them back to back. */
int hymor_recept_size(hymor_ctx* ctx, int nw, int64_t* n);
/* Y = scale L_ X, or scale L_^H X (adjoint: the conjugate transpose). Device pointers. */
int hymor_recept_apply_dev(hymor_ctx* ctx, int k, int nw, const double* w, double scale, const double* dX,
                           double* dY, int adjoint);
/* EXPONENTIAL! (Transient_growth_downstream/CONSTRUCT_C.jl:78-111) with L_ (or L_^H): per
 * step term = Y, then term = (L_ dt) term / j and Y += term for j = 1..order. */
int hymor_recept_expm_dev(hymor_ctx* ctx, int k, int nw, const double* w, double dt, int nsteps, int order,
                          const double* dX, double* dY, int adjoint);

/* ---- Device-resident Krylov building blocks (replace the host Arpack loop around the
 * GPU matvec, Eigenvalues/EIGENVALUES.jl:159 and TRANSIENT_GROWTH_DOWNSTREAM.jl:103).
 * Reductions are deterministic (fixed block partition, fixed-order trees). */
/* out[j] = A[:, j] . w for j < m (A device, column stride lda); out on the host. */
int hymor_dot_dev(hymor_ctx* ctx, int64_t n, int m, const double* dA, int64_t lda, const double* dw,
                  double* out);
/* Classical Gram-Schmidt twice of device vector w against V[:, 0:m]; h[0..m-1] = the
 * coefficients, h[m] = ||w|| after orthogonalisation (host array of m+1); if out_col >= 0
 * the normalised w is written to V[:, out_col]. */
int hymor_krylov_orthogonalize(hymor_ctx* ctx, int64_t n, int m, double* dV, int64_t ldv,
                               double* dw, double* h, int out_col);
/* V[:, 0:k] = V[:, 0:m] Q with Q host, column-major m x k (Krylov-Schur restart). */
int hymor_krylov_rotate(hymor_ctx* ctx, int64_t n, int m, int k, double* dV, int64_t ldv,
                        const double* Q);
/* Y = blockdiag(B) X for k 4N-vectors; B device, row-major 4x4 per cell (N x 16). Applies
 * the Chu-norm weights R'MR and R'M^R of CONSTRUCT_R/M/M_HAT (Transient_growth_downstream/
 * CONSTRUCT_R.jl:24-133, CONSTRUCT_M.jl:27-94, CONSTRUCT_M_HAT.jl:25-105). */
int hymor_block4_apply_dev(hymor_ctx* ctx, int k, const double* dB, const double* dX, double* dY);
/* Same for k vectors of 4N + ntail entries: the cells as above, the tail scaled by dTail
 * (ntail doubles) — the shock-position entries of R'M^R (CONSTRUCT_M_HAT.jl:78-90), or
 * the freestream blocks of the receptivity operator. */
int hymor_block4_apply_ext_dev(hymor_ctx* ctx, int k, int64_t ntail, const double* dB, const double* dTail,
                               const double* dX, double* dY);

/* ---- Device-resident eigen and transient-growth solvers (Krylov-Schur on the device
 * basis; the host handles only the projected matrix, at most (ncv + 2 block)^2). ---- */
typedef struct {
  int32_t nev;        /* eigenvalues / gains wanted (the reference's n_modes)                    */
  int32_t ncv;        /* basis size; 0 picks max(2 nev + 1, 20, nev + 4 block)                   */
  int32_t maxit;      /* Krylov-Schur cycles (restarts + 1)                                      */
  int32_t block;      /* vectors per batched propagation; 1 = Krylov-Schur, > 1 = block variant  */
  int32_t order;      /* Taylor degree of one propagator step (5: POWER_METHOD!, 4: RK4 substeps) */
  int32_t flow_start; /* start vectors vanish outside the flow cells (when x0 is NULL)            */
  uint64_t seed;      /* start vectors when x0 is NULL (deterministic normal variates)            */
  double tol;         /* converged when every Ritz residual <= tol |theta|                        */
} hymor_krylov_opts;
/* EIGENVALUES_GPU_ARNOLDI (Stability_analysis/Eigenvalues/EIGENVALUES.jl:112-205, the Arpack
 * call of :152-162 with the matvec closure of ARNOLDI_POWER_GPU.jl:36-82): the nev eigenvalues
 * mu of largest modulus of P = exp(L dt nsteps) (nsteps Taylor steps of degree order), in
 * decreasing modulus (lambda = log(mu) / (dt nsteps) is the caller's mapping, as the
 * reference's :166). x0: host start block (n x block, n = hymor_operator_size) or NULL.
 * resid: Ritz residual norms (may be NULL). info[3]: operator applications (vectors),
 * restarts, converged (1/0). dvecs: NULL, or a device buffer of n x 2 nev receiving the unit
 * eigenvectors' real parts (first nev columns) and imaginary parts (needs 2 nev <= ncv). A
 * solve that stops at maxit returns 0 with info[2] = 0: the reference then warns and returns
 * NaN (EIGENVALUES.jl:184-204), which is the caller's choice here. */
int hymor_eigs(hymor_ctx* ctx, const hymor_krylov_opts* opts, double dt, int nsteps, const double* x0, double* mu_re,
               double* mu_im, double* resid, int32_t* info, double* dvecs);
/* TRANSIENT_GROWTH_DOWNSTREAM (Stability_analysis/Transient_growth_downstream/
 * TRANSIENT_GROWTH_DOWNSTREAM.jl:34-153, the Arpack call of :96-106 with CONSTRUCT_C.jl's
 * operator): the nev largest optimal energy gains G(T) of exp(L' T) R'MR exp(L T) x = G R'M^R x
 * for nh horizons T[h], with R, M, M^ built on the device context's solution (CONSTRUCT_R.jl,
 * CONSTRUCT_M.jl, CONSTRUCT_M_HAT.jl) and the problem reduced by the per-cell Cholesky factor
 * of R'M^R. Each horizon uses steps = round(T / dt_CFL) Taylor steps of dt = T / steps (:40-44;
 * dt_out, nsteps_out per horizon, may be NULL). Several horizons (nh > 1, block 1) run in
 * lockstep, one batched propagation per round for all unfinished horizons (no counterpart in
 * the reference, which solves one horizon per call). gains, resid: nh x nev; info: nh x 3 as
 * hymor_eigs. dvecs (nh = 1 only): NULL or a device buffer of n x nev receiving the optimal
 * initial conditions x (x' R'M^R x = 1), the reference's V. */
int hymor_tg_gain(hymor_ctx* ctx, const hymor_krylov_opts* opts, int nh, const double* T, const double* x0,
                  double* gains, double* resid, int32_t* info, double* dt_out, int32_t* nsteps_out, double* dvecs);
/* The dense steps of the two solvers, exposed for testing and for callers with their own
 * Krylov loops (no counterpart in the reference, whose dense steps are Arpack's LAPACK calls):
 * real Schur form A = Z T Z' (column-major n x n, n <= 1024) with the nsel eigenvalues of
 * largest modulus leading (whole conjugate pairs; *nlead = rows they fill), wr/wi the
 * eigenvalues in T's order; and the symmetric eigen-decomposition A = V diag(w) V'. */
int hymor_dense_schur(int n, const double* A, int nsel, double* T, double* Z, double* wr, double* wi, int32_t* nlead);
int hymor_dense_symeig(int n, const double* A, double* w, double* V);

/* Device buffer helpers for the *_dev entry points. */
int hymor_device_alloc(hymor_ctx* ctx, uint64_t bytes, void** dptr);
int hymor_device_free(hymor_ctx* ctx, void* dptr);
int hymor_memcpy_h2d(hymor_ctx* ctx, void* dst, const void* src, uint64_t bytes);
int hymor_memcpy_d2h(hymor_ctx* ctx, void* dst, const void* src, uint64_t bytes);
int hymor_memcpy_d2d(hymor_ctx* ctx, void* dst, const void* src, uint64_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* HYMOR_H */
