// C ABI of libhymor: context, state transfer, residual, RK4 step (CUDA graph),
// CFL, timing. Declarations and reference citations: include/hymor.h.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include "kernels.h"

namespace hymor {
void flux_kernel_setup();
void linear_state_release(void* p);
}

using namespace hymor;

struct hymor_ctx_s {
  DevCtx d;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;      // high-priority stream of the shock/BC chain inside the step graph
  cudaStream_t fit = nullptr;       // the first spline fit and the first jump kernels of a step
  cudaStream_t c1 = nullptr;        // the shock/boundary-class flux, beside the interior-class flux
  cudaStream_t cfl = nullptr;       // the step's CFL reduction, at the lowest priority
  cudaEvent_t fork_ev[8] = {}, join_ev[8] = {};
  cudaEvent_t fit_fork = nullptr, fit_join = nullptr;
  cudaEvent_t c1_fork[4] = {}, c1_join[4] = {};
  cudaEvent_t u0_ev = nullptr, cfl_ev = nullptr, cls_ev = nullptr, cfl_fork = nullptr;
  int device = 0;
  std::string err;
  std::vector<void*> allocs;
  // step graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int step_kernels = 0;  // kernel nodes of the step graph
  // flux-kernel profiling: event-record nodes around the flux launches of the 4 stages
  // (2 launches per stage: the interior tiles on the main stream, the shock/boundary tiles
  // on their own stream)
  bool profile = false;
  // 4 k .. 4 k + 3: around the two flux launches of stage k; 16 + k: start of stage k's
  // stage update; 20: step start; 21: step end (main stream)
  static constexpr int kEv = 22;
  cudaGraphNode_t ev_nodes[kEv] = {};
  cudaEvent_t cap_ev[kEv] = {};
  std::vector<cudaEvent_t> prof_ev;  // kEv per profiled step
  int prof_steps = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  int timer_running = 0;
  // L2 flush scratch of hymor_bench_steps
  void* flush_buf = nullptr;
  uint64_t flush_bytes = 0;
  // state of the linear entry points: propagator work vectors, Krylov scratch (linear.cu)
  void* linear_state = nullptr;
  // pinned host staging of the small state arrays (shock points, cell indices, scalars),
  // so that set_state / get_state move them by DMA instead of pageable staged copies
  unsigned char* stage = nullptr;
  // the persistent sound speed has not been computed for the state set last (set_state
  // without it); the next call that reads it computes it first
  bool a_stale = false;
  // the flux halo can be staged by TMA (descriptors made at creation)
  int tma_able = 0;
};

namespace {

int fail(hymor_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CU(call)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(ctx, HYMOR_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                              \
  } while (0)

template <typename T>
int dalloc(hymor_ctx* ctx, T** p, size_t count) {
  void* v = nullptr;
  CU(cudaMalloc(&v, count * sizeof(T) + 16));
  CU(cudaMemset(v, 0, count * sizeof(T) + 16));
  ctx->allocs.push_back(v);
  *p = static_cast<T*>(v);
  return 0;
}

#define TRY(x)            \
  do {                    \
    int r_ = (x);         \
    if (r_) return r_;    \
  } while (0)

int check_config(hymor_ctx* ctx, const hymor_config* c) {
  if (c->nchi < 3 || c->neta < 4) return fail(ctx, HYMOR_ERR_INVALID, "grid too small: %d x %d", c->nchi, c->neta);
  if (c->nchi > 4096) return fail(ctx, HYMOR_ERR_INVALID, "Nchi = %d exceeds 4096 (shock spline workspace)", c->nchi);
  if ((long)(c->nchi + 2) * (c->neta + 2) > (1L << 31) / 2) return fail(ctx, HYMOR_ERR_INVALID, "grid too large");
  const int bcs[4] = {c->bc_chi0, c->bc_chi1, c->bc_eta0, c->bc_eta1};
  for (int e = 0; e < 4; ++e) {
    if (bcs[e] < 0 || bcs[e] > HYMOR_BC_SHOCK) return fail(ctx, HYMOR_ERR_INVALID, "unknown boundary condition %d", bcs[e]);
    if (bcs[e] == HYMOR_BC_SHOCK && e != 3)
      return fail(ctx, HYMOR_ERR_INVALID, "Non defined Boundary-condition: shock is only valid on eta1");
  }
  if (c->shock_enabled && c->bc_eta1 != HYMOR_BC_SHOCK)
    return fail(ctx, HYMOR_ERR_INVALID, "shock fitting needs boundary_eta1 = shock");
  if (c->shock_interp < 1 || c->shock_interp > 3) return fail(ctx, HYMOR_ERR_INVALID, "Invalid shock.interpolate");
  if (!(c->gamma > 1)) return fail(ctx, HYMOR_ERR_INVALID, "freestream.gamma must be > 1");
  if (!(c->Re > 0) || !(c->Pr > 0)) return fail(ctx, HYMOR_ERR_INVALID, "Re and Pr must be positive");
  if (c->mapping < 0 || c->mapping > 3) return fail(ctx, HYMOR_ERR_INVALID, "unknown mapping %d", c->mapping);
  if (c->rk_variant < 0 || c->rk_variant > 1) return fail(ctx, HYMOR_ERR_INVALID, "unknown rk_variant");
  if (c->viscosity_model < 0 || c->viscosity_model > 1) return fail(ctx, HYMOR_ERR_INVALID, "unknown viscosity model");
  if (c->shock_enabled && !(c->spline_param > 0 && c->spline_param <= 1))
    return fail(ctx, HYMOR_ERR_INVALID, "spline_param must be in (0, 1]");
  return 0;
}

int upload(hymor_ctx* ctx, double** dst, const double* src, size_t n, const char* name) {
  if (!src) return fail(ctx, HYMOR_ERR_INVALID, "mesh array %s is NULL", name);
  TRY(dalloc(ctx, dst, n));
  CU(cudaMemcpy(*dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

// Geometry planes of the flux kernel (see common.cuh), computed once per mesh on the
// host in FP64 from the reference's mesh arrays (VISCOUS_FLUX.jl:72-95).
void face_geometry(const hymor_config& c, const hymor_mesh& m, std::vector<double>& lrg,
                   std::vector<double>& btg, std::vector<double>& rvol, std::vector<double>& rxl,
                   std::vector<double>& rxb, std::vector<double>& gvis) {
  const int nchi = c.nchi, neta = c.neta;
  const long NLR = (long)(nchi + 1) * neta, NBT = (long)nchi * (neta + 1), N = (long)nchi * neta;
  lrg.assign(kGeoPlanes * NLR, 0.0);
  btg.assign(kGeoPlanes * NBT, 0.0);
  // the gradient planes carry 2 mu*/Re (mu* = 1 for CPG), so that the face kernel forms
  // twice the viscous traction without a multiply (Sutherland faces scale it by mu_f)
  const double vs = 2.0 / c.Re;
  rvol.assign(N, 0.0);
  rxl.assign(NLR, 0.0);
  rxb.assign(NBT, 0.0);
  auto X = [&](int i, int j) { return m.x_ext[i + (long)j * (nchi + 2)]; };
  auto Y = [&](int i, int j) { return m.y_ext[i + (long)j * (nchi + 2)]; };
  auto xc = [&](int i, int j) { return m.x_corner[i + (long)j * (nchi + 1)]; };
  auto yc = [&](int i, int j) { return m.y_corner[i + (long)j * (nchi + 1)]; };
  for (int j = 0; j < neta; ++j)
    for (int i = 0; i <= nchi; ++i) {
      const long f = i + (long)j * (nchi + 1);
      const double nx = m.lr_xn[f], ny = m.lr_yn[f];
      const double dX = X(i + 1, j + 1) - X(i, j + 1), dY = Y(i + 1, j + 1) - Y(i, j + 1);
      const double cld = std::sqrt(dY * dY + dX * dX);
      const double c1x = -dX / cld, c1y = -dY / cld;
      const double Cnn = -c1x * nx - c1y * ny;
      const double Cft = c1x * ny - c1y * nx;
      const double lx = xc(i, j + 1) - xc(i, j), ly = yc(i, j + 1) - yc(i, j);
      const double len = std::sqrt(lx * lx + ly * ly);
      lrg[0 * NLR + f] = nx;
      lrg[1 * NLR + f] = ny;
      lrg[2 * NLR + f] = 0.5 * m.lr_a[f];
      lrg[3 * NLR + f] = vs * (-1.0 / (cld * Cnn));
      lrg[4 * NLR + f] = vs * (0.25 * (-Cft / (len * Cnn)));
      lrg[5 * NLR + f] = vs * (0.25 * (1.0 / len));
      rxl[f] = vs * (1.0 / ((X(i + 1, j + 1) + X(i, j + 1)) / 2));
    }
  for (int j = 0; j <= neta; ++j)
    for (int i = 0; i < nchi; ++i) {
      const long f = i + (long)j * nchi;
      const double nx = m.bt_xn[f], ny = m.bt_yn[f];
      const double dX = X(i + 1, j + 1) - X(i + 1, j), dY = Y(i + 1, j + 1) - Y(i + 1, j);
      const double cbd = std::sqrt(dY * dY + dX * dX);
      const double c2x = dX / cbd, c2y = dY / cbd;
      const double Cnn = c2x * nx + c2y * ny;
      const double Cft = c2x * ny - c2y * nx;
      const double lx = xc(i + 1, j) - xc(i, j), ly = yc(i + 1, j) - yc(i, j);
      const double len = std::sqrt(lx * lx + ly * ly);
      btg[0 * NBT + f] = nx;
      btg[1 * NBT + f] = ny;
      btg[2 * NBT + f] = 0.5 * m.bt_a[f];
      btg[3 * NBT + f] = vs * (1.0 / (cbd * Cnn));
      btg[4 * NBT + f] = vs * (0.25 * (Cft / (len * Cnn)));
      btg[5 * NBT + f] = vs * (0.25 * (1.0 / len));
      rxb[f] = vs * (1.0 / ((X(i + 1, j + 1) + X(i + 1, j)) / 2));
    }
  for (long k = 0; k < N; ++k) rvol[k] = 1.0 / m.vol[k];
  gvis.assign(N, 0.0);
  // max(4/3, gamma/Pr) / Re times the viscous CFL factor, over the volume once more: the
  // viscous rate the CFL kernel adds to the convective one before dividing by the volume
  const double kv = std::fmax(4.0 / 3.0, c.gamma / c.Pr) / c.Re;
  for (int j = 0; j < neta; ++j)
    for (int i = 0; i < nchi; ++i) {
      const long k = i + (long)j * nchi;
      const double Axi = 0.5 * (m.lr_a[i + (long)j * (nchi + 1)] + m.lr_a[i + 1 + (long)j * (nchi + 1)]);
      const double Aeta = 0.5 * (m.bt_a[i + (long)j * nchi] + m.bt_a[i + (long)(j + 1) * nchi]);
      gvis[k] = kv * (2 * (Axi * Axi + Aeta * Aeta) / m.vol[k]) / m.vol[k];
    }
}

int enqueue_step(hymor_ctx* ctx, bool with_events) {
  DevCtx& d = ctx->d;
  cudaStream_t st = ctx->stream, sx = ctx->side;
  const hymor_config& c = d.cfg;
  const bool shock = c.shock_enabled;
  const double wA[4] = {1.0 / 6, 1.0 / 3, 1.0 / 3, 1.0 / 6};
  const double wY[4] = {0.5, 0.5, 1.0, 0.0};
  double* const F[4] = {d.F[0], d.F[1], d.F[2], d.F[3]};
  int nf = 0, nj = 0;
  auto fork = [&]() -> int {  // side stream waits for the work enqueued so far on the main stream
    CU(cudaEventRecord(ctx->fork_ev[nf], st));
    CU(cudaStreamWaitEvent(sx, ctx->fork_ev[nf], 0));
    ++nf;
    return 0;
  };
  auto join = [&]() -> int {  // main stream waits for the side stream
    CU(cudaEventRecord(ctx->join_ev[nj], sx));
    CU(cudaStreamWaitEvent(st, ctx->join_ev[nj], 0));
    ++nj;
    return 0;
  };
  auto ev_on = [&](int k, cudaStream_t s) -> int {
    // cudaEventRecordExternal makes a real event-record node under stream capture
    if (with_events) CU(cudaEventRecordWithFlags(ctx->cap_ev[k], s, cudaEventRecordExternal));
    return 0;
  };
  auto ev = [&](int k) -> int { return ev_on(k, st); };
  CU(cudaMemsetAsync(d.scal + kCmax, 0, 3 * sizeof(double), st));
  TRY(ev(20));
  if (c.rk_variant == 0) {
    // Third stream: the first fit reads only the shock points of S, which nothing before
    // the first jump kernel changes, so it runs beside the flow cells and the CFL; the
    // first stage's jump and boundary kernels follow it there.
    CU(cudaEventRecord(ctx->fit_fork, st));
    CU(cudaStreamWaitEvent(ctx->fit, ctx->fit_fork, 0));
    launch_spline(d, false, true, ctx->fit);
    if (shock) launch_flow_cells(d, st);
    // Side stream: the tile classes and the CFL reduction beside the first stage update,
    // and every later smoothing-spline fit one stage early (a fit needs only the shock
    // points, which the previous stage's jump kernel moved); then per stage the jump +
    // boundary kernels beside the flux of the interior tiles.
    TRY(fork());
    launch_classify_tiles(d, sx);
    CU(cudaEventRecord(ctx->cls_ev, sx));
    // The CFL reduction on a stream of the lowest priority: its full-grid kernels would
    // otherwise take the block slots that the interior flux leaves free ahead of the first
    // stage's jump and boundary kernels, which the boundary-class flux waits for; dt is
    // needed only by the first MOVE_SHOCK and the second stage update. With shock fitting
    // the step recomputes the sound speed for the CFL maximum only (and the outflow_NRCBC
    // lines); the full field is recomputed when next needed.
    CU(cudaEventRecord(ctx->cfl_fork, st));
    CU(cudaStreamWaitEvent(ctx->cfl, ctx->cfl_fork, 0));
    if (shock && d.cfl_screen) {
      launch_cfl_screened(d, ctx->cfl);
    } else {
      launch_sound_cmax(d, shock, ctx->cfl, true);
      launch_cfl(d, ctx->cfl);
    }
    CU(cudaEventRecord(ctx->cfl_ev, ctx->cfl));
    TRY(ev(16));
    launch_update_thermo(d, 0, 0, 0, st);
    for (int k = 0; k < 4; ++k) {
      cudaStream_t sj = sx;  // the stream of this stage's jump and boundary kernels
      if (k == 0) {
        // The first stage's jump and boundary kernels need no time step (only MOVE_SHOCK
        // does): they run on the fit stream beside the CFL, and the move follows the CFL.
        sj = ctx->fit;
        CU(cudaEventRecord(ctx->u0_ev, st));
        CU(cudaStreamWaitEvent(sj, ctx->u0_ev, 0));
        CU(cudaStreamWaitEvent(sj, ctx->cls_ev, 0));  // the tile lists, for the flux below
        launch_columns_bc(d, false, false, wY[0], wA[0], 0, true, true, sj);
      } else {
        TRY(ev(16 + k));
        launch_update_thermo(d, 1, wY[k - 1], wA[k - 1], st);
        TRY(fork());
        launch_columns_bc(d, false, shock, wY[k], wA[k], 0, true, true, sx);
      }
      // the shock/boundary-class flux on its own stream as soon as the jump and boundary
      // kernels are done, beside the rest of the interior-class flux
      CU(cudaEventRecord(ctx->c1_fork[k], sj));
      CU(cudaStreamWaitEvent(ctx->c1, ctx->c1_fork[k], 0));
      TRY(ev_on(4 * k + 2, ctx->c1));
      launch_flux_class(d, false, F, 1, ctx->c1, 0, d.step_ffv != 0);
      TRY(ev_on(4 * k + 3, ctx->c1));
      CU(cudaEventRecord(ctx->c1_join[k], ctx->c1));
      if (k == 0) {
        CU(cudaStreamWaitEvent(sx, ctx->c1_fork[0], 0));
        CU(cudaStreamWaitEvent(sx, ctx->cfl_ev, 0));
        launch_move_shock(d, false, wY[0], wA[0], sx);
      }
      // next fit (stage k+1 on Y, or the step-end fit on S) overlaps this stage's remaining work
      launch_spline(d, k == 3, false, sx);
      TRY(ev(4 * k));
      // the interior flux leaves spare block slots per SM (flux_spare) to the side-stream
      // kernels and the shock/boundary-class flux
      if (k == 0) CU(cudaStreamWaitEvent(st, ctx->cls_ev, 0));
      launch_flux_class(d, false, F, 0, st, d.flux_spare, d.step_ffv != 0);
      TRY(ev(4 * k + 1));
      CU(cudaStreamWaitEvent(st, ctx->c1_join[k], 0));
      if (k == 0) CU(cudaStreamWaitEvent(st, ctx->cfl_ev, 0));  // dt, for the next stage update
    }
    launch_update_thermo(d, 2, 0, wA[3], st);
    TRY(join());
    launch_columns_bc(d, true, false, 0, 0, 1, true, true, st);
  } else {
    if (shock) launch_flow_cells(d, st);
    launch_sound_cmax(d, shock, st);
    launch_cfl(d, st);
    launch_snapshot(d, st);
    TRY(ev(16));
    launch_update_thermo(d, 0, 0, 0, st);
    launch_shock_bc(d, false, true, shock, 0.0, wA[0], 0, st);
    TRY(ev(0));
    launch_flux_class(d, false, F, -1, st, 0, d.step_ffv != 0);
    TRY(ev(1));
    TRY(ev(2));
    TRY(ev(3));
    for (int k = 1; k < 4; ++k) {
      TRY(ev(16 + k));
      launch_classical_stage(d, wY[k - 1], st);
      launch_update_thermo(d, 5, 0, wA[k - 1], st);
      launch_shock_bc(d, false, false, shock, 0.0, wA[k], 0, st);
      TRY(ev(4 * k));
      launch_flux_class(d, false, F, -1, st, 0, d.step_ffv != 0);
      TRY(ev(4 * k + 1));
      TRY(ev(4 * k + 2));
      TRY(ev(4 * k + 3));
    }
    launch_update_thermo(d, 2, 0, wA[3], st);
    launch_shock_bc(d, true, false, false, 0, 0, 1, st);
  }
  launch_fill_minrho(d, true, st);
  TRY(ev(21));
  CU(cudaGetLastError());
  return 0;
}

int build_graph(hymor_ctx* ctx) {
  if (ctx->gexec) return 0;
  CU(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int r = enqueue_step(ctx, true);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (r) return r;
  if (e != cudaSuccess) return fail(ctx, HYMOR_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  ctx->graph = g;
  // per-node priorities: the kernels keep the priority of the stream they were captured on
  // (the shock chain and the boundary-class flux above the interior flux, the CFL reduction
  // below it); without the flag every node runs at the launch stream's priority
  CU(cudaGraphInstantiate(&ctx->gexec, g, cudaGraphInstantiateFlagUseNodePriority));
  // map the event-record nodes to their flux-launch slots
  size_t nn = 0;
  CU(cudaGraphGetNodes(g, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  CU(cudaGraphGetNodes(g, nodes.data(), &nn));
  ctx->step_kernels = 0;
  for (auto n : nodes) {
    cudaGraphNodeType ty;
    CU(cudaGraphNodeGetType(n, &ty));
    if (ty == cudaGraphNodeTypeKernel) ++ctx->step_kernels;
    if (ty != cudaGraphNodeTypeEventRecord) continue;
    cudaEvent_t ev;
    CU(cudaGraphEventRecordNodeGetEvent(n, &ev));
    for (int k = 0; k < hymor_ctx_s::kEv; ++k)
      if (ctx->cap_ev[k] == ev) ctx->ev_nodes[k] = n;
  }
  return 0;
}

// TMA descriptors of the ghosted planes the flux halo reads (kernels.h, DevCtx::tmS ..): 2-D
// (Nchi + 2) x (Neta + 2) FP64 planes, boxes of 36 x (rows + 2) for tiles of 8 and 16 rows.
// The encoder is the driver's cuTensorMapEncodeTiled, reached through the runtime's entry-
// point query (no link against libcuda). Returns 1 when every descriptor was made.
int make_flux_maps(DevCtx& d) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return 0;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t pitch = (cuuint64_t)(d.nchi + 2) * sizeof(double);
  if (pitch % 16) return 0;  // the row pitch of a TMA tensor is a multiple of 16 bytes
  const cuuint64_t dims[2] = {(cuuint64_t)d.nchi + 2, (cuuint64_t)d.neta + 2};
  const cuuint64_t strides[1] = {pitch};
  const cuuint32_t estr[2] = {1, 1};
  const int rows[2] = {8, 16};
  auto one = [&](CUtensorMap* m, const double* base, int r) {
    const cuuint32_t box[2] = {36, (cuuint32_t)r + 2};
    return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  for (int ri = 0; ri < 2; ++ri) {
    const double* sp[4] = {d.S.rho, d.S.ru, d.S.rv, d.S.rE};
    const double* yp[4] = {d.Y.rho, d.Y.ru, d.Y.rv, d.Y.rE};
    for (int v = 0; v < 4; ++v)
      if (!one(&d.tmS[ri][v], sp[v], rows[ri]) || !one(&d.tmY[ri][v], yp[v], rows[ri])) return 0;
    if (!one(&d.tmP[ri], d.p, rows[ri]) || !one(&d.tmT[ri], d.T, rows[ri])) return 0;
  }
  return 1;
}

int check_err_words(hymor_ctx* ctx, const unsigned* h) {
  if (h[kErrFlags] & kBitTimeout)
    return fail(ctx, HYMOR_ERR_TIMEOUT, "a bounded wait for a TMA transfer of the flux halo gave up");
  if (h[kErrFlags] & kBitShockRange)
    return fail(ctx, HYMOR_ERR_SHOCK_RANGE, "shocked cell outside rows 2..Neta-1 (the shock left the mesh)");
  if (h[kErrFlags] & kBitNumeric)
    return fail(ctx, HYMOR_ERR_NUMERIC, "non-positive density or pressure, or NaN, in the flow field");
  return 0;
}

int read_err(hymor_ctx* ctx) {
  unsigned h[kErrCount];
  CU(cudaMemcpyAsync(h, ctx->d.err, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return check_err_words(ctx, h);
}

int set_device(hymor_ctx* ctx) {
  CU(cudaSetDevice(ctx->device));
  return 0;
}

// State layout shared by the device block and the pinned staging buffer: each plane is
// padded to a multiple of 32 doubles (256 bytes).
//   header: pts x, y, chi, eta (np doubles each), scalars (kScalPitch doubles), cell_idx (n int32)
constexpr size_t kScalPitch = 32;
size_t state_pitch(size_t n) { return (n + 31) & ~size_t(31); }
size_t header_doubles(size_t n) { return 4 * state_pitch(n) + kScalPitch + (n + 1) / 2; }
size_t stage_bytes(int n) { return header_doubles(n) * sizeof(double) + kErrCount * sizeof(unsigned); }

void drop_step_graph(hymor_ctx* ctx);

// The stored flux s["flux"] is no longer all zero: a step graph captured while it was
// (whose CFL kernel skips the stored-flux term) is dropped and captured again.
void stored_flux_written(hymor_ctx* ctx) {
  if (!ctx->d.sf_zero) return;
  ctx->d.sf_zero = 0;
  drop_step_graph(ctx);
}

// The next step captures its graph again (its launches changed).
void drop_step_graph(hymor_ctx* ctx) {
  if (ctx->gexec) {
    cudaStreamSynchronize(ctx->stream);
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  if (ctx->graph) {
    cudaGraphDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  for (auto& n : ctx->ev_nodes) n = nullptr;
}

// A step with shock fitting (Julia RK4 variant) computes the sound speed only where it
// reads it (its maximum and the outflow_NRCBC lines): the full field is stale afterwards.
void mark_sound_after_steps(hymor_ctx* ctx, int nsteps) {
  if (nsteps > 0 && ctx->d.cfg.shock_enabled && ctx->d.cfg.rk_variant == 0) ctx->a_stale = true;
}

// Computes the persistent sound speed of S if set_state left it stale, unless the work
// about to be enqueued recomputes it before reading it.
void refresh_sound(hymor_ctx* ctx, bool recomputed_anyway) {
  if (!ctx->a_stale) return;
  if (!recomputed_anyway) launch_sound_cmax(ctx->d, true, ctx->stream);
  ctx->a_stale = false;
}

// Validates a host state and enqueues its upload (no synchronisation): q in one 2-D copy,
// the shock points, scalars and shocked rows through the pinned staging buffer.
int enqueue_upload(hymor_ctx* ctx, const double* q, const double* pts_x, const double* pts_y,
                   const double* pts_chi, const double* pts_eta, const int32_t* cell_idx, double t,
                   const double* a) {
  if (!q) return fail(ctx, HYMOR_ERR_INVALID, "q is NULL");
  DevCtx& d = ctx->d;
  const size_t G = d.G, n = d.nchi;
  const bool shock = d.cfg.shock_enabled;
  if (shock && (!pts_x || !pts_y || !pts_chi || !pts_eta || !cell_idx))
    return fail(ctx, HYMOR_ERR_INVALID, "shock fitting needs the shock points and cell indices");
  const size_t np = state_pitch(n), Gp = state_pitch(G);
  double* sp = reinterpret_cast<double*>(ctx->stage);  // staged header, same layout as on the device
  double* sc = sp + 4 * np;
  int32_t* sci = reinterpret_cast<int32_t*>(sc + kScalPitch);
  for (size_t i = 0; i < n; ++i) {
    const int32_t v = cell_idx ? cell_idx[i] : d.neta + 1;
    if (cell_idx && shock && (v < 2 || v > d.neta - 1))
      return fail(ctx, HYMOR_ERR_SHOCK_RANGE, "cell_idx[%zu] = %d outside 2..Neta-1", i, v);
    sci[i] = v;
  }
  cudaStream_t st = ctx->stream;
  CU(cudaMemcpy2DAsync(d.S.rho, Gp * 8, q, G * 8, G * 8, 4, cudaMemcpyHostToDevice, st));
  const double* src[4] = {pts_x, pts_y, pts_chi, pts_eta};
  double* dst[4] = {d.Sp.x, d.Sp.y, d.Sp.chi, d.Sp.eta};
  const bool all_pts = pts_x && pts_y && pts_chi && pts_eta;
  for (int k = 0; k < 4; ++k)
    if (src[k]) std::memcpy(sp + k * np, src[k], n * 8);
  for (size_t k = 0; k < kScalPitch; ++k) sc[k] = 0;
  sc[kT] = t;
  if (all_pts) {
    CU(cudaMemcpyAsync(d.Sp.x, sp, header_doubles(n) * 8, cudaMemcpyHostToDevice, st));
  } else {  // keep the device copies of the points the caller did not pass
    for (int k = 0; k < 4; ++k)
      if (src[k]) CU(cudaMemcpyAsync(dst[k], sp + k * np, n * 8, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d.scal, sc, (header_doubles(n) - 4 * np) * 8, cudaMemcpyHostToDevice, st));
  }
  if (a) CU(cudaMemcpyAsync(d.aS, a, G * 8, cudaMemcpyHostToDevice, st));
  ctx->a_stale = !a;
  return 0;
}

// Enqueues the download of S (if q) and of the header into the staging buffer (and of the
// error word behind it, with_err); the caller synchronises and unpacks.
int enqueue_download(hymor_ctx* ctx, double* q, bool with_err) {
  DevCtx& d = ctx->d;
  const size_t G = d.G, n = d.nchi, Gp = state_pitch(G);
  cudaStream_t st = ctx->stream;
  if (q) CU(cudaMemcpy2DAsync(q, G * 8, d.S.rho, Gp * 8, G * 8, 4, cudaMemcpyDeviceToHost, st));
  // the error words follow the header on the device as in the staging buffer: one copy
  CU(cudaMemcpyAsync(ctx->stage, d.Sp.x, with_err ? stage_bytes(n) : header_doubles(n) * 8,
                     cudaMemcpyDeviceToHost, st));
  return 0;
}

void unpack_header(hymor_ctx* ctx, double* pts_x, double* pts_y, double* pts_chi, double* pts_eta,
                   int32_t* cell_idx, double* t, double* dt) {
  const size_t n = ctx->d.nchi, np = state_pitch(n);
  const double* sp = reinterpret_cast<const double*>(ctx->stage);
  const double* sc = sp + 4 * np;
  const int32_t* sci = reinterpret_cast<const int32_t*>(sc + kScalPitch);
  double* out[4] = {pts_x, pts_y, pts_chi, pts_eta};
  for (int k = 0; k < 4; ++k)
    if (out[k]) std::memcpy(out[k], sp + k * np, n * 8);
  if (cell_idx) std::memcpy(cell_idx, sci, n * 4);
  if (t) *t = sc[kT];
  if (dt) *dt = sc[kDt];
}

}  // namespace

extern "C" {

int hymor_ctx_create(const hymor_config* cfg, const hymor_mesh* mesh, hymor_ctx** out) {
  if (!out) return HYMOR_ERR_INVALID;
  *out = nullptr;
  if (!cfg || !mesh) return HYMOR_ERR_INVALID;
  hymor_ctx* ctx = new hymor_ctx_s();
  auto bail = [&](int r) {
    // keep the context so the caller can read the message, then let them destroy it
    *out = ctx;
    return r;
  };
  int r = check_config(ctx, cfg);
  if (r) return bail(r);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return bail(fail(ctx, HYMOR_ERR_CUDA, "no CUDA device visible"));
  cudaGetDevice(&ctx->device);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(ctx, HYMOR_ERR_CUDA, "stream creation failed"));
  flux_kernel_setup();
  DevCtx& d = ctx->d;
  d.cfg = *cfg;
  d.nchi = cfg->nchi;
  d.neta = cfg->neta;
  d.NI = d.nchi + 2;
  d.NJ = d.neta + 2;
  d.G = (long)d.NI * d.NJ;
  d.N = (long)d.nchi * d.neta;
  d.NLR = (long)(d.nchi + 1) * d.neta;
  d.NBT = (long)d.nchi * (d.neta + 1);
  const long NC = (long)(d.nchi + 1) * (d.neta + 1);
  DevMesh& m = d.m;
  m.nchi = d.nchi;
  m.neta = d.neta;
  double* tmp;
#define UP(field, n)                                                  \
  do {                                                                \
    if ((r = upload(ctx, &tmp, mesh->field, (n), #field))) return bail(r); \
    m.field = tmp;                                                    \
  } while (0)
  UP(lr_xn, d.NLR); UP(lr_yn, d.NLR); UP(lr_a, d.NLR);
  UP(bt_xn, d.NBT); UP(bt_yn, d.NBT); UP(bt_a, d.NBT);
  UP(vol, d.N); UP(x_ext, d.G); UP(y_ext, d.G);
  UP(x_corner, NC); UP(y_corner, NC); UP(chi1, d.nchi);
  if (cfg->axisymmetric) {
    UP(fb_area, d.N);
  } else {
    m.fb_area = nullptr;
  }
#undef UP
  m.fb_yn_front = mesh->fb_yn_front;
  m.fb_yn_back = mesh->fb_yn_back;
  {
    std::vector<double> lrg, btg, rvol, rxl, rxb, gvis;
    face_geometry(*cfg, *mesh, lrg, btg, rvol, rxl, rxb, gvis);
    {  // float-float copies of the planes the viscous terms read: nx, ny, g1, g2/4, 1/(4 len),
       // and the half area that scales them
      const long NLR = (long)(cfg->nchi + 1) * cfg->neta, NBT = (long)cfg->nchi * (cfg->neta + 1);
      const int planes[6] = {0, 1, 3, 4, 5, 2};
      auto split = [](const std::vector<double>& g, long nf, const int* pl) {
        std::vector<float2> out(6 * nf);
        for (int q = 0; q < 6; ++q)
          for (long f = 0; f < nf; ++f) {
            const double x = g[pl[q] * nf + f];
            const float h = (float)x;
            out[q * nf + f] = make_float2(h, (float)(x - (double)h));
          }
        return out;
      };
      const std::vector<float2> lf = split(lrg, NLR, planes), bf = split(btg, NBT, planes);
      float2 *q1 = nullptr, *q2 = nullptr;
      if (cudaMalloc(&q1, sizeof(float2) * lf.size()) != cudaSuccess ||
          cudaMalloc(&q2, sizeof(float2) * bf.size()) != cudaSuccess) {
        if (q1) cudaFree(q1);
        return bail(fail(ctx, HYMOR_ERR_CUDA, "float-float geometry allocation failed"));
      }
      ctx->allocs.push_back(q1);
      ctx->allocs.push_back(q2);
      if (cudaMemcpy(q1, lf.data(), sizeof(float2) * lf.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(q2, bf.data(), sizeof(float2) * bf.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(ctx, HYMOR_ERR_CUDA, "float-float geometry upload failed"));
      m.lrf = q1;
      m.btf = q2;
      // the normals times the half area, rounded once
      auto fold = [](const std::vector<double>& g, long nf) {
        std::vector<double> out(2 * nf);
        for (int q = 0; q < 2; ++q)
          for (long f = 0; f < nf; ++f) out[q * nf + f] = g[q * nf + f] * g[2 * nf + f];
        return out;
      };
      const std::vector<double> la = fold(lrg, NLR), ba = fold(btg, NBT);
      double *a1 = nullptr, *a2 = nullptr;
      if ((r = upload(ctx, &a1, la.data(), la.size(), "lr n A/2")) ||
          (r = upload(ctx, &a2, ba.data(), ba.size(), "bt n A/2")))
        return bail(r);
      m.lra = a1;
      m.bta = a2;
    }
    double *p1, *p2, *p3, *p4, *p5, *p6;
    if ((r = upload(ctx, &p1, lrg.data(), lrg.size(), "lr geometry"))) return bail(r);
    if ((r = upload(ctx, &p2, btg.data(), btg.size(), "bt geometry"))) return bail(r);
    if ((r = upload(ctx, &p3, rvol.data(), rvol.size(), "1/vol"))) return bail(r);
    if ((r = upload(ctx, &p4, rxl.data(), rxl.size(), "1/x lr"))) return bail(r);
    if ((r = upload(ctx, &p5, rxb.data(), rxb.size(), "1/x bt"))) return bail(r);
    if ((r = upload(ctx, &p6, gvis.data(), gvis.size(), "viscous CFL geometry"))) return bail(r);
    m.lrg = p1; m.btg = p2; m.rvol = p3; m.rx_lr = p4; m.rx_bt = p5; m.gvis = p6;
    // cell centres transposed (row index fastest), for scans along a chi column
    const int NI = cfg->nchi + 2, NJ = cfg->neta + 2;
    std::vector<double> xt((size_t)NI * NJ), yt((size_t)NI * NJ);
    for (int j = 0; j < NJ; ++j)
      for (int i = 0; i < NI; ++i) {
        xt[(size_t)i * NJ + j] = mesh->x_ext[i + (size_t)j * NI];
        yt[(size_t)i * NJ + j] = mesh->y_ext[i + (size_t)j * NI];
      }
    double *p7 = nullptr, *p8 = nullptr;
    if ((r = upload(ctx, &p7, xt.data(), xt.size(), "x centres")) || (r = upload(ctx, &p8, yt.data(), yt.size(), "y centres")))
      return bail(r);
    m.xt = p7; m.yt = p8;
  }
  auto cons = [&](Cons& q) -> int {
    TRY(dalloc(ctx, &q.rho, d.G)); TRY(dalloc(ctx, &q.ru, d.G));
    TRY(dalloc(ctx, &q.rv, d.G)); TRY(dalloc(ctx, &q.rE, d.G));
    return 0;
  };
  auto pts = [&](ShockPts& s) -> int {
    TRY(dalloc(ctx, &s.x, d.nchi)); TRY(dalloc(ctx, &s.y, d.nchi));
    TRY(dalloc(ctx, &s.chi, d.nchi)); TRY(dalloc(ctx, &s.eta, d.nchi));
    return 0;
  };
  {  // S in one block (4 planes, each 256-byte aligned) so that a state moves in one 2-D copy
    const size_t Gp = state_pitch(d.G);
    double* b = nullptr;
    if ((r = dalloc(ctx, &b, 4 * Gp))) return bail(r);
    d.S = Cons{b, b + Gp, b + 2 * Gp, b + 3 * Gp};
  }
  if ((r = cons(d.Y))) return bail(r);
  if (cfg->rk_variant == 1) {
    if ((r = cons(d.Yc)) || (r = pts(d.Ycp))) return bail(r);
  } else {
    d.Yc = d.S;
    d.Ycp = ShockPts{};
  }
  if ((r = dalloc(ctx, &d.p, d.G)) || (r = dalloc(ctx, &d.T, d.G)) || (r = dalloc(ctx, &d.aS, d.G)) ||
      (r = dalloc(ctx, &d.aY, d.G)))
    return bail(r);
  for (int v = 0; v < 4; ++v)
    if ((r = dalloc(ctx, &d.F[v], d.N)) || (r = dalloc(ctx, &d.SF[v], d.N))) return bail(r);
  {  // shock points of S, the scalars, the cell indices and the error words in one block,
     // laid out like the pinned staging buffer, so that they move in one copy
    const size_t np = state_pitch(d.nchi);
    double* b = nullptr;
    if ((r = dalloc(ctx, &b, header_doubles(d.nchi) + (kErrCount + 1) / 2))) return bail(r);
    d.Sp = ShockPts{b, b + np, b + 2 * np, b + 3 * np};
    d.scal = b + 4 * np;
    d.cell_idx = reinterpret_cast<int*>(b + 4 * np + kScalPitch);
    d.err = reinterpret_cast<unsigned*>(b + header_doubles(d.nchi));
  }
  if ((r = pts(d.Yp))) return bail(r);
  if ((r = dalloc(ctx, &d.beta, 2L * d.nchi)) ||
      (r = dalloc(ctx, &d.speed_x, d.nchi)) || (r = dalloc(ctx, &d.speed_y, d.nchi)) ||
      (r = dalloc(ctx, &d.rel, d.nchi)) || (r = dalloc(ctx, &d.spl, 17 * (long)d.nchi + 16)) ||
      (r = dalloc(ctx, &d.tiles, 2 + 2 * (long)flux_tiles_max(d))) ||
      (r = dalloc(ctx, &d.ticket, 6L)) ||
      (r = dalloc(ctx, &d.cflw, d.NLR + d.NBT)))
    return bail(r);
  if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || d.sms < 1)
    return bail(fail(ctx, HYMOR_ERR_CUDA, "multiprocessor count"));
  d.coef = nullptr;
  d.jwork = nullptr;
  d.sj = ShockJac{};
  d.up_cols = nullptr;
  d.bq = nullptr;
  d.bs = nullptr;
  d.brows = nullptr;
  d.res_up = nullptr;
  d.bwork = nullptr;
  d.sf_zero = 1;  // the flux arrays are allocated zeroed
  d.step_ffv = 1;
  d.expm_ff = 1;
  d.cfl_screen = 1;
  d.flux_rows = 4;  // the split tiling
  d.flux_spare = 1;
  d.tma = make_flux_maps(d);
  ctx->tma_able = d.tma;
  for (int k = 0; k < hymor_ctx_s::kEv; ++k)
    if (cudaEventCreate(&ctx->cap_ev[k]) != cudaSuccess) return bail(fail(ctx, HYMOR_ERR_CUDA, "event"));
  for (int k = 0; k < 8; ++k)  // 5 forks and 5 joins per step
    if (cudaEventCreateWithFlags(&ctx->fork_ev[k], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->join_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(ctx, HYMOR_ERR_CUDA, "event"));
  {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->fit, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->cfl, cudaStreamNonBlocking, lo) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->c1, cudaStreamNonBlocking, hi) != cudaSuccess)
      return bail(fail(ctx, HYMOR_ERR_CUDA, "side stream creation failed"));
    for (int k = 0; k < 4; ++k)
      if (cudaEventCreateWithFlags(&ctx->c1_fork[k], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&ctx->c1_join[k], cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(ctx, HYMOR_ERR_CUDA, "event"));
    if (cudaEventCreateWithFlags(&ctx->fit_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fit_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->u0_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->cfl_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->cls_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->cfl_fork, cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(ctx, HYMOR_ERR_CUDA, "event"));
  }
  if (cudaMallocHost(&ctx->stage, stage_bytes(d.nchi)) != cudaSuccess)
    return bail(fail(ctx, HYMOR_ERR_CUDA, "pinned staging allocation failed"));
  cudaEventCreate(&ctx->t0);
  cudaEventCreate(&ctx->t1);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return bail(fail(ctx, HYMOR_ERR_CUDA, "create: %s", cudaGetErrorString(e)));
  *out = ctx;
  return 0;
}

int hymor_ctx_destroy(hymor_ctx* ctx) {
  if (!ctx) return HYMOR_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  linear_state_release(ctx->linear_state);
  if (ctx->d.res_up) cudaFree(ctx->d.res_up);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  for (auto e : ctx->cap_ev)
    if (e) cudaEventDestroy(e);
  for (auto e : ctx->fork_ev)
    if (e) cudaEventDestroy(e);
  for (auto e : ctx->join_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->fit_fork) cudaEventDestroy(ctx->fit_fork);
  if (ctx->fit_join) cudaEventDestroy(ctx->fit_join);
  if (ctx->u0_ev) cudaEventDestroy(ctx->u0_ev);
  if (ctx->cfl_ev) cudaEventDestroy(ctx->cfl_ev);
  if (ctx->cls_ev) cudaEventDestroy(ctx->cls_ev);
  if (ctx->cfl_fork) cudaEventDestroy(ctx->cfl_fork);
  for (auto e : ctx->c1_fork)
    if (e) cudaEventDestroy(e);
  for (auto e : ctx->c1_join)
    if (e) cudaEventDestroy(e);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->fit) cudaStreamDestroy(ctx->fit);
  if (ctx->cfl) cudaStreamDestroy(ctx->cfl);
  if (ctx->c1) cudaStreamDestroy(ctx->c1);
  for (auto e : ctx->prof_ev) cudaEventDestroy(e);
  if (ctx->t0) cudaEventDestroy(ctx->t0);
  if (ctx->t1) cudaEventDestroy(ctx->t1);
  for (void* p : ctx->allocs) cudaFree(p);
  if (ctx->flush_buf) cudaFree(ctx->flush_buf);
  if (ctx->stage) cudaFreeHost(ctx->stage);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return 0;
}

const char* hymor_last_error(const hymor_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int hymor_set_state(hymor_ctx* ctx, const double* q, const double* pts_x, const double* pts_y,
                    const double* pts_chi, const double* pts_eta, const int32_t* cell_idx, double t,
                    const double* a) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  TRY(enqueue_upload(ctx, q, pts_x, pts_y, pts_chi, pts_eta, cell_idx, t, a));
  CU(cudaStreamSynchronize(ctx->stream));
  CU(cudaGetLastError());
  return 0;
}

int hymor_get_state(hymor_ctx* ctx, double* q, double* pts_x, double* pts_y, double* pts_chi,
                    double* pts_eta, int32_t* cell_idx, double* t, double* dt) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  TRY(enqueue_download(ctx, q, false));
  CU(cudaStreamSynchronize(ctx->stream));
  unpack_header(ctx, pts_x, pts_y, pts_chi, pts_eta, cell_idx, t, dt);
  return 0;
}

int hymor_advect(hymor_ctx* ctx, int nsteps, double* q, double* pts_x, double* pts_y, double* pts_chi,
                 double* pts_eta, int32_t* cell_idx, double* t) {
  if (!ctx || !t) return HYMOR_ERR_INVALID;
  if (nsteps < 0) return fail(ctx, HYMOR_ERR_INVALID, "nsteps < 0");
  TRY(set_device(ctx));
  TRY(build_graph(ctx));
  TRY(enqueue_upload(ctx, q, pts_x, pts_y, pts_chi, pts_eta, cell_idx, *t, nullptr));
  if (nsteps > 0) refresh_sound(ctx, ctx->d.cfg.shock_enabled);
  for (int s = 0; s < nsteps; ++s) CU(cudaGraphLaunch(ctx->gexec, ctx->stream));
  mark_sound_after_steps(ctx, nsteps);
  TRY(enqueue_download(ctx, q, true));
  CU(cudaStreamSynchronize(ctx->stream));
  unpack_header(ctx, pts_x, pts_y, pts_chi, pts_eta, cell_idx, t, nullptr);
  return check_err_words(ctx, reinterpret_cast<const unsigned*>(ctx->stage + header_doubles(ctx->d.nchi) * 8));
}

int hymor_residual(hymor_ctx* ctx, double* flux) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  DevCtx& d = ctx->d;
  cudaStream_t st = ctx->stream;
  launch_update_thermo(d, 3, 0, 0, st);
  launch_sound_cmax(d, true, st);
  ctx->a_stale = false;
  d.up_cols = d.res_up;  // rho_0_upstream_p of the reference's Dict, when set
  launch_shock_bc(d, true, false, false, 0, 0, 1, st);
  d.up_cols = nullptr;
  double* const SF[4] = {d.SF[0], d.SF[1], d.SF[2], d.SF[3]};
  launch_flux(d, true, SF, st);
  stored_flux_written(ctx);
  CU(cudaGetLastError());
  if (flux)
    for (int v = 0; v < 4; ++v)
      CU(cudaMemcpyAsync(flux + v * d.N, d.SF[v], d.N * 8, cudaMemcpyDeviceToHost, st));
  return read_err(ctx);
}

int hymor_set_upstream(hymor_ctx* ctx, const double* cols) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  DevCtx& d = ctx->d;
  if (!cols) {
    if (d.res_up) {
      CU(cudaStreamSynchronize(ctx->stream));
      CU(cudaFree(d.res_up));
    }
    d.res_up = nullptr;
    return 0;
  }
  if (!d.res_up) CU(cudaMalloc(&d.res_up, sizeof(double) * 4 * d.nchi));
  CU(cudaMemcpyAsync(d.res_up, cols, sizeof(double) * 4 * d.nchi, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return 0;
}

int hymor_set_flux(hymor_ctx* ctx, const double* flux) {
  if (!ctx || !flux) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  for (int v = 0; v < 4; ++v)
    CU(cudaMemcpyAsync(ctx->d.SF[v], flux + v * ctx->d.N, ctx->d.N * 8, cudaMemcpyHostToDevice, ctx->stream));
  stored_flux_written(ctx);
  CU(cudaStreamSynchronize(ctx->stream));
  return 0;
}

int hymor_step(hymor_ctx* ctx, int nsteps) {
  if (!ctx) return HYMOR_ERR_INVALID;
  if (nsteps < 0) return fail(ctx, HYMOR_ERR_INVALID, "nsteps < 0");
  TRY(set_device(ctx));
  TRY(build_graph(ctx));
  if (nsteps > 0) refresh_sound(ctx, ctx->d.cfg.shock_enabled);  // the step recomputes it with shock fitting
  for (int s = 0; s < nsteps; ++s) {
    if (ctx->profile) {
      for (int k = 0; k < hymor_ctx_s::kEv; ++k) {
        cudaEvent_t ev;
        CU(cudaEventCreate(&ev));
        ctx->prof_ev.push_back(ev);
        if (ctx->ev_nodes[k]) CU(cudaGraphExecEventRecordNodeSetEvent(ctx->gexec, ctx->ev_nodes[k], ev));
      }
      ctx->prof_steps++;
    }
    CU(cudaGraphLaunch(ctx->gexec, ctx->stream));
  }
  mark_sound_after_steps(ctx, nsteps);
  return read_err(ctx);
}

int hymor_bench_steps(hymor_ctx* ctx, int nsteps, uint64_t flush_bytes, float* ms) {
  if (!ctx || nsteps < 0) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  TRY(build_graph(ctx));
  if (flush_bytes > ctx->flush_bytes) {
    if (ctx->flush_buf) CU(cudaFree(ctx->flush_buf));
    ctx->flush_buf = nullptr;
    CU(cudaMalloc(&ctx->flush_buf, flush_bytes));
    ctx->flush_bytes = flush_bytes;
  }
  if (nsteps > 0) refresh_sound(ctx, ctx->d.cfg.shock_enabled);
  std::vector<cudaEvent_t> ev(2 * (size_t)nsteps);
  for (auto& e : ev) CU(cudaEventCreate(&e));
  for (int s = 0; s < nsteps; ++s) {
    if (flush_bytes) CU(cudaMemsetAsync(ctx->flush_buf, s & 0xff, flush_bytes, ctx->stream));
    if (ctx->profile) {
      for (int k = 0; k < hymor_ctx_s::kEv; ++k) {
        cudaEvent_t e;
        CU(cudaEventCreate(&e));
        ctx->prof_ev.push_back(e);
        if (ctx->ev_nodes[k]) CU(cudaGraphExecEventRecordNodeSetEvent(ctx->gexec, ctx->ev_nodes[k], e));
      }
      ctx->prof_steps++;
    }
    CU(cudaEventRecord(ev[2 * s], ctx->stream));
    CU(cudaGraphLaunch(ctx->gexec, ctx->stream));
    CU(cudaEventRecord(ev[2 * s + 1], ctx->stream));
  }
  mark_sound_after_steps(ctx, nsteps);
  CU(cudaStreamSynchronize(ctx->stream));
  double tot = 0;
  for (int s = 0; s < nsteps; ++s) {
    float v = 0;
    CU(cudaEventElapsedTime(&v, ev[2 * s], ev[2 * s + 1]));
    tot += v;
  }
  for (auto e : ev) cudaEventDestroy(e);
  if (ms) *ms = (float)tot;
  return read_err(ctx);
}

int hymor_autotune(hymor_ctx* ctx, int steps, int32_t* choice, float* ms_per_step) {
  if (!ctx || steps < 1 || !choice) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  DevCtx& d = ctx->d;
  cudaStream_t st = ctx->stream;
  // what a step changes, saved so that every candidate starts from the same state and the
  // context leaves the tuning as it entered it
  struct Part {
    void* p;
    size_t bytes;
  };
  const size_t n = (size_t)d.nchi;
  const Part parts[] = {
      {d.S.rho, sizeof(double) * d.G}, {d.S.ru, sizeof(double) * d.G}, {d.S.rv, sizeof(double) * d.G},
      {d.S.rE, sizeof(double) * d.G},  {d.aS, sizeof(double) * d.G},   {d.Sp.x, sizeof(double) * n},
      {d.Sp.y, sizeof(double) * n},    {d.Sp.chi, sizeof(double) * n}, {d.Sp.eta, sizeof(double) * n},
      {d.cell_idx, sizeof(int) * n},   {d.beta, sizeof(double) * 2 * n}, {d.speed_x, sizeof(double) * n},
      {d.speed_y, sizeof(double) * n}, {d.rel, sizeof(double) * n},    {d.scal, sizeof(double) * kCount},
      {d.err, sizeof(unsigned) * kErrCount}};
  size_t total = 0;
  for (const Part& q : parts) total += (q.bytes + 255) & ~(size_t)255;
  unsigned char* save = nullptr;
  CU(cudaMalloc(&save, total));
  auto copy = [&](bool store) -> int {
    size_t off = 0;
    for (const Part& q : parts) {
      unsigned char* dst = store ? save + off : static_cast<unsigned char*>(q.p);
      const unsigned char* src = store ? static_cast<const unsigned char*>(q.p) : save + off;
      CU(cudaMemcpyAsync(dst, src, q.bytes, cudaMemcpyDeviceToDevice, st));
      off += (q.bytes + 255) & ~(size_t)255;
    }
    return 0;
  };
  const bool stale = ctx->a_stale;
  const int rows0 = d.flux_rows, spare0 = d.flux_spare, tma0 = d.tma;
  int r = copy(true);
  // candidates: halo by TMA or by thread loads x tile rows (8, 16, or the split 4/8) x spare
  // block slots per SM of the interior grid (without TMA descriptors only the thread-load half)
  const int rows_c[3] = {8, 16, 4}, spare_c[3] = {0, 1, 2};
  float best = 0;
  int bi = -1, c = 0;
  for (int a = 0; a < 6 && !r; ++a)
    for (int b = 0; b < 3 && !r; ++b, ++c) {
      if (ms_per_step) ms_per_step[c] = 0;
      if (a >= 3 && !ctx->tma_able) continue;
      d.tma = a >= 3;
      d.flux_rows = rows_c[a % 3];
      d.flux_spare = spare_c[b];
      drop_step_graph(ctx);
      float ms = 0;
      if ((r = copy(false))) break;
      ctx->a_stale = stale;
      if ((r = hymor_bench_steps(ctx, 1, 0, &ms))) break;  // capture and warm up
      if ((r = copy(false))) break;
      ctx->a_stale = stale;
      if ((r = hymor_bench_steps(ctx, steps, 0, &ms))) break;
      ms /= steps;
      if (ms_per_step) ms_per_step[c] = ms;
      if (bi < 0 || ms < best) {
        best = ms;
        bi = c;
      }
    }
  if (!r) r = copy(false);
  cudaStreamSynchronize(st);
  cudaFree(save);
  ctx->a_stale = stale;
  if (r || bi < 0) {
    d.flux_rows = rows0;
    d.flux_spare = spare0;
    d.tma = tma0;
    drop_step_graph(ctx);
    return r ? r : fail(ctx, HYMOR_ERR_CUDA, "autotune: no candidate ran");
  }
  d.tma = bi / 9;
  d.flux_rows = rows_c[(bi / 3) % 3];
  d.flux_spare = spare_c[bi % 3];
  drop_step_graph(ctx);
  choice[0] = d.flux_rows;
  choice[1] = d.flux_spare;
  choice[2] = d.tma;
  return 0;
}

int hymor_set_flux_tiling(hymor_ctx* ctx, int rows, int spare, int tma) {
  if (!ctx || (rows != 4 && rows != 8 && rows != 16) || spare < 0 || spare > 4 || tma < 0 || tma > 1) return HYMOR_ERR_INVALID;
  if (tma && !ctx->tma_able) return fail(ctx, HYMOR_ERR_INVALID, "no TMA descriptors for this grid (Nchi odd)");
  TRY(set_device(ctx));
  if (ctx->d.flux_rows != rows || ctx->d.flux_spare != spare || ctx->d.tma != tma) {
    ctx->d.flux_rows = rows;
    ctx->d.flux_spare = spare;
    ctx->d.tma = tma;
    drop_step_graph(ctx);
  }
  return 0;
}

int hymor_update_flow_cells(hymor_ctx* ctx) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  if (ctx->d.cfg.shock_enabled) {
    launch_flow_cells(ctx->d, ctx->stream);
    launch_sound_cmax(ctx->d, true, ctx->stream);
    ctx->a_stale = false;
  }
  CU(cudaGetLastError());
  return read_err(ctx);
}

int hymor_cfl_timestep(hymor_ctx* ctx, double* dt) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  DevCtx& d = ctx->d;
  refresh_sound(ctx, false);
  CU(cudaMemsetAsync(d.scal + kCmax, 0, 3 * sizeof(double), ctx->stream));
  launch_sound_cmax(d, false, ctx->stream);
  launch_cfl(d, ctx->stream);
  CU(cudaGetLastError());
  double sc[kCount];
  CU(cudaMemcpyAsync(sc, d.scal, sizeof sc, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (dt) *dt = sc[kDt];
  return 0;
}

int hymor_counters(hymor_ctx* ctx, int32_t* rho_limited, int32_t* rh_warnings) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  unsigned h[kErrCount];
  CU(cudaMemcpyAsync(h, ctx->d.err, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (rho_limited) *rho_limited = (int32_t)h[kRhoLimited];
  if (rh_warnings) *rh_warnings = (int32_t)h[kRhWarn];
  return 0;
}

int hymor_set_step_viscous(hymor_ctx* ctx, int mode) {
  if (!ctx || mode < 0 || mode > 1) return HYMOR_ERR_INVALID;
  if (ctx->d.step_ffv != mode) {
    TRY(set_device(ctx));
    ctx->d.step_ffv = mode;
    drop_step_graph(ctx);
  }
  return 0;
}

int hymor_set_expm_arith(hymor_ctx* ctx, int mode) {
  if (!ctx || mode < 0 || mode > 1) return HYMOR_ERR_INVALID;
  ctx->d.expm_ff = mode;
  return 0;
}

int hymor_set_cfl_screen(hymor_ctx* ctx, int on) {
  if (!ctx || on < 0 || on > 1) return HYMOR_ERR_INVALID;
  if (ctx->d.cfl_screen != on) {
    TRY(set_device(ctx));
    ctx->d.cfl_screen = on;
    drop_step_graph(ctx);
  }
  return 0;
}

int hymor_step_kernels(hymor_ctx* ctx, int32_t* n) {
  if (!ctx || !n) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  TRY(build_graph(ctx));
  *n = ctx->step_kernels;
  return 0;
}

int hymor_timer_start(hymor_ctx* ctx) {
  if (!ctx) return HYMOR_ERR_INVALID;
  CU(cudaEventRecord(ctx->t0, ctx->stream));
  ctx->timer_running = 1;
  return 0;
}

int hymor_timer_stop(hymor_ctx* ctx, float* ms) {
  if (!ctx || !ctx->timer_running) return HYMOR_ERR_INVALID;
  CU(cudaEventRecord(ctx->t1, ctx->stream));
  CU(cudaEventSynchronize(ctx->t1));
  ctx->timer_running = 0;
  float v = 0;
  CU(cudaEventElapsedTime(&v, ctx->t0, ctx->t1));
  if (ms) *ms = v;
  return 0;
}

int hymor_profile_flux(hymor_ctx* ctx, int enable, float* total_ms, int32_t* launches) {
  if (!ctx) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  if (total_ms || launches) {
    CU(cudaStreamSynchronize(ctx->stream));
    double tot = 0;
    int n = 0;
    const size_t E = hymor_ctx_s::kEv;
    for (size_t s = 0; s + E <= ctx->prof_ev.size(); s += E)
      for (int k = 0; k < 4; ++k) {  // one residual evaluation per stage, in two launches
        // from the start of the interior-class flux to the later end of the two classes
        float v1 = 0, v2 = 0;
        CU(cudaEventElapsedTime(&v1, ctx->prof_ev[s + 4 * k], ctx->prof_ev[s + 4 * k + 1]));
        CU(cudaEventElapsedTime(&v2, ctx->prof_ev[s + 4 * k], ctx->prof_ev[s + 4 * k + 3]));
        tot += v1 > v2 ? v1 : v2;
        ++n;
      }
    if (total_ms) *total_ms = (float)tot;
    if (launches) *launches = n;
  }
  // point the graph's event nodes back at the capture events before releasing the
  // per-step events they reference
  if (ctx->gexec) {
    for (int k = 0; k < hymor_ctx_s::kEv; ++k)
      if (ctx->ev_nodes[k]) CU(cudaGraphExecEventRecordNodeSetEvent(ctx->gexec, ctx->ev_nodes[k], ctx->cap_ev[k]));
  }
  CU(cudaStreamSynchronize(ctx->stream));
  for (auto e : ctx->prof_ev) cudaEventDestroy(e);
  ctx->prof_ev.clear();
  ctx->prof_steps = 0;
  ctx->profile = enable != 0;
  return 0;
}

int hymor_profile_phases(hymor_ctx* ctx, float* ms) {
  if (!ctx || !ms) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  CU(cudaStreamSynchronize(ctx->stream));
  const size_t E = hymor_ctx_s::kEv;
  for (int k = 0; k < 18; ++k) ms[k] = 0;
  int steps = 0;
  auto dt = [&](size_t s, int a, int b, float& acc) -> int {
    float v = 0;
    CU(cudaEventElapsedTime(&v, ctx->prof_ev[s + a], ctx->prof_ev[s + b]));
    acc += v;
    return 0;
  };
  for (size_t s = 0; s + E <= ctx->prof_ev.size(); s += E, ++steps) {
    TRY(dt(s, 20, 16, ms[0]));
    for (int k = 0; k < 4; ++k) {
      TRY(dt(s, 16 + k, 4 * k, ms[1 + 4 * k]));          // stage update (+ fork)
      TRY(dt(s, 4 * k, 4 * k + 1, ms[2 + 4 * k]));       // flux, interior tiles
      TRY(dt(s, 4 * k, 4 * k + 2, ms[3 + 4 * k]));       // start of the shock/boundary-tile flux,
                                                          // after the interior flux's start
      TRY(dt(s, 4 * k + 2, 4 * k + 3, ms[4 + 4 * k]));   // flux, shock/boundary tiles
    }
    // from the later end of the last stage's two flux launches to the step end
    float e1 = 0, e2 = 0;
    TRY(dt(s, 13, 21, e1));
    TRY(dt(s, 15, 21, e2));
    ms[17] += e1 < e2 ? e1 : e2;
  }
  if (steps)
    for (int k = 0; k < 18; ++k) ms[k] /= steps;
  return 0;
}

int hymor_synchronize(hymor_ctx* ctx) {
  if (!ctx) return HYMOR_ERR_INVALID;
  CU(cudaStreamSynchronize(ctx->stream));
  return read_err(ctx);
}

int hymor_device_alloc(hymor_ctx* ctx, uint64_t bytes, void** dptr) {
  if (!ctx || !dptr) return HYMOR_ERR_INVALID;
  TRY(set_device(ctx));
  CU(cudaMalloc(dptr, bytes));
  return 0;
}

int hymor_device_free(hymor_ctx* ctx, void* dptr) {
  if (!ctx) return HYMOR_ERR_INVALID;
  CU(cudaFree(dptr));
  return 0;
}

int hymor_memcpy_h2d(hymor_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
  if (!ctx) return HYMOR_ERR_INVALID;
  CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return 0;
}

int hymor_memcpy_d2h(hymor_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
  if (!ctx) return HYMOR_ERR_INVALID;
  CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return 0;
}

int hymor_memcpy_d2d(hymor_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
  if (!ctx) return HYMOR_ERR_INVALID;
  CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return 0;
}

}  // extern "C"

// DevCtx accessor for linear.cu
namespace hymor {
DevCtx& ctx_dev(hymor_ctx* c) { return c->d; }
cudaStream_t ctx_stream(hymor_ctx* c) { return c->stream; }
int ctx_fail(hymor_ctx* c, int code, const char* msg) { return fail(c, code, "%s", msg); }
std::vector<void*>& ctx_allocs(hymor_ctx* c) { return c->allocs; }
void*& ctx_linear_state(hymor_ctx* c) { return c->linear_state; }
int ctx_select_device(hymor_ctx* c) { return cudaSetDevice(c->device) == cudaSuccess ? 0 : HYMOR_ERR_CUDA; }
}  // namespace hymor
