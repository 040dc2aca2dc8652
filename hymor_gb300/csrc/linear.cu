// Linearised residual on the device: coloured finite-difference Jacobian assembly
// into stencil blocks, the block-stencil matvec (and its transpose) and the
// Taylor propagator exp(A dt)^n used by the exponential-transform eigen solvers.
//
// Device layout of the Jacobian: 144 planes of N doubles (plane (q*4 + vout)*4 + vin,
// q = neighbour slot), so that consecutive threads (cells) read consecutive
// addresses. hymor_jacobian_get/set convert to the per-cell block layout of
// include/hymor.h.
#include <cmath>
#include <cstdio>
#include <vector>

#include <cooperative_groups.h>

#include <algorithm>

#include "ff.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace hymor {
DevCtx& ctx_dev(hymor_ctx* c);
cudaStream_t ctx_stream(hymor_ctx* c);
int ctx_fail(hymor_ctx* c, int code, const char* msg);
std::vector<void*>& ctx_allocs(hymor_ctx* c);
void*& ctx_linear_state(hymor_ctx* c);
void launch_shock_bc_flags(const DevCtx& d, bool on_S, bool copy_pts, bool do_shock, bool do_bc, int a_mode,
                           cudaStream_t st);

namespace {

constexpr int kMvThreads = 256;

// Threads per block of a matvec over `items` work items: 256, or fewer when that would
// leave SMs idle. One vector on a 100 x 80 grid is 8000 items: in 256-thread blocks they
// sit on 32 SMs, whose FP64 pipes then bound the matvec; in 64-thread blocks they spread
// over 125.
int mv_threads(long items, int sms) {
  if (items >= (long)sms * kMvThreads) return kMvThreads;
  const long per_sm = (items + sms - 1) / sms;
  const long t = ((per_sm + 31) / 32) * 32;
  return (int)(t < 32 ? 32 : t);
}
constexpr int kVecChunk = 4;

struct Wrap {
  int nchi, neta, per_chi, per_eta;
  // input cell of output (i, j) at offset (a, b); -1 if the reference assembles no entry
  __device__ __forceinline__ long nbr(int i, int j, int a, int b) const {
    int ii = i + a, jj = j + b;
    const bool wi = ii < 0 || ii >= nchi, wj = jj < 0 || jj >= neta;
    if ((wi && !per_chi) || (wj && !per_eta) || (wi && wj)) return -1;
    if (wi) ii = ii < 0 ? ii + nchi : ii - nchi;
    if (wj) jj = jj < 0 ? jj + neta : jj - neta;
    return (long)ii + (long)jj * nchi;
  }
};

Wrap make_wrap(const hymor_config& c) {
  return Wrap{c.nchi, c.neta, c.bc_chi0 == HYMOR_BC_PERIODIC && c.bc_chi1 == HYMOR_BC_PERIODIC,
              c.bc_eta0 == HYMOR_BC_PERIODIC && c.bc_eta1 == HYMOR_BC_PERIODIC};
}

// Y = S with variable `var` of every interior cell of colour `colour` (1..9, the
// pattern of GET_PERTURBATION_MATRIX, LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:959-983)
// raised by flow_cells * eps; then p, T of Y. shock_row = j > 0 raises instead the
// cell (i, sc_i - j) of every column by eps (the flow-to-shock-speed perturbations,
// :140-258).
struct PertArgs {
  Cons S, Y;
  double *p, *T;
  double* aY;
  int nrcbc;
  const int* cell_idx;
  double eps, gm1;
  int nchi, neta, var, colour, shock, shock_row;
};

__global__ void k_perturb_thermo(PertArgs a) {
  const int NI = a.nchi + 2;
  const long G = (long)NI * (a.neta + 2);
  const int si = (a.colour % 3 == 0) ? 3 : a.colour % 3;  // 1-based start in chi
  const int sj = (a.colour + 2) / 3;                       // 1-based start in eta
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < G; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)(k % NI), j = (int)(k / NI);
    double v[4] = {a.S.rho[k], a.S.ru[k], a.S.rv[k], a.S.rE[k]};
    if (a.var >= 0 && i >= 1 && i <= a.nchi && j >= 1 && j <= a.neta) {
      if (a.shock_row) {
        if (j == a.cell_idx[i - 1] - a.shock_row) v[a.var] += a.eps;
      } else {
        const bool hit = (i >= si) && ((i - si) % 3 == 0) && (j >= sj) && ((j - sj) % 3 == 0);
        const double flow = (!a.shock || j < a.cell_idx[i - 1]) ? 1.0 : 0.0;
        v[a.var] = v[a.var] + flow * (hit ? 1.0 : 0.0) * a.eps;
      }
    }
    a.Y.rho[k] = v[0]; a.Y.ru[k] = v[1]; a.Y.rv[k] = v[2]; a.Y.rE[k] = v[3];
    const double ir = 1.0 / v[0];
    const double ke = fma(v[1], v[1], v[2] * v[2]) * ir;
    const double eint = fma(-0.5, ke, v[3]);
    a.p[k] = eint * a.gm1;
    a.T[k] = eint * ir;
    if (a.nrcbc) {
      const int NJ = a.neta + 2;
      const bool nb = ((a.nrcbc & 1) && i == 1) || ((a.nrcbc & 2) && i == NI - 2) ||
                      ((a.nrcbc & 4) && j == 1) || ((a.nrcbc & 8) && j == NJ - 2);
      if (nb) a.aY[k] = sqrt((a.gm1 + 1) * (eint * a.gm1) / v[0]);
    }
  }
}

// coef[plane(q, vo, var)][m] = (Fp[vo][m] - Fb[vo][m]) / eps for every slot q whose
// input cell m + offset(q) has the perturbed colour (GET_OUTPUT_INDEXING_A11,
// LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:306-788; REMOVE_BASE_OUTPUT :935-946).
struct ScatArgs {
  const double* Fp[4];
  const double* Fb[4];
  double* coef;
  Wrap w;
  double inv_eps_dummy;
  double eps;
  int var, colour;
  long N;
};

__global__ void k_scatter(ScatArgs a) {
  const long N = a.N;
  const int si = (a.colour % 3 == 0) ? 3 : a.colour % 3;
  const int sj = (a.colour + 2) / 3;
  for (long m = blockIdx.x * (long)blockDim.x + threadIdx.x; m < N; m += (long)gridDim.x * blockDim.x) {
    const int i = (int)(m % a.w.nchi), j = (int)(m / a.w.nchi);
    double d[4];
#pragma unroll
    for (int vo = 0; vo < 4; ++vo) d[vo] = (a.Fp[vo][m] - a.Fb[vo][m]) / a.eps;
#pragma unroll
    for (int b = -1; b <= 1; ++b)
#pragma unroll
      for (int aa = -1; aa <= 1; ++aa) {
        const long n = a.w.nbr(i, j, aa, b);
        if (n < 0) continue;
        const int ni = (int)(n % a.w.nchi) + 1, nj = (int)(n / a.w.nchi) + 1;  // 1-based
        const bool hit = (ni >= si) && ((ni - si) % 3 == 0) && (nj >= sj) && ((nj - sj) % 3 == 0);
        if (!hit) continue;
        const int q = (b + 1) * 3 + (aa + 1);
#pragma unroll
        for (int vo = 0; vo < 4; ++vo) a.coef[((long)(q * 4 + vo) * 4 + a.var) * N + m] = d[vo];
      }
  }
}

// y_j = scale * (L x_j) (transpose 0) or scale * (Lᵀ x_j) (transpose 1); optionally
// acc_j += c_acc * y_j. Vectors: 4N each, column-major batch.
struct MvArgs {
  const double* coef;
  const double* X;
  double* Y;
  double* acc;
  double scale, c_acc;
  // a term of the previous matvec to add into acc first (acc += c_prev acc_prev), or null:
  // the propagator accumulates each Taylor term one matvec late, so that the first matvec
  // of a step can read acc as its input without a copy
  const double* acc_prev;
  double c_prev;
  // per-vector scale (k entries) replacing `scale`, or null: a batch of propagations with
  // different time steps (transient-growth horizons)
  const double* vscale;
  Wrap w;
  long N;
  long ld;  // vector stride (4N, or 4N + Nchi with the shock unknowns)
  int k, transpose;
};

// ST: the blocks exceed L2 and are read with streaming (evict-first) loads, which keep the
// vectors that every neighbour re-reads in L2; blocks that fit stay cached from one matvec
// of a propagation to the next (a compile-time choice: a branch per load slowed the loads)
template <bool ST>
__device__ __forceinline__ double ld_coef(const double* p) {
  return ST ? __ldcs(p) : *p;
}

// y = scale * A x (or A^T x), acc += c_acc y. The work items are (cell, chunk of
// kVecChunk vectors) pairs, cell fastest, over a grid-stride loop: a batch of vectors on
// a small grid still spreads over every SM (a 100 x 80 grid is 8000 cells, 64 vectors are
// 16 chunks of it), and neighbouring threads read neighbouring cells.
// Few cells x vectors (a small grid, one or a few vectors): one thread per (cell, output
// component, vector), the same FMA chain per output as matvec_multi (bit-identical). On
// GB300 one warp issues one FP64 instruction per ~76 cycles of its SM sub-partition, so a
// warp per 32 cells (148 FP64 instructions each, per vector) would bound a small grid's
// matvec by its own issue rate; a thread per output spreads the work over four times the
// warps per vector. The next neighbour block's coefficients and inputs are loaded while
// the current block's FMAs run.
template <bool ST>
__device__ __forceinline__ void matvec_one(const MvArgs& a) {
  const long N = a.N;
  const long outs = 4 * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < outs * a.k; t += (long)gridDim.x * blockDim.x) {
    const long vec = t / outs;
    const long w = t - vec * outs;
    const long m = w % N;
    const int comp = (int)(w / N);  // output component (v_out, or v_in of the transpose)
    const int i = (int)(m % a.w.nchi), j = (int)(m / a.w.nchi);
    const double* xv = a.X + vec * a.ld;
    double y = 0;
    double B[2][4], X[2][4];
    bool ok[2];
    auto load = [&](int q, int slot) {
      const int b = q / 3 - 1, aa = q % 3 - 1;
      long n, cell;  // input cell, and the cell that owns the block
      if (!a.transpose) {
        n = a.w.nbr(i, j, aa, b);
        cell = m;
      } else {
        // m is the input cell of output cell n = m - (aa, b); block slot of (aa, b)
        n = a.w.nbr(i, j, -aa, -b);
        cell = n;
      }
      ok[slot] = n >= 0;
      if (n >= 0) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          // row comp of the block (columns e), or column comp of it for the transpose
          const int plane = a.transpose ? q * 16 + e * 4 + comp : q * 16 + comp * 4 + e;
          B[slot][e] = ld_coef<ST>(a.coef + (long)plane * N + cell);
          X[slot][e] = xv[e * N + n];
        }
      }
    };
    load(0, 0);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const int c = q & 1;
      if (q + 1 < 9) load(q + 1, c ^ 1);
      if (!ok[c]) continue;
      y = fma(B[c][0], X[c][0], fma(B[c][1], X[c][1], fma(B[c][2], X[c][2], fma(B[c][3], X[c][3], y))));
    }
    const double val = (a.vscale ? a.vscale[vec] : a.scale) * y;
    const long o = vec * a.ld + comp * N + m;
    a.Y[o] = val;
    if (a.acc) {
      double r = a.acc[o];
      if (a.acc_prev) r = fma(a.acc_prev[o], a.c_prev, r);
      a.acc[o] = fma(val, a.c_acc, r);
    }
  }
}

// The thread-per-output path (matvec_one) when the cells x vectors are fewer than 32 per
// warp slot of 8 warps on every SM sub-partition; more of them already fill those slots
// with one thread per (cell, chunk of vectors) (matvec_multi, whose single pass over the
// 144 coefficients for a chunk of vectors is then cheaper).
__host__ __device__ inline long mv_one_limit(int sms) { return 8L * 32 * 4 * sms; }
// the Jacobian's blocks (144 per cell, 8 bytes each) larger than this many bytes take
// streaming loads in the matvecs (about a third of the L2, leaving the rest to the
// vectors); smaller blocks stay cached from one matvec of a propagation to the next
constexpr long kCoefStreamBytes = 48L << 20;
bool mv_one(long N, int k, int sms) { return N * k < mv_one_limit(sms); }

// Work items of a matvec over k vectors: (cell, output component, vector) on the
// thread-per-output path, (cell, chunk of kVecChunk vectors) otherwise.
long mv_items(long N, int k, int sms) {
  return mv_one(N, k, sms) ? 4 * N * k : N * ((k + kVecChunk - 1) / kVecChunk);
}

template <bool ST>
__device__ __forceinline__ void matvec_multi(const MvArgs& a) {
  const long N = a.N;
  const long n4 = a.ld;
  const int chunks = (a.k + kVecChunk - 1) / kVecChunk;
  const long items = N * chunks;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < items; w += (long)gridDim.x * blockDim.x) {
    const long m = w % N;
    const int i = (int)(m % a.w.nchi), j = (int)(m / a.w.nchi);
    {
      const int v0 = (int)(w / N) * kVecChunk;
      const int nv = min(kVecChunk, a.k - v0);
      double y[kVecChunk][4];
#pragma unroll
      for (int v = 0; v < kVecChunk; ++v)
#pragma unroll
        for (int c = 0; c < 4; ++c) y[v][c] = 0;
#pragma unroll
      for (int b = -1; b <= 1; ++b)
#pragma unroll
        for (int aa = -1; aa <= 1; ++aa) {
          long n;
          long cell;  // cell that owns the block
          int q;
          if (!a.transpose) {
            n = a.w.nbr(i, j, aa, b);
            cell = m;
            q = (b + 1) * 3 + (aa + 1);
          } else {
            // m is the input cell of output cell n = m - (aa, b); block slot of (aa, b)
            n = a.w.nbr(i, j, -aa, -b);
            cell = n;
            q = (b + 1) * 3 + (aa + 1);
          }
          if (n < 0) continue;
          double B[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) B[e] = ld_coef<ST>(a.coef + (long)(q * 16 + e) * N + cell);
          for (int v = 0; v < nv; ++v) {
            const double* x = a.X + (long)(v0 + v) * n4;
            const double x0 = x[n], x1 = x[N + n], x2 = x[2 * N + n], x3 = x[3 * N + n];
            if (!a.transpose) {
#pragma unroll
              for (int vo = 0; vo < 4; ++vo)
                y[v][vo] = fma(B[vo * 4 + 0], x0, fma(B[vo * 4 + 1], x1, fma(B[vo * 4 + 2], x2, fma(B[vo * 4 + 3], x3, y[v][vo]))));
            } else {
#pragma unroll
              for (int vi = 0; vi < 4; ++vi)
                y[v][vi] = fma(B[0 * 4 + vi], x0, fma(B[1 * 4 + vi], x1, fma(B[2 * 4 + vi], x2, fma(B[3 * 4 + vi], x3, y[v][vi]))));
            }
          }
        }
      for (int v = 0; v < nv; ++v) {
        double* yo = a.Y + (long)(v0 + v) * n4;
        const double sc = a.vscale ? a.vscale[v0 + v] : a.scale;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const double val = sc * y[v][c];
          yo[c * N + m] = val;
          if (a.acc) {
            double* ac = a.acc + (long)(v0 + v) * n4;
            double r = ac[c * N + m];
            if (a.acc_prev) r = fma(a.acc_prev[(long)(v0 + v) * n4 + c * N + m], a.c_prev, r);
            ac[c * N + m] = fma(val, a.c_acc, r);
          }
        }
      }
    }
  }
}

// ONE: the one-vector path (its own kernel, so that its registers do not lower the
// occupancy of the batched path)
template <bool ONE, bool ST>
__device__ __forceinline__ void matvec_cells(const MvArgs& a) {
  if (ONE) matvec_one<ST>(a);
  else matvec_multi<ST>(a);
}

template <bool ONE, bool ST>
__global__ void __launch_bounds__(kMvThreads) k_matvec(MvArgs a) { matvec_cells<ONE, ST>(a); }

// The whole Taylor propagation in one cooperative launch: the blocks are co-resident
// (cudaLaunchCooperativeKernel) and meet at a grid barrier after every matvec, instead of
// one kernel per matvec. Same per-cell arithmetic, in the same order, as launch_expm.
// vsteps (k entries, non-increasing, or null): vector c takes vsteps[c] steps, so that at
// step s only the first #{c : vsteps[c] > s} vectors advance (a contiguous prefix).
template <bool ONE, bool ST>
__global__ void __launch_bounds__(kMvThreads, 2) k_expm_coop(MvArgs base, int nsteps, int order, double* v,
                                                             double* t1, double* t2, double* vout,
                                                             const int* vsteps) {
  cg::grid_group grid = cg::this_grid();
  for (int s = 0; s < nsteps; ++s) {
    if (vsteps) {
      int ka = 0;
      while (ka < base.k && vsteps[ka] > s) ++ka;
      base.k = ka;
    }
    const long n = 4 * base.N * (long)base.k;
    // order >= 2: the first matvec reads vout itself and adds nothing to it, the second
    // adds the first term before its own (the same additions in the same order as adding
    // each term in its own matvec), so no copy vout -> v closes the step
    const bool late = order >= 2;
    const double* src = late ? vout : v;
    const double* prev = nullptr;
    double c_prev = 0;
    long fact = 1;
    for (int j = 1; j <= order; ++j) {
      fact *= j;
      MvArgs a = base;
      a.X = src;
      a.Y = (j % 2) ? t1 : t2;
      a.acc = (late && j == 1) ? nullptr : vout;
      a.acc_prev = prev;
      a.c_prev = c_prev;
      a.c_acc = 1.0 / (double)fact;
      matvec_cells<ONE, ST>(a);
      grid.sync();
      src = a.Y;
      prev = (late && j == 1) ? a.Y : nullptr;
      c_prev = a.c_acc;
    }
    if (!late) {
      for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        v[q] = vout[q];
      grid.sync();
    }
  }
}

// ---------------------------------------------------------------------------
// Float-float Taylor propagation (the cooperative propagator's default arithmetic). The
// Taylor terms and their running sum are float-float pairs (ff.cuh) and the blocks a
// float-float copy of the Jacobian (coef_ff, split once per linearisation), so that the
// 144 multiply-adds per cell and vector run on the FP32 pipe, which this GPU issues ~70x
// faster than FP64; only the input and output vectors are FP64. Each neighbour block adds
// its four products with ff_dot4 (the products' high parts exact by FMA, the sums by
// TwoSum, one renormalisation per block), in the order of the FP64 chains (input component
// 3 down to 0), so that the one-vector and the batched paths give the same pairs. A Taylor step of degree 4-5 at the CFL time step truncates at a far larger
// relative level than this rounding; the Jacobian is a finite-difference one (~1e-8).
struct MvFf {
  const float2* coef;
  const float2* X;
  float2* Y;
  float2* acc;             // the running sum, or null
  const float2* acc_prev;  // the previous term, added into acc first (acc += c_prev acc_prev)
  double scale;            // the time step (split on the device, as the per-vector ones)
  ff c_acc, c_prev;
  const double* vscale;    // per-vector time steps, or null
  Wrap w;
  long N, ld;
  int k, transpose;
};

__device__ __forceinline__ ff ldff(const float2* p, long i) {
  const float2 v = p[i];
  return ff{v.x, v.y};
}
__device__ __forceinline__ void stff(float2* p, long i, ff v) { p[i] = make_float2(v.h, v.l); }
// the block entries, read once per cell and chunk of vectors: when they exceed L2, streaming
// loads (evict-first), so that they do not push the vectors, which every neighbour re-reads,
// out of L2; when they fit, ordinary loads, which keep them cached across the matvecs
template <bool ST>
__device__ __forceinline__ ff ldff_coef(const float2* p, long i) {
  const float2 v = ST ? __ldcs(p + i) : p[i];
  return ff{v.x, v.y};
}

// one output of a term: val = scale y into Y, and the running sum
__device__ __forceinline__ void mvff_out(const MvFf& a, int vec, long o, ff y) {
  const ff sc = ff_from_double(a.vscale ? a.vscale[vec] : a.scale);
  const ff val = ff_mul(sc, y);
  stff(a.Y, o, val);
  if (a.acc) {
    ff r = ldff(a.acc, o);
    if (a.acc_prev) r = ff_add(r, ff_mul(ldff(a.acc_prev, o), a.c_prev));
    stff(a.acc, o, ff_add(r, ff_mul(val, a.c_acc)));
  }
}

// thread per (cell, output component, vector), as matvec_one
template <bool ST>
__device__ __forceinline__ void matvec_one_ff(const MvFf& a) {
  const long N = a.N;
  const long outs = 4 * N;
  // 32-bit decomposition of the work item (the host keeps the items below 2^31)
  const unsigned outs_u = (unsigned)outs, N_u = (unsigned)N, nchi_u = (unsigned)a.w.nchi;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < outs * a.k; t += (long)gridDim.x * blockDim.x) {
    const unsigned tu = (unsigned)t;
    const unsigned vec = tu / outs_u;
    const unsigned w = tu - vec * outs_u;
    const unsigned comp_u = w / N_u;
    const unsigned m = w - comp_u * N_u;
    const int comp = (int)comp_u;
    const unsigned j_u = m / nchi_u;
    const int i = (int)(m - j_u * nchi_u), j = (int)j_u;
    const float2* xv = a.X + (long)vec * a.ld;
    ff y{0.0f, 0.0f};
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const int b = q / 3 - 1, aa = q % 3 - 1;
      const long n = a.transpose ? a.w.nbr(i, j, -aa, -b) : a.w.nbr(i, j, aa, b);
      if (n < 0) continue;
      const long cell = a.transpose ? n : m;
      ff B[4], X[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int plane = a.transpose ? q * 16 + e * 4 + comp : q * 16 + comp * 4 + e;
        B[e] = ldff_coef<ST>(a.coef, (long)plane * N + cell);
        X[e] = ldff(xv, e * N + n);
      }
      y = ff_dot4(B, X, y);
    }
    mvff_out(a, (int)vec, (long)vec * a.ld + comp * N + m, y);
  }
}

// (cell, chunk of KV vectors) items, as matvec_multi (KV = kVecChunk; KV = 1 for a single
// vector on a large grid, where the smaller register set raises the occupancy of this
// HBM-bound case: the 144 block entries are read once per cell and vector)
template <int KV, bool ST>
__device__ __forceinline__ void matvec_multi_ff(const MvFf& a) {
  const long N = a.N;
  const long n4 = a.ld;
  const int chunks = (a.k + KV - 1) / KV;
  const long items = N * chunks;
  const unsigned N_u = (unsigned)N, nchi_u = (unsigned)a.w.nchi;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < items; w += (long)gridDim.x * blockDim.x) {
    const unsigned wu = (unsigned)w;
    const unsigned ch = wu / N_u;
    const unsigned m = wu - ch * N_u;
    const unsigned j_u = m / nchi_u;
    const int i = (int)(m - j_u * nchi_u), j = (int)j_u;
    const int v0 = (int)ch * KV;
    const int nv = min(KV, a.k - v0);
    ff y[KV][4];
#pragma unroll
    for (int v = 0; v < KV; ++v)
#pragma unroll
      for (int c = 0; c < 4; ++c) y[v][c] = ff{0.0f, 0.0f};
    // one neighbour block at a time for a single vector (its 16 pairs in registers), all
    // nine unrolled for a chunk
#pragma unroll(KV == 1 ? 1 : 3)
    for (int b = -1; b <= 1; ++b)
#pragma unroll(KV == 1 ? 1 : 3)
      for (int aa = -1; aa <= 1; ++aa) {
        const long n = a.transpose ? a.w.nbr(i, j, -aa, -b) : a.w.nbr(i, j, aa, b);
        if (n < 0) continue;
        const long cell = a.transpose ? n : m;
        const int q = (b + 1) * 3 + (aa + 1);
        ff B[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) B[e] = ldff_coef<ST>(a.coef, (long)(q * 16 + e) * N + cell);
        // unrolled over the chunk with a predicate, so that the pairs of y stay in registers
#pragma unroll
        for (int v = 0; v < KV; ++v) {
          if (v >= nv) continue;
          const float2* x = a.X + (long)(v0 + v) * n4;
          const ff xs[4] = {ldff(x, n), ldff(x, N + n), ldff(x, 2 * N + n), ldff(x, 3 * N + n)};
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            // row c of the block, or column c for the transpose
            const ff bs[4] = {B[a.transpose ? c : c * 4], B[a.transpose ? 4 + c : c * 4 + 1],
                              B[a.transpose ? 8 + c : c * 4 + 2], B[a.transpose ? 12 + c : c * 4 + 3]};
            y[v][c] = ff_dot4(bs, xs, y[v][c]);
          }
        }
      }
#pragma unroll
    for (int v = 0; v < KV; ++v)
      if (v < nv)
#pragma unroll
        for (int c = 0; c < 4; ++c) mvff_out(a, v0 + v, (long)(v0 + v) * n4 + c * N + m, y[v][c]);
  }
}

// (cell, output component, chunk of KV vectors) items: 4 block entries per neighbour in
// registers instead of 16, for the occupancy that keeps the FP32 pipe busy with a batch
// (the four threads of a cell read its inputs four times, from L1)
template <int KV, bool ST>
__device__ __forceinline__ void matvec_comp_ff(const MvFf& a) {
  const long N = a.N;
  const long n4 = a.ld;
  const int chunks = (a.k + KV - 1) / KV;
  const long items = 4 * N * chunks;
  const unsigned N_u = (unsigned)N, nchi_u = (unsigned)a.w.nchi;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < items; t += (long)gridDim.x * blockDim.x) {
    const unsigned tu = (unsigned)t;
    const unsigned r = tu / N_u;
    const unsigned m = tu - r * N_u;
    const int comp = (int)(r & 3u);
    const int v0 = (int)(r >> 2) * KV;
    const int nv = min(KV, a.k - v0);
    const unsigned j_u = m / nchi_u;
    const int i = (int)(m - j_u * nchi_u), j = (int)j_u;
    ff y[KV];
#pragma unroll
    for (int v = 0; v < KV; ++v) y[v] = ff{0.0f, 0.0f};
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const int b = q / 3 - 1, aa = q % 3 - 1;
      const long n = a.transpose ? a.w.nbr(i, j, -aa, -b) : a.w.nbr(i, j, aa, b);
      if (n < 0) continue;
      const long cell = a.transpose ? n : m;
      ff B[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int plane = a.transpose ? q * 16 + e * 4 + comp : q * 16 + comp * 4 + e;
        B[e] = ldff_coef<ST>(a.coef, (long)plane * N + cell);
      }
#pragma unroll
      for (int v = 0; v < KV; ++v) {
        if (v >= nv) continue;
        const float2* x = a.X + (long)(v0 + v) * n4;
        const ff xs[4] = {ldff(x, n), ldff(x, N + n), ldff(x, 2 * N + n), ldff(x, 3 * N + n)};
        y[v] = ff_dot4(B, xs, y[v]);
      }
    }
#pragma unroll
    for (int v = 0; v < KV; ++v)
      if (v < nv) mvff_out(a, v0 + v, (long)(v0 + v) * n4 + comp * N + m, y[v]);
  }
}

// The cooperative propagation in float-float (degree >= 2, the late-sum order of
// k_expm_coop): the input vectors are split into the running sum, and the sum is joined
// into the FP64 output after the last step. MODE 0: matvec_comp_ff<kVecChunk> (a batch on a
// large grid), 1: matvec_one_ff (few cells x vectors), 2: matvec_multi_ff<1> (one vector on
// a large grid), 3: matvec_multi_ff<kVecChunk> (a batch on a small grid). Measured on the
// 800 x 400 Jacobian: 68 us per vector-matvec for one vector (MODE 2; 111 in FP64) and for
// 8 (MODE 0; 83 with MODE 3, 91 in FP64); 64 vectors on the 100 x 80 one: 18.5 ms for 250
// matvecs with MODE 3, 24 with MODE 0, 40 in FP64.
template <int MODE, bool ST>
__global__ void __launch_bounds__(kMvThreads, MODE == 1 || MODE == 3 ? 2 : 3) k_expm_coop_ff(MvFf base, int nsteps, int order, const double* xin,
                                                                double* yout, float2* t1, float2* t2, float2* vout,
                                                                const int* vsteps) {
  cg::grid_group grid = cg::this_grid();
  const long nall = base.ld * (long)base.k;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nall; q += (long)gridDim.x * blockDim.x)
    stff(vout, q, ff_from_double_checked(xin[q]));
  grid.sync();
  const int kall = base.k;
  for (int s = 0; s < nsteps; ++s) {
    if (vsteps) {
      int ka = 0;
      while (ka < kall && vsteps[ka] > s) ++ka;
      base.k = ka;
    }
    const float2* src = vout;
    const float2* prev = nullptr;
    ff c_prev{0.0f, 0.0f};
    long fact = 1;
    for (int j = 1; j <= order; ++j) {
      fact *= j;
      MvFf a = base;
      a.X = src;
      a.Y = (j % 2) ? t1 : t2;
      a.acc = j == 1 ? nullptr : vout;
      a.acc_prev = prev;
      a.c_prev = c_prev;
      a.c_acc = ff_from_double(1.0 / (double)fact);
      if (MODE == 1) matvec_one_ff<ST>(a);
      else if (MODE == 2) matvec_multi_ff<1, ST>(a);
      else if (MODE == 3) matvec_multi_ff<kVecChunk, ST>(a);
      else matvec_comp_ff<kVecChunk, ST>(a);
      grid.sync();
      src = a.Y;
      prev = j == 1 ? a.Y : nullptr;
      c_prev = a.c_acc;
    }
  }
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nall; q += (long)gridDim.x * blockDim.x)
    yout[q] = ff_to_double(ldff(vout, q));
}

__global__ void k_coef_to_ff(const double* __restrict__ c, float2* __restrict__ f, long n) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
    stff(f, q, ff_from_double_checked(c[q]));
}

__global__ void k_copy(const double* __restrict__ s, double* __restrict__ d, long n) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) d[k] = s[k];
}

// per-cell block layout <-> plane layout
__global__ void k_blocks_to_planes(const double* blk, double* pl, long N) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < N * 144; t += (long)gridDim.x * blockDim.x) {
    const long m = t / 144;
    const int e = (int)(t % 144);
    pl[(long)e * N + m] = blk[t];
  }
}
__global__ void k_planes_to_blocks(const double* pl, double* blk, long N) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < N * 144; t += (long)gridDim.x * blockDim.x) {
    const long m = t / 144;
    const int e = (int)(t % 144);
    blk[t] = pl[(long)e * N + m];
  }
}


// ---------------------------------------------------------------------------
// Krylov helpers on device-resident bases. Reductions are deterministic: stage 1
// gives each (block, column) a fixed slice of rows and a fixed warp-shuffle tree,
// stage 2 sums the block partials of a column in a fixed order.
constexpr int kDotBlocks = 296;  // 2 x 148-152 SMs
constexpr int kDotThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// partial[j * kDotBlocks + b] = Σ_{rows of block b} A[i + j lda] * w[i]
__global__ void __launch_bounds__(kDotThreads) k_dot_stage1(const double* A, long lda, const double* w, long n,
                                                            double* partial) {
  const int j = blockIdx.y;
  const double* a = A + (long)j * lda;
  double acc = 0;
  for (long i = blockIdx.x * (long)kDotThreads + threadIdx.x; i < n; i += (long)kDotBlocks * kDotThreads)
    acc = fma(a[i], w[i], acc);
  acc = warp_sum(acc);
  __shared__ double red[kDotThreads / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kDotThreads / 32 ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[(long)j * kDotBlocks + blockIdx.x] = v;
  }
}

// out[j] (+)= Σ_b partial[j * kDotBlocks + b]; mode 0 store, 1 add
__global__ void k_dot_stage2(const double* partial, double* out, int mode) {
  const int j = blockIdx.x;
  double acc = 0;
  for (int b = threadIdx.x; b < kDotBlocks; b += 32) acc += partial[(long)j * kDotBlocks + b];
  acc = warp_sum(acc);
  if (threadIdx.x == 0) out[j] = mode ? out[j] + acc : acc;
}

// w -= A[:, 0:m] h
__global__ void __launch_bounds__(256) k_gemv_sub(const double* A, long lda, long n, int m, const double* h, double* w) {
  extern __shared__ double sh[];
  for (int j = threadIdx.x; j < m; j += blockDim.x) sh[j] = h[j];
  __syncthreads();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int j = 0; j < m; ++j) acc = fma(A[i + (long)j * lda], sh[j], acc);
    w[i] -= acc;
  }
}

// dst = src / sqrt(nrm2[0])
__global__ void k_normalize(const double* src, double* dst, long n, const double* nrm2) {
  const double s = 1.0 / sqrt(nrm2[0]);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) dst[i] = src[i] * s;
}

// out[:, c] = A[:, 0:m] Q[:, c] for c < k (Q column-major m x k, in global memory)
__global__ void __launch_bounds__(128) k_rotate(const double* A, long lda, long n, int m, int k, const double* Q,
                                                double* out, long ldo) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    for (int c0 = 0; c0 < k; c0 += 8) {
      double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      const int nc = min(8, k - c0);
      for (int j = 0; j < m; ++j) {
        const double a = A[i + (long)j * lda];
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (c < nc) acc[c] = fma(a, Q[j + (long)(c0 + c) * m], acc[c]);
      }
      for (int c = 0; c < nc; ++c) out[i + (long)(c0 + c) * ldo] = acc[c];
    }
  }
}

// y = blockdiag(B) x with B row-major 4x4 per cell (N x 16), vectors [v0; v1; v2; v3] x N, k columns
__global__ void k_block4(const double* B, const double* x, double* y, long N, int k) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < N * k; t += (long)gridDim.x * blockDim.x) {
    const long m = t % N;
    const long col = t / N;
    const double* xc = x + col * 4 * N;
    double* yc = y + col * 4 * N;
    const double x0 = xc[m], x1 = xc[N + m], x2 = xc[2 * N + m], x3 = xc[3 * N + m];
    const double* b = B + m * 16;
#pragma unroll
    for (int r = 0; r < 4; ++r) yc[r * N + m] = fma(b[4 * r], x0, fma(b[4 * r + 1], x1, fma(b[4 * r + 2], x2, b[4 * r + 3] * x3)));
  }
}

// Tail of vectors of 4N + nt entries: y = B x on the cells (k_block4), y = t x on the tail.
__global__ void k_block4_tail(const double* B, const double* tail, const double* x, double* y, long N, long nt,
                              int k) {
  const long ld = 4 * N + nt;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < N * k; t += (long)gridDim.x * blockDim.x) {
    const long m = t % N;
    const long col = t / N;
    const double* xc = x + col * ld;
    double* yc = y + col * ld;
    const double x0 = xc[m], x1 = xc[N + m], x2 = xc[2 * N + m], x3 = xc[3 * N + m];
    const double* b = B + m * 16;
#pragma unroll
    for (int r = 0; r < 4; ++r) yc[r * N + m] = fma(b[4 * r], x0, fma(b[4 * r + 1], x1, fma(b[4 * r + 2], x2, b[4 * r + 3] * x3)));
  }
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nt * k; t += (long)gridDim.x * blockDim.x) {
    const long m = t % nt, col = t / nt;
    y[col * ld + 4 * N + m] = tail[m] * x[col * ld + 4 * N + m];
  }
}

// ---------------------------------------------------------------------------
// Shock-position blocks (perturb_shock, LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-274).

// PERTURB_SHOCK (:906-913) direction of every point: ang = beta - pi/2 - phi with
// phi = atan(rho_v_0, rho_u_0), so (cos ang, sin ang) = (sin(beta - phi), -cos(beta - phi)),
// from the sine and cosine of beta that the last shock update of S stored.
__global__ void k_shock_dir(const double* beta, double* dir, int nchi, double cph, double sph) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nchi) return;
  const double sb = beta[i], cb = beta[nchi + i];
  dir[i] = sb * cph - cb * sph;
  dir[nchi + i] = -(cb * cph + sb * sph);
}

// Y's shock points = S's, point p displaced by eps along its PERTURB_SHOCK direction.
__global__ void k_perturb_point(ShockPts S, ShockPts Y, const double* dir, int nchi, int p, double eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nchi) return;
  double x = S.x[i], y = S.y[i];
  if (i == p) {
    x = x + eps * dir[i];
    y = y + eps * dir[nchi + i];
  }
  Y.x[i] = x;
  Y.y[i] = y;
  Y.chi[i] = S.chi[i];
  Y.eta[i] = S.eta[i];
}

// A21 column (j, var) of every point: (speed_i(x + eps e) - speed_i(x)) / eps
// (GET_OUTPUT_INDEXING_A21, :800-820; REMOVE_BASE_OUTPUT, :935-946)
__global__ void k_gather_a21(const double* rel, const double* rel_b, double* a21, int nchi, int col, double eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nchi) return;
  a21[i * 8 + col] = (rel[i] - rel_b[i]) / eps;
}

// A12 and A22 columns of point p (GET_OUTPUT_INDEXING_A12_A22, :854-903): the flux of the
// cells (i, sc_i - 1) and the shock speeds of every column.
struct Flux4 {
  const double* v[4];
};
__global__ void k_gather_a12(Flux4 Fp, Flux4 Fb, const double* rel, const double* rel_b, const int* rows,
                             double* a12, double* a22, int nchi, int p, double eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nchi) return;
  const long m = i + (long)(rows[i] - 2) * nchi;
#pragma unroll
  for (int v = 0; v < 4; ++v) a12[((long)v * nchi + i) * nchi + p] = (Fp.v[v][m] - Fb.v[v][m]) / eps;
  a22[(long)i * nchi + p] = (rel[i] - rel_b[i]) / eps;
}

// out (cols x rows) = in (rows x cols) transposed, both row-major
__global__ void k_transpose(const double* in, double* out, long rows, long cols) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < rows * cols; t += (long)gridDim.x * blockDim.x) {
    const long r = t / cols, c = t % cols;
    out[c * rows + r] = in[t];
  }
}

struct ShockMvArgs {
  ShockJac sj;
  const double* X;
  double* Y;
  long N, ld;
  double scale;
  int nchi, k, transpose;
};

// The shock-block part of y = scale A x (after the stencil matvec has written y's cell
// rows). Block (bx, col) stages what every row of vector col reads — r, and for the
// transpose the cells (i, sc_i - 1) of q — in shared memory, then gives each of its warps
// whole output rows: lanes over the row's entries (coalesced), a fixed shuffle tree.
//   forward:   rows (v, i) of A12 add scale (A12 r) into the flux rows (i, sc_i - 1);
//              speed rows i set y_r = scale (A21 q + A22 r).
//   transpose: speed rows p set y_r = scale (A12ᵀ q + A22ᵀ r); lanes 0-7 of the same warp
//              add scale A21ᵀ r into the cells (p, sc_p - j).
constexpr int kShockThreads = 128;
__host__ __device__ inline long shock_mv_smem(int nchi, int transpose) {
  return (long)(transpose ? 5 : 1) * nchi * (long)sizeof(double);
}

// Σ_p a[p] b[p] over the lane's entries p = lane, lane + 32, ... (one FMA chain: the FP64
// pipe, not the loads, bounds these rows; partial sums would add FP64 instructions)
__device__ __forceinline__ double lane_dot(const double* __restrict__ a, const double* b, int n, int lane) {
  double t = 0;
  for (int p = lane; p < n; p += 32) t = fma(a[p], b[p], t);
  return t;
}

__global__ void __launch_bounds__(kShockThreads) k_shock_mv(ShockMvArgs a) {
  extern __shared__ double sh[];
  const int lane = threadIdx.x & 31;
  const int nchi = a.nchi;
  const long N = a.N;
  const int* rows = a.sj.rows;
  const long col = blockIdx.y;
  const double* x = a.X + col * a.ld;
  double* y = a.Y + col * a.ld;
  const double* xr = x + 4 * N;
  double* sr = sh;  // r
  if (a.transpose) {
    sr = sh + 4 * nchi;
    for (int t = threadIdx.x; t < 4 * nchi; t += blockDim.x) {
      const int v = t / nchi, i = t % nchi;
      sh[t] = x[v * N + i + (long)(rows[i] - 2) * nchi];
    }
  }
  for (int t = threadIdx.x; t < nchi; t += blockDim.x) sr[t] = xr[t];
  __syncthreads();
  const int per = a.transpose ? nchi : 5 * nchi;
  const int wpb = blockDim.x / 32;
  for (int r = blockIdx.x * wpb + (threadIdx.x >> 5); r < per; r += gridDim.x * wpb) {
    double s = 0;
    if (!a.transpose) {
      if (r < 4 * nchi) {
        s = warp_sum(lane_dot(a.sj.a12 + (long)r * nchi, sr, nchi, lane));
        if (lane == 0) {
          const int v = r / nchi, i = r % nchi;
          y[v * N + i + (long)(rows[i] - 2) * nchi] += a.scale * s;
        }
      } else {
        const int i = r - 4 * nchi;
        s = lane_dot(a.sj.a22 + (long)i * nchi, sr, nchi, lane);
        if (lane < 8) {
          const int j = lane / 4 + 1, v = lane % 4;
          s = fma(a.sj.a21[i * 8 + lane], x[v * N + i + (long)(rows[i] - 1 - j) * nchi], s);
        }
        s = warp_sum(s);
        if (lane == 0) y[4 * N + i] = a.scale * s;
      }
    } else {
      const int p = r;
      s = lane_dot(a.sj.a12t + (long)p * 4 * nchi, sh, 4 * nchi, lane);
      s += lane_dot(a.sj.a22t + (long)p * nchi, sr, nchi, lane);
      s = warp_sum(s);
      if (lane == 0) y[4 * N + p] = a.scale * s;
      if (lane < 8) {
        const int j = lane / 4 + 1, v = lane % 4;
        y[v * N + p + (long)(rows[p] - 1 - j) * nchi] += a.scale * (a.sj.a21[p * 8 + lane] * sr[p]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Upstream-boundary operator B (freestream receptivity, Freestream_receptivity/LINEARIZE_B.jl).

// Per-column upstream state: the freestream, with variable `var` of the columns i = colour
// (mod 3) raised by eps (LINEARIZE_B.jl:49-70; var < 0: the unperturbed state).
__global__ void k_up_cols(double* cols, int nchi, double r0, double ru0, double rv0, double rE0, int var,
                          int colour, double eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nchi) return;
  const double f[4] = {r0, ru0, rv0, rE0};
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const double hit = (v == var && i % 3 == colour) ? 1.0 : 0.0;
    cols[v * nchi + i] = f[v] + eps * hit;
  }
}

// GET_BLOCK (LINEARIZE_B.jl:186-253): the raised column n = m + d (d in -1, 0, 1) of output
// column m is the one of this colour; its entries are the flux change of the cell
// (m, sc_m - 1) and the change of speed m over eps.
__global__ void k_gather_b(Flux4 Fp, Flux4 Fb, const double* rel, const double* rel_b, const int* rows, double* bq,
                           double* bs, int nchi, int var, int colour, double eps) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nchi) return;
  int d = 2;  // the offset in -1..1 whose column has this colour
  for (int dd = -1; dd <= 1; ++dd)
    if (((m + dd) % 3 + 3) % 3 == colour) d = dd;
  const int n = m + d;
  if (d == 2 || n < 0 || n >= nchi) return;
  const long cell = m + (long)(rows[m] - 2) * nchi;
#pragma unroll
  for (int vo = 0; vo < 4; ++vo)
    bq[((m * 3 + d + 1) * 4 + vo) * 4 + var] = (Fp.v[vo][cell] - Fb.v[vo][cell]) / eps;
  if (bs) bs[(m * 3 + d + 1) * 4 + var] = (rel[m] - rel_b[m]) / eps;
}

struct RecArgs {
  const double* X;
  double* Y;
  const double *bq, *bs, *w;
  const int* rows;
  long N, ld, nop;  // vector stride; nop = start of the freestream blocks
  double scale;
  int nchi, nw, k, adjoint, shock;
};

// The freestream part of the receptivity operator L_ = [L, B ... B; 0, diag(-i w_k I)]
// (LINEARIZE_L_.jl:60-68) on k complex vectors, each stored as its real and imaginary
// parts (real vectors 2c and 2c + 1 of stride ld), after the matvec with L has written the
// downstream rows. Forward: the flux rows (m, sc_m - 1) (and speed rows) add B (sum_k u_k);
// the freestream rows are -i w_k u_k. Adjoint (the conjugate transpose): every freestream
// block gets B^T q + i w_k u_k.
__global__ void __launch_bounds__(256) k_recept_mv(RecArgs a) {
  const int nchi = a.nchi;
  const long p4 = 4L * nchi;
  const long nre = 2L * a.k;
  const long items = a.adjoint ? nre * p4 : nre * nchi + nre * a.nw * p4;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < items; t += (long)gridDim.x * blockDim.x) {
    if (a.adjoint) {
      const long r = t / p4;
      const int e = (int)(t % p4), vin = e / nchi, n = e % nchi;
      const double* x = a.X + r * a.ld;
      const double* xo = a.X + (r ^ 1) * a.ld;
      double* y = a.Y + r * a.ld;
      double bt = 0;
      for (int m = max(n - 1, 0); m <= min(n + 1, nchi - 1); ++m) {
        const int slot = (m * 3 + (n - m) + 1) * 4;
        const long cell = m + (long)(a.rows[m] - 2) * nchi;
#pragma unroll
        for (int vo = 0; vo < 4; ++vo) bt = fma(a.bq[(slot + vo) * 4 + vin], x[vo * a.N + cell], bt);
        if (a.shock) bt = fma(a.bs[slot + vin], x[4 * a.N + m], bt);
      }
      const double sg = (r & 1) ? 1.0 : -1.0;  // i w u: real part -w u_im, imaginary part +w u_re
      for (int kk = 0; kk < a.nw; ++kk) {
        const long idx = a.nop + kk * p4 + e;
        y[idx] = a.scale * fma(sg * a.w[kk], xo[idx], bt);
      }
    } else if (t < nre * nchi) {
      const long r = t / nchi;
      const int m = (int)(t % nchi);
      const double* x = a.X + r * a.ld;
      double* y = a.Y + r * a.ld;
      double acc[4] = {0, 0, 0, 0}, accs = 0;
      for (int dd = -1; dd <= 1; ++dd) {
        const int n = m + dd;
        if (n < 0 || n >= nchi) continue;
        const int slot = (m * 3 + dd + 1) * 4;
#pragma unroll
        for (int vin = 0; vin < 4; ++vin) {
          double u = 0;
          for (int kk = 0; kk < a.nw; ++kk) u += x[a.nop + kk * p4 + vin * nchi + n];
#pragma unroll
          for (int vo = 0; vo < 4; ++vo) acc[vo] = fma(a.bq[(slot + vo) * 4 + vin], u, acc[vo]);
          accs = fma(a.bs[slot + vin], u, accs);
        }
      }
      const long cell = m + (long)(a.rows[m] - 2) * nchi;
#pragma unroll
      for (int vo = 0; vo < 4; ++vo) y[vo * a.N + cell] += a.scale * acc[vo];
      if (a.shock) y[4 * a.N + m] += a.scale * accs;
    } else {
      const long u = t - nre * nchi;
      const long r = u / (a.nw * p4);
      const long f = u % (a.nw * p4);
      const int kk = (int)(f / p4);
      const long idx = a.nop + f;
      const double sg = (r & 1) ? -1.0 : 1.0;  // -i w u: real part +w u_im, imaginary part -w u_re
      a.Y[r * a.ld + idx] = a.scale * (sg * a.w[kk] * a.X[(r ^ 1) * a.ld + idx]);
    }
  }
}

// t *= c, acc += t (n entries): one term of EXPONENTIAL!'s recurrence (CONSTRUCT_C.jl:78-111)
__global__ void k_scale_acc(double* t, double* acc, double c, long n) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const double v = t[q] * c;
    t[q] = v;
    acc[q] += v;
  }
}

// acc += c t (n entries)
__global__ void k_axpy(double* acc, const double* t, double c, long n) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
    acc[q] = fma(t[q], c, acc[q]);
}

int grid_for(long n, int threads) {
  long b = (n + threads - 1) / threads;
  const long cap = 152L * 16;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

void launch_shock_mv(const DevCtx& d, int k, const double* X, double* Y, int transpose, double scale,
                     cudaStream_t st, long ld) {
  ShockMvArgs a;
  a.sj = d.sj;
  a.X = X;
  a.Y = Y;
  a.N = d.N;
  a.ld = ld;
  a.scale = scale;
  a.nchi = d.nchi;
  a.k = k;
  a.transpose = transpose;
  // enough blocks per vector to spread the rows over the SMs, few enough that staging
  // the vector into each block stays small next to the blocks' reads of A12 and A22
  const long per = (transpose ? 1L : 5L) * d.nchi;
  const long wpb = kShockThreads / 32;
  const long cap = std::max(1L, 8L * d.sms / k);
  const int bx = (int)std::max(1L, std::min((per + wpb - 1) / wpb, cap));
  k_shock_mv<<<dim3(bx, k), kShockThreads, shock_mv_smem(d.nchi, transpose), st>>>(a);
}

// y = scale A x over k vectors of op_size(d) entries (stride ld, 0: op_size(d)): the stencil
// blocks, then the shock-position blocks when the operator has them.
int coef_stream(const DevCtx& d) { return 144L * d.N * 8 > kCoefStreamBytes ? 1 : 0; }

void launch_k_matvec(const DevCtx& d, int k, const MvArgs& a, int grid, int th, cudaStream_t st) {
  const bool one = mv_one(d.N, k, d.sms), stream = coef_stream(d);
  if (one && stream) k_matvec<true, true><<<grid, th, 0, st>>>(a);
  else if (one) k_matvec<true, false><<<grid, th, 0, st>>>(a);
  else if (stream) k_matvec<false, true><<<grid, th, 0, st>>>(a);
  else k_matvec<false, false><<<grid, th, 0, st>>>(a);
}

void launch_matvec(const DevCtx& d, int k, const double* X, double* Y, int transpose, double scale,
                   cudaStream_t st, long ld) {
  if (ld <= 0) ld = op_size(d);
  MvArgs a;
  a.acc_prev = nullptr;
  a.c_prev = 0;
  a.vscale = nullptr;
  a.coef = d.coef;
  a.X = X;
  a.Y = Y;
  a.acc = nullptr;
  a.scale = scale;
  a.c_acc = 0;
  a.w = make_wrap(d.cfg);
  a.N = d.N;
  a.ld = ld;
  a.k = k;
  a.transpose = transpose;
  const long items = mv_items(d.N, k, d.sms);
  const int th = mv_threads(items, d.sms);
  launch_k_matvec(d, k, a, grid_for(items, th), th, st);
  if (d.sj.on) launch_shock_mv(d, k, X, Y, transpose, scale, st, ld);
}

long recept_size(const DevCtx& d, int nw) { return op_size(d) + (long)nw * 4 * d.nchi; }

// y = scale L_ x (or scale L_^H x) for k complex vectors ([re; im] of recept_size each)
void launch_recept_apply(const DevCtx& d, int k, int nw, const double* dw, const double* X, double* Y, int adjoint,
                         double scale, cudaStream_t st) {
  const long ld = recept_size(d, nw);
  launch_matvec(d, 2 * k, X, Y, adjoint, scale, st, ld);
  RecArgs a;
  a.X = X;
  a.Y = Y;
  a.bq = d.bq;
  a.bs = d.bs;
  a.w = dw;
  a.rows = d.brows;
  a.N = d.N;
  a.ld = ld;
  a.nop = op_size(d);
  a.scale = scale;
  a.nchi = d.nchi;
  a.nw = nw;
  a.k = k;
  a.adjoint = adjoint;
  a.shock = d.sj.on;
  const long items = adjoint ? 8L * k * d.nchi : 2L * k * d.nchi + 8L * k * nw * d.nchi;
  k_recept_mv<<<grid_for(items, 256), 256, 0, st>>>(a);
}

// Runs `step` (the launches of one Taylor step, the same every step) nsteps times: captured
// once into a CUDA graph and replayed, so that the dozen small launches of a step cost one
// graph launch; launched directly when the stream is already being captured by the caller
// or the capture fails.
// graph_ok false: always launch directly (the allocation-free propagator builds no graph).
template <class Step>
static void repeat_steps(int nsteps, cudaStream_t st, Step step, bool graph_ok = true) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  if (graph_ok && nsteps > 1 && cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone &&
      cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    step();
    if (cudaStreamEndCapture(st, &g) == cudaSuccess && g && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) {
      for (int s = 0; s < nsteps; ++s) cudaGraphLaunch(ge, st);
      cudaGraphExecDestroy(ge);
      cudaGraphDestroy(g);
      return;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();  // a failed capture leaves nothing launched: run the steps directly
  }
  for (int s = 0; s < nsteps; ++s) step();
}

// EXPONENTIAL! (Transient_growth_downstream/CONSTRUCT_C.jl:78-111) with L_: per step term =
// vout, then term = (L_ dt) term / j and vout += term for j = 1..order. work: 2 x 2k x ld.
void launch_recept_expm(const DevCtx& d, int k, int nw, const double* dw, double dt, int nsteps, int order,
                        const double* X, double* Y, int adjoint, double* work, cudaStream_t st) {
  const long n = 2L * k * recept_size(d, nw);
  double* term = work;
  double* t2 = work + n;
  k_copy<<<grid_for(n, 256), 256, 0, st>>>(X, Y, n);
  repeat_steps(nsteps, st, [&]() {
    k_copy<<<grid_for(n, 256), 256, 0, st>>>(Y, term, n);
    double* src = term;
    double* dst = t2;
    for (int j = 1; j <= order; ++j) {
      launch_recept_apply(d, k, nw, dw, src, dst, adjoint, dt, st);
      k_scale_acc<<<grid_for(n, 256), 256, 0, st>>>(dst, Y, 1.0 / (double)j, n);
      std::swap(src, dst);
    }
  });
}

// POWER_METHOD! (Eigenvalues/ARNOLDI_POWER_GPU.jl:64-82): per step vout = v,
// term_j = (A dt) term_{j-1}, vout += term_j / j!, v = vout. The body assumes v and vout
// already hold the input.
static void launch_expm_body(const DevCtx& d, int k, double dt, int nsteps, int order, double* v, double* t1,
                             double* t2, double* vout, int transpose, cudaStream_t st, bool graph_ok) {
  const long n = op_size(d) * (long)k;
  if (d.sj.on) {
    // with the shock blocks every term is a full operator application, then vout += term / j!
    repeat_steps(nsteps, st, [&]() {
      const double* src = v;
      long fact = 1;
      for (int j = 1; j <= order; ++j) {
        fact *= j;
        double* dst = (j % 2) ? t1 : t2;
        launch_matvec(d, k, src, dst, transpose, dt, st);
        k_axpy<<<grid_for(n, 256), 256, 0, st>>>(vout, dst, 1.0 / (double)fact, n);
        src = dst;
      }
      k_copy<<<grid_for(n, 256), 256, 0, st>>>(vout, v, n);
    }, graph_ok);
    return;
  }
  const long items = mv_items(d.N, k, d.sms);
  const int th = mv_threads(items, d.sms);
  MvArgs a;
  a.acc_prev = nullptr;
  a.c_prev = 0;
  a.vscale = nullptr;
  a.coef = d.coef;
  a.w = make_wrap(d.cfg);
  a.N = d.N;
  a.ld = n / k;
  a.k = k;
  a.transpose = transpose;
  a.scale = dt;
  const bool late = order >= 2;  // as k_expm_coop: the first term is added one matvec late
  for (int s = 0; s < nsteps; ++s) {
    const double* src = late ? vout : v;
    const double* prev = nullptr;
    double c_prev = 0;
    long fact = 1;
    for (int j = 1; j <= order; ++j) {
      fact *= j;
      double* dst = (j % 2) ? t1 : t2;
      a.X = src;
      a.Y = dst;
      a.acc = (late && j == 1) ? nullptr : vout;
      a.acc_prev = prev;
      a.c_prev = c_prev;
      a.c_acc = 1.0 / (double)fact;
      launch_k_matvec(d, k, a, grid_for(items, th), th, st);
      src = dst;
      prev = (late && j == 1) ? dst : nullptr;
      c_prev = a.c_acc;
    }
    if (!late) k_copy<<<grid_for(n, 256), 256, 0, st>>>(vout, v, n);
  }
}

void launch_expm(const DevCtx& d, int k, double dt, int nsteps, int order, const double* X, double* Yout,
                 int transpose, double* work, cudaStream_t st, bool graph_ok) {
  const long n = op_size(d) * (long)k;
  double* v = work;
  double* t1 = work + n;
  double* t2 = work + 2 * n;
  k_copy<<<grid_for(n, 256), 256, 0, st>>>(X, v, n);
  k_copy<<<grid_for(n, 256), 256, 0, st>>>(X, Yout, n);
  launch_expm_body(d, k, dt, nsteps, order, v, t1, t2, Yout, transpose, st, graph_ok);
}

// Workspaces of the perturbed residuals of a linearisation (the A11 colours, the shock-point
// residuals, LINEARIZE_B's columns): each lane has its own stage array, p, T, edge sound
// speed, shock points, spline workspace, shock speeds, prescribed upstream columns and flux,
// and its own stream, so that the residuals of different perturbations run concurrently. The
// base state, the mesh, the base flux and the assembled blocks are shared: read-only, or
// written at entries no other perturbation writes, with the same arithmetic as one after
// another, so the result does not depend on the lanes.
constexpr int kJacLanes = 8;
static PertArgs pert_args(const DevCtx& d);
struct JacLane {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  double* mem = nullptr;
  Cons Y;
  double *p, *T, *aY, *spl, *speed_x, *speed_y, *rel, *cols;
  ShockPts Yp;
  double* F[4];
};
struct JacLanes {
  std::vector<JacLane> lane;
  cudaEvent_t fork = nullptr;
};

// The lane's view of the context: its own buffers in place of the shared ones. TMA
// descriptors name the context's own stage array, so a lane loads its halo thread by thread
// (the same values, the same arithmetic).
DevCtx lane_ctx(const DevCtx& d, const JacLane& l) {
  DevCtx ld = d;
  ld.Y = l.Y;
  ld.p = l.p;
  ld.T = l.T;
  ld.aY = l.aY;
  ld.spl = l.spl;
  ld.speed_x = l.speed_x;
  ld.speed_y = l.speed_y;
  ld.rel = l.rel;
  ld.Yp = l.Yp;
  ld.tma = 0;
  if (d.up_cols) ld.up_cols = l.cols;
  return ld;
}

// every lane waits for the work enqueued on st so far
void lanes_fork(JacLanes& L, cudaStream_t st) {
  cudaEventRecord(L.fork, st);
  for (JacLane& l : L.lane) cudaStreamWaitEvent(l.st, L.fork, 0);
}
// st waits for every lane
void lanes_join(JacLanes& L, cudaStream_t st) {
  for (JacLane& l : L.lane) {
    cudaEventRecord(l.done, l.st);
    cudaStreamWaitEvent(st, l.done, 0);
  }
}

// The shock-position blocks (perturb_shock), after the A11 assembly has left the base
// flux in Fb and the base shock speeds in sj.rel_b, on the shocked rows d.cell_idx:
//   A21 (LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-258): the shock speed of column i
//     reads only the cells (i, sc_i - 1) and (i, sc_i - 2) of its own column
//     (UPDATE_SHOCK_JUMP_PROPERTIES.jl:354-405), so raising the cell (i, sc_i - j) of every
//     column at once gives each column's speed the same inputs, and the same result, as the
//     reference's one perturbed cell per residual; the reference's other entries of such
//     a column are exact zeros. 8 residuals (j = 1, 2; 4 variables), no flux needed.
//   A12, A22 (:262-274): one residual per shock point, the point moved by eps along the
//     PERTURB_SHOCK direction (the smoothing spline couples every point to every other).
void launch_shock_assemble(DevCtx& d, const double* const Fb[4], PertArgs pa, JacLanes& L, cudaStream_t st) {
  const hymor_config& c = d.cfg;
  const int nchi = d.nchi;
  const int cb = (nchi + 127) / 128;
  const double eps = c.perturbation_magnitude;
  const double h = std::hypot(c.rho_u_0, c.rho_v_0);
  const int K = (int)L.lane.size();
  k_shock_dir<<<cb, 128, 0, st>>>(d.beta, d.sj.dir, nchi, c.rho_u_0 / h, c.rho_v_0 / h);
  cudaMemcpyAsync(d.sj.rows, d.cell_idx, sizeof(int) * nchi, cudaMemcpyDeviceToDevice, st);
  // only the flux of the cells (i, sc_i - 1) is read: the tiles whose halo the shock and
  // boundary kernels write (class 1 of the step's tile lists) hold them all, and compute
  // them with the same per-cell arithmetic as the whole grid
  launch_classify_tiles(d, st);
  lanes_fork(L, st);
  int q = 0;
  for (int j = 1; j <= 2; ++j)
    for (int var = 0; var < 4; ++var, ++q) {
      const JacLane& l = L.lane[q % K];
      const DevCtx ld = lane_ctx(d, l);
      PertArgs pl = pert_args(ld);
      pl.var = var;
      pl.shock_row = j;
      k_perturb_thermo<<<grid_for(d.G, 256), 256, 0, l.st>>>(pl);
      launch_shock_bc_flags(ld, false, true, true, false, 0, l.st);
      k_gather_a21<<<cb, 128, 0, l.st>>>(ld.rel, d.sj.rel_b, d.sj.a21, nchi, (j - 1) * 4 + var, eps);
    }
  Flux4 fb;
  for (int v = 0; v < 4; ++v) fb.v[v] = Fb[v];
  for (int p = 0; p < nchi; ++p, ++q) {
    const JacLane& l = L.lane[q % K];
    const DevCtx ld = lane_ctx(d, l);
    PertArgs pl = pert_args(ld);
    pl.var = -1;
    pl.shock_row = 0;
    Flux4 fp;
    for (int v = 0; v < 4; ++v) fp.v[v] = l.F[v];
    double* const Fp[4] = {l.F[0], l.F[1], l.F[2], l.F[3]};
    k_perturb_thermo<<<grid_for(d.G, 256), 256, 0, l.st>>>(pl);
    k_perturb_point<<<cb, 128, 0, l.st>>>(d.Sp, ld.Yp, d.sj.dir, nchi, p, eps);
    launch_shock_bc_flags(ld, false, false, true, true, 0, l.st);
    launch_flux_class(ld, false, Fp, 1, l.st);
    k_gather_a12<<<cb, 128, 0, l.st>>>(fp, fb, ld.rel, d.sj.rel_b, d.sj.rows, d.sj.a12, d.sj.a22, nchi, p, eps);
  }
  lanes_join(L, st);
  k_transpose<<<grid_for(4L * nchi * nchi, 256), 256, 0, st>>>(d.sj.a12, d.sj.a12t, 4L * nchi, nchi);
  k_transpose<<<grid_for((long)nchi * nchi, 256), 256, 0, st>>>(d.sj.a22, d.sj.a22t, nchi, nchi);
}

static PertArgs pert_args(const DevCtx& d) {
  const hymor_config& c = d.cfg;
  PertArgs pa;
  pa.S = d.S;
  pa.Y = d.Y;
  pa.p = d.p;
  pa.T = d.T;
  pa.cell_idx = d.cell_idx;
  pa.eps = c.perturbation_magnitude;
  pa.gm1 = c.gamma - 1;
  pa.nchi = d.nchi;
  pa.neta = d.neta;
  pa.shock = c.shock_enabled;
  pa.shock_row = 0;
  pa.aY = d.aY;
  pa.nrcbc = (c.bc_chi0 == HYMOR_BC_OUTFLOW_NRCBC) | ((c.bc_chi1 == HYMOR_BC_OUTFLOW_NRCBC) << 1) |
             ((c.bc_eta0 == HYMOR_BC_OUTFLOW_NRCBC) << 2) | ((c.bc_eta1 == HYMOR_BC_OUTFLOW_NRCBC) << 3);
  pa.var = -1;
  pa.colour = 1;
  return pa;
}

void launch_jacobian_assemble(DevCtx& d, cudaStream_t st, JacLanes& L) {
  ++d.coef_version;
  const hymor_config& c = d.cfg;
  const long N = d.N;
  double* Fb[4];
  for (int v = 0; v < 4; ++v) Fb[v] = d.jwork + v * N;
  const bool shock_blocks = c.shock_enabled && c.perturb_shock;
  PertArgs pa = pert_args(d);
  // base output: NON_LINEAR_DYNAMICS(deepcopy(s))
  k_perturb_thermo<<<grid_for(d.G, 256), 256, 0, st>>>(pa);
  launch_shock_bc_flags(d, false, true, c.shock_enabled, true, 0, st);
  launch_flux(d, false, Fb, st);
  if (shock_blocks)
    cudaMemcpyAsync(d.sj.rel_b, d.rel, sizeof(double) * d.nchi, cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(d.coef, 0, sizeof(double) * 144 * N, st);
  ScatArgs sa;
  for (int v = 0; v < 4; ++v) sa.Fb[v] = Fb[v];
  sa.coef = d.coef;
  sa.w = make_wrap(c);
  sa.eps = c.perturbation_magnitude;
  sa.N = N;
  // the 36 colour x variable residuals, spread over the lanes
  const int K = (int)L.lane.size();
  lanes_fork(L, st);
  int q = 0;
  for (int var = 0; var < 4; ++var)
    for (int colour = 1; colour <= 9; ++colour, ++q) {
      const JacLane& l = L.lane[q % K];
      const DevCtx ld = lane_ctx(d, l);
      PertArgs pl = pert_args(ld);
      pl.var = var;
      pl.colour = colour;
      double* const Fp[4] = {l.F[0], l.F[1], l.F[2], l.F[3]};
      k_perturb_thermo<<<grid_for(d.G, 256), 256, 0, l.st>>>(pl);
      launch_shock_bc_flags(ld, false, true, c.shock_enabled, true, 0, l.st);
      launch_flux(ld, false, Fp, l.st);
      ScatArgs sl = sa;
      for (int v = 0; v < 4; ++v) sl.Fp[v] = l.F[v];
      sl.var = var;
      sl.colour = colour;
      k_scatter<<<grid_for(N, 256), 256, 0, l.st>>>(sl);
    }
  lanes_join(L, st);
  if (shock_blocks) launch_shock_assemble(d, Fb, pa, L, st);
}

// LINEARIZE_B (Freestream_receptivity/LINEARIZE_B.jl:40-170): the residual with a prescribed
// per-column upstream state (rho_0_upstream_p), once unperturbed and once per variable and
// colour of columns (i = colour mod 3 raised by eps): 13 residuals. Each output column m has
// exactly one raised column among m - 1, m, m + 1 per colour.
void launch_b_assemble(DevCtx& d, cudaStream_t st, JacLanes& L) {
  const hymor_config& c = d.cfg;
  const long N = d.N;
  const int nchi = d.nchi, cb = (nchi + 127) / 128;
  const double eps = c.perturbation_magnitude;
  double* Fb[4];
  Flux4 fb;
  for (int v = 0; v < 4; ++v) {
    Fb[v] = d.jwork + v * N;
    fb.v[v] = Fb[v];
  }
  double* cols = d.bwork;
  double* rel_b = d.bwork + 4 * nchi;
  cudaMemcpyAsync(d.brows, d.cell_idx, sizeof(int) * nchi, cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(d.bq, 0, sizeof(double) * 48 * nchi, st);
  cudaMemsetAsync(d.bs, 0, sizeof(double) * 12 * nchi, st);
  d.up_cols = cols;
  // base: the uniform upstream state
  k_up_cols<<<cb, 128, 0, st>>>(cols, nchi, c.rho_0, c.rho_u_0, c.rho_v_0, c.rho_E_0, -1, 0, eps);
  k_perturb_thermo<<<grid_for(d.G, 256), 256, 0, st>>>(pert_args(d));
  launch_shock_bc_flags(d, false, true, true, true, 0, st);
  launch_flux(d, false, Fb, st);
  cudaMemcpyAsync(rel_b, d.rel, sizeof(double) * nchi, cudaMemcpyDeviceToDevice, st);
  // one residual per variable and colour of columns, spread over the lanes (each with its own
  // upstream columns)
  const int K = (int)L.lane.size();
  lanes_fork(L, st);
  int q = 0;
  for (int var = 0; var < 4; ++var)
    for (int colour = 0; colour < 3; ++colour, ++q) {
      const JacLane& l = L.lane[q % K];
      const DevCtx ld = lane_ctx(d, l);
      Flux4 fp;
      for (int v = 0; v < 4; ++v) fp.v[v] = l.F[v];
      double* const Fp[4] = {l.F[0], l.F[1], l.F[2], l.F[3]};
      k_up_cols<<<cb, 128, 0, l.st>>>(l.cols, nchi, c.rho_0, c.rho_u_0, c.rho_v_0, c.rho_E_0, var, colour, eps);
      k_perturb_thermo<<<grid_for(d.G, 256), 256, 0, l.st>>>(pert_args(ld));
      launch_shock_bc_flags(ld, false, true, true, true, 0, l.st);
      launch_flux(ld, false, Fp, l.st);
      k_gather_b<<<cb, 128, 0, l.st>>>(fp, fb, ld.rel, rel_b, d.brows, d.bq, d.bs, nchi, var, colour, eps);
    }
  lanes_join(L, st);
  d.up_cols = nullptr;
}

}  // namespace hymor

using namespace hymor;

namespace {
// Storage of the shock-position blocks (one allocation of doubles, one of the rows).
int ensure_shock(hymor_ctx* ctx) {
  DevCtx& d = ctx_dev(ctx);
  if (d.sj.a12) return 0;
  const long n = d.nchi;
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(double) * (8 * n + 10 * n * n + 3 * n)) != cudaSuccess)
    return ctx_fail(ctx, HYMOR_ERR_CUDA, "shock-block allocation failed");
  ctx_allocs(ctx).push_back(p);
  double* b = static_cast<double*>(p);
  ShockJac& j = d.sj;
  j.a21 = b;
  j.a12 = j.a21 + 8 * n;
  j.a22 = j.a12 + 4 * n * n;
  j.a12t = j.a22 + n * n;
  j.a22t = j.a12t + 4 * n * n;
  j.rel_b = j.a22t + n * n;
  j.dir = j.rel_b + n;
  if (cudaMalloc(&p, sizeof(int) * n) != cudaSuccess) return ctx_fail(ctx, HYMOR_ERR_CUDA, "shock-block allocation failed");
  ctx_allocs(ctx).push_back(p);
  j.rows = static_cast<int*>(p);
  // the transposed shock matvec stages 5 Nchi doubles per block
  const long smem = shock_mv_smem(d.nchi, 1);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_shock_mv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return ctx_fail(ctx, HYMOR_ERR_INVALID, "perturb_shock: Nchi too large for the shock matvec's shared memory");
  return 0;
}

// The A21 block reads the cells (i, sc_i - 2): a shocked row below 3 has no such cell (the
// reference's column index i + (sc_i - 3) Nchi would be out of range).
int check_shock_rows_for_blocks(hymor_ctx* ctx, const int* rows, int nchi, int neta) {
  for (int i = 0; i < nchi; ++i)
    if (rows[i] < 3 || rows[i] > neta - 1) {
      char msg[200];
      snprintf(msg, sizeof msg, "perturb_shock: shocked row %d of column %d outside 3..%d", rows[i], i + 1, neta - 1);
      return ctx_fail(ctx, HYMOR_ERR_SHOCK_RANGE, msg);
    }
  return 0;
}

// Storage of the upstream-boundary operator B.
int ensure_b(hymor_ctx* ctx) {
  DevCtx& d = ctx_dev(ctx);
  if (d.bq) return 0;
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(double) * 65 * (long)d.nchi) != cudaSuccess)
    return ctx_fail(ctx, HYMOR_ERR_CUDA, "upstream-boundary operator allocation failed");
  ctx_allocs(ctx).push_back(p);
  d.bq = static_cast<double*>(p);
  d.bs = d.bq + 48 * d.nchi;
  d.bwork = d.bs + 12 * d.nchi;
  if (cudaMalloc(&p, sizeof(int) * d.nchi) != cudaSuccess)
    return ctx_fail(ctx, HYMOR_ERR_CUDA, "upstream-boundary operator allocation failed");
  ctx_allocs(ctx).push_back(p);
  d.brows = static_cast<int*>(p);
  return 0;
}

// B's flux rows are the cells (m, sc_m - 1): sc_m must leave one flow cell below it.
int check_b_rows(hymor_ctx* ctx, const int* rows, int nchi, int neta) {
  for (int i = 0; i < nchi; ++i)
    if (rows[i] < 2 || rows[i] > neta - 1) {
      char msg[200];
      snprintf(msg, sizeof msg, "upstream-boundary operator: shocked row %d of column %d outside 2..%d", rows[i], i + 1,
               neta - 1);
      return ctx_fail(ctx, HYMOR_ERR_SHOCK_RANGE, msg);
    }
  return 0;
}

int ensure_linear(hymor_ctx* ctx) {
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(double) * 144 * d.N) != cudaSuccess)
      return ctx_fail(ctx, HYMOR_ERR_CUDA, "Jacobian allocation failed");
    ctx_allocs(ctx).push_back(p);
    d.coef = static_cast<double*>(p);
    if (cudaMalloc(&p, sizeof(double) * 8 * d.N) != cudaSuccess)
      return ctx_fail(ctx, HYMOR_ERR_CUDA, "Jacobian workspace allocation failed");
    ctx_allocs(ctx).push_back(p);
    d.jwork = static_cast<double*>(p);
  }
  return 0;
}

int cuda_check(hymor_ctx* ctx, cudaError_t e) {
  if (e != cudaSuccess) return ctx_fail(ctx, HYMOR_ERR_CUDA, cudaGetErrorString(e));
  return 0;
}

// Propagations of more than a few launches run as one cooperative kernel (k_expm_coop)
// over four context buffers (v, two Taylor terms, vout): a call copies its input into v
// and vout, launches once and copies vout out. This removes the per-launch overhead that
// dominates small grids (a 200 x 100 stencil matvec is ~5 us of FP64 work).
struct ExpmCache {
  double* buf = nullptr;
  long cap = 0;  // doubles
};
struct KrylovScratch {
  double* partial = nullptr;
  int cols = 0;
  double* h = nullptr;  // device coefficients (2 x cols + 2)
  double* tmp = nullptr;
  long tmp_n = 0;
};
// Per-context state of the linear entry points, owned by the context (created on first
// use, released by hymor_ctx_destroy).
struct LinearState {
  ExpmCache expm;
  KrylovScratch kry;
  int coop_blocks[12] = {};  // co-resident blocks per SM of k_expm_coop<false>, <true>,
                             // k_expm_coop_ff<0>, <1>, <2>, <3>, each with ordinary and
                             // streaming block loads
  JacLanes lanes;               // workspaces of the linearisations' perturbed residuals
};
LinearState& linear_state(hymor_ctx* ctx) {
  void*& slot = ctx_linear_state(ctx);
  if (!slot) slot = new LinearState();
  return *static_cast<LinearState*>(slot);
}
ExpmCache& expm_cache(hymor_ctx* ctx) { return linear_state(ctx).expm; }

// The linearisation lanes, made on first use (kJacLanes x ~(7 G + 4 N) doubles).
int ensure_lanes(hymor_ctx* ctx, JacLanes** out) {
  JacLanes& L = linear_state(ctx).lanes;
  *out = &L;
  if (!L.lane.empty()) return 0;
  const DevCtx& d = ctx_dev(ctx);
  const size_t G = d.G, N = d.N, n = d.nchi;
  auto pad = [](size_t k) { return (k + 31) & ~size_t(31); };  // 256-byte aligned parts
  const size_t total = 7 * pad(G) + 4 * pad(N) + 4 * pad(n) + pad(17 * n + 16) + 3 * pad(n) + pad(4 * n);
  if (cudaEventCreateWithFlags(&L.fork, cudaEventDisableTiming) != cudaSuccess)
    return ctx_fail(ctx, HYMOR_ERR_CUDA, "linearisation lane event");
  L.lane.resize(kJacLanes);
  for (JacLane& l : L.lane) {
    if (cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&l.mem, sizeof(double) * total) != cudaSuccess)
      return ctx_fail(ctx, HYMOR_ERR_CUDA, "linearisation lane allocation failed");
    cudaMemset(l.mem, 0, sizeof(double) * total);
    double* b = l.mem;
    auto take = [&](size_t k) {
      double* r = b;
      b += pad(k);
      return r;
    };
    l.Y = Cons{take(G), take(G), take(G), take(G)};
    l.p = take(G);
    l.T = take(G);
    l.aY = take(G);
    for (int v = 0; v < 4; ++v) l.F[v] = take(N);
    l.Yp = ShockPts{take(n), take(n), take(n), take(n)};
    l.spl = take(17 * n + 16);
    l.speed_x = take(n);
    l.speed_y = take(n);
    l.rel = take(n);
    l.cols = take(4 * n);
  }
  return 0;
}
constexpr int kExpmCoopMinLaunches = 16;
// grids from this many cells take the thread-per-component float-float batch
constexpr long kFfCompCells = 65536;


// hdts, hsteps (host, k entries, hsteps non-increasing), or null: vector c is propagated
// hsteps[c] steps of hdts[c] instead of nsteps of dt.
int expm_cooperative(hymor_ctx* ctx, int k, double dt, int nsteps, int order, const double* dX, double* dY,
                     int transpose, const double* hdts = nullptr, const int* hsteps = nullptr) {
  DevCtx& d = ctx_dev(ctx);
  cudaStream_t st = ctx_stream(ctx);
  ExpmCache& c = expm_cache(ctx);
  const long n = 4 * d.N * (long)k;
  int r;
  if (4 * n + 2 * k > c.cap) {
    if ((r = cuda_check(ctx, cudaStreamSynchronize(st)))) return r;
    if (c.buf) cudaFree(c.buf);
    c.buf = nullptr;
    c.cap = 0;
    void* p = nullptr;
    if ((r = cuda_check(ctx, cudaMalloc(&p, sizeof(double) * (4 * n + 2 * k))))) return r;
    c.buf = static_cast<double*>(p);
    c.cap = 4 * n + 2 * k;
  }
  double* v = c.buf;
  double* t1 = c.buf + n;
  double* t2 = c.buf + 2 * n;
  double* vout = c.buf + 3 * n;
  // float-float (degree >= 2; its kernels decompose their work items in 32 bits), with the
  // blocks' float-float copy split again after each write of the blocks
  const bool ffp = d.expm_ff && order >= 2 && 4L * d.N * k < (1L << 31);
  if (ffp && (!d.coef_ff || d.coef_ff_version != d.coef_version)) {
    if (!d.coef_ff) {
      void* p = nullptr;
      if ((r = cuda_check(ctx, cudaMalloc(&p, sizeof(float2) * 144 * d.N)))) return r;
      ctx_allocs(ctx).push_back(p);
      d.coef_ff = static_cast<float2*>(p);
    }
    k_coef_to_ff<<<grid_for(144 * d.N, 256), 256, 0, st>>>(d.coef, d.coef_ff, 144 * d.N);
    d.coef_ff_version = d.coef_version;
  }
  int* blocks_per_sm = linear_state(ctx).coop_blocks;
  const bool one = mv_one(d.N, k, d.sms);
  // float-float: thread per output on few cells x vectors, one cell per thread for one vector,
  // a thread per output component for a batch on a large grid, a chunk per thread on a small
  const int ffmode = one ? 1 : (k == 1 ? 2 : (d.N >= kFfCompCells ? 0 : 3));
  const int kind = ffp ? 2 + ffmode : (one ? 1 : 0);
  const int kst = 2 * kind + coef_stream(d);
  const void* kerns[12] = {(const void*)k_expm_coop<false, false>,  (const void*)k_expm_coop<false, true>,
                           (const void*)k_expm_coop<true, false>,   (const void*)k_expm_coop<true, true>,
                           (const void*)k_expm_coop_ff<0, false>,   (const void*)k_expm_coop_ff<0, true>,
                           (const void*)k_expm_coop_ff<1, false>,   (const void*)k_expm_coop_ff<1, true>,
                           (const void*)k_expm_coop_ff<2, false>,   (const void*)k_expm_coop_ff<2, true>,
                           (const void*)k_expm_coop_ff<3, false>,   (const void*)k_expm_coop_ff<3, true>};
  const void* kern = kerns[kst];
  if (!blocks_per_sm[kst] &&
      (r = cuda_check(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm[kst], kern, kMvThreads, 0))))
    return r;
  // the batched float-float path takes a thread per output component
  const long items = mv_items(d.N, k, d.sms) * (kind == 2 ? 4 : 1);
  const int th = mv_threads(items, d.sms);
  const long want = (items + th - 1) / th;
  // co-resident: blocks of th <= 256 threads need no more than a 256-thread block
  const int grid = (int)std::min<long>(want, (long)blocks_per_sm[kst] * d.sms);
  MvArgs base;
  base.acc_prev = nullptr;
  base.c_prev = 0;
  base.vscale = nullptr;
  base.coef = d.coef;
  base.w = make_wrap(d.cfg);
  base.N = d.N;
  base.ld = 4 * d.N;
  base.k = k;
  base.transpose = transpose;
  base.scale = dt;
  base.X = nullptr;
  base.Y = nullptr;
  base.acc = nullptr;
  base.c_acc = 0;
  int* vsteps = nullptr;
  if (hdts && hsteps) {
    double* vscale = c.buf + 4 * n;
    vsteps = reinterpret_cast<int*>(c.buf + 4 * n + k);
    if ((r = cuda_check(ctx, cudaMemcpyAsync(vscale, hdts, sizeof(double) * k, cudaMemcpyHostToDevice, st)))) return r;
    if ((r = cuda_check(ctx, cudaMemcpyAsync(vsteps, hsteps, sizeof(int) * k, cudaMemcpyHostToDevice, st)))) return r;
    base.vscale = vscale;
    nsteps = hsteps[0];
  }
  if (ffp) {
    MvFf bf;
    bf.coef = d.coef_ff;
    bf.X = nullptr;
    bf.Y = nullptr;
    bf.acc = nullptr;
    bf.acc_prev = nullptr;
    bf.scale = dt;
    bf.c_acc = ff{0.0f, 0.0f};
    bf.c_prev = ff{0.0f, 0.0f};
    bf.vscale = base.vscale;
    bf.w = base.w;
    bf.N = base.N;
    bf.ld = base.ld;
    bf.k = k;
    bf.transpose = transpose;
    float2* f1 = reinterpret_cast<float2*>(t1);
    float2* f2 = reinterpret_cast<float2*>(t2);
    float2* fo = reinterpret_cast<float2*>(vout);
    void* fargs[] = {&bf, &nsteps, &order, &dX, &dY, &f1, &f2, &fo, &vsteps};
    return cuda_check(ctx, cudaLaunchCooperativeKernel(kern, grid, th, fargs, 0, st));
  }
  if ((r = cuda_check(ctx, cudaMemcpyAsync(v, dX, sizeof(double) * n, cudaMemcpyDeviceToDevice, st)))) return r;
  if ((r = cuda_check(ctx, cudaMemcpyAsync(vout, dX, sizeof(double) * n, cudaMemcpyDeviceToDevice, st)))) return r;
  void* args[] = {&base, &nsteps, &order, &v, &t1, &t2, &vout, &vsteps};
  if ((r = cuda_check(ctx, cudaLaunchCooperativeKernel(kern, grid, th, args, 0, st))))
    return r;
  return cuda_check(ctx, cudaMemcpyAsync(dY, vout, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
}
}  // namespace

namespace hymor {
// Called by hymor_ctx_destroy after its stream has drained.
void linear_state_release(void* p) {
  if (!p) return;
  LinearState* s = static_cast<LinearState*>(p);
  if (s->expm.buf) cudaFree(s->expm.buf);
  for (JacLane& l : s->lanes.lane) {
    if (l.st) cudaStreamDestroy(l.st);
    if (l.done) cudaEventDestroy(l.done);
    if (l.mem) cudaFree(l.mem);
  }
  if (s->lanes.fork) cudaEventDestroy(s->lanes.fork);
  delete s;  // the Krylov buffers are context allocations, freed with the context
}
}  // namespace hymor

extern "C" {

int hymor_linearize(hymor_ctx* ctx) {
  if (!ctx) return HYMOR_ERR_INVALID;
  int r = ensure_linear(ctx);
  if (r) return r;
  DevCtx& d = ctx_dev(ctx);
  cudaStream_t st = ctx_stream(ctx);
  const bool shock_blocks = d.cfg.shock_enabled && d.cfg.perturb_shock;
  if (shock_blocks && (r = ensure_shock(ctx))) return r;
  d.sj.on = 0;
  // LINEARIZE_L.jl:43-56: flow cells and shock BC, thermo, sound speed, boundary conditions
  if (d.cfg.shock_enabled) {
    launch_flow_cells(d, st);
    launch_update_thermo(d, 3, 0, 0, st);
    launch_sound_cmax(d, true, st);
    launch_shock_bc_flags(d, true, false, true, false, 1, st);
  }
  launch_update_thermo(d, 3, 0, 0, st);
  launch_sound_cmax(d, true, st);
  launch_shock_bc_flags(d, true, false, false, true, 1, st);
  if (shock_blocks) {
    std::vector<int> rows(d.nchi);
    cudaMemcpyAsync(rows.data(), d.cell_idx, sizeof(int) * d.nchi, cudaMemcpyDeviceToHost, st);
    if ((r = cuda_check(ctx, cudaStreamSynchronize(st)))) return r;
    if ((r = check_shock_rows_for_blocks(ctx, rows.data(), d.nchi, d.neta))) return r;
  }
  JacLanes* L = nullptr;
  if ((r = ensure_lanes(ctx, &L))) return r;
  launch_jacobian_assemble(d, st, *L);
  if ((r = cuda_check(ctx, cudaGetLastError()))) return r;
  if ((r = cuda_check(ctx, cudaStreamSynchronize(st)))) return r;
  d.sj.on = shock_blocks;
  return 0;
}

int hymor_operator_size(hymor_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return HYMOR_ERR_INVALID;
  *n = op_size(ctx_dev(ctx));
  return 0;
}

int hymor_shock_blocks_get(hymor_ctx* ctx, int32_t* rows, double* a21, double* a12, double* a22) {
  if (!ctx || !rows || !a21 || !a12 || !a22) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.sj.on) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no shock blocks: linearise with perturb_shock");
  cudaStream_t st = ctx_stream(ctx);
  const long n = d.nchi;
  cudaMemcpyAsync(rows, d.sj.rows, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(a21, d.sj.a21, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(a12, d.sj.a12, sizeof(double) * 4 * n * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(a22, d.sj.a22, sizeof(double) * n * n, cudaMemcpyDeviceToHost, st);
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_shock_blocks_set(hymor_ctx* ctx, const int32_t* rows, const double* a21, const double* a12,
                           const double* a22) {
  if (!ctx) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!rows) {
    d.sj.on = 0;
    return 0;
  }
  if (!a21 || !a12 || !a22) return HYMOR_ERR_INVALID;
  if (!d.cfg.shock_enabled) return ctx_fail(ctx, HYMOR_ERR_INVALID, "shock blocks need shock fitting");
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  int r;
  if ((r = check_shock_rows_for_blocks(ctx, rows, d.nchi, d.neta))) return r;
  if ((r = ensure_shock(ctx))) return r;
  cudaStream_t st = ctx_stream(ctx);
  const long n = d.nchi;
  cudaMemcpyAsync(d.sj.rows, rows, sizeof(int) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.sj.a21, a21, sizeof(double) * 8 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.sj.a12, a12, sizeof(double) * 4 * n * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.sj.a22, a22, sizeof(double) * n * n, cudaMemcpyHostToDevice, st);
  k_transpose<<<grid_for(4 * n * n, 256), 256, 0, st>>>(d.sj.a12, d.sj.a12t, 4 * n, n);
  k_transpose<<<grid_for(n * n, 256), 256, 0, st>>>(d.sj.a22, d.sj.a22t, n, n);
  if ((r = cuda_check(ctx, cudaGetLastError()))) return r;
  if ((r = cuda_check(ctx, cudaStreamSynchronize(st)))) return r;
  d.sj.on = 1;
  return 0;
}

int hymor_shock_fields(hymor_ctx* ctx, double* beta, double* rel_vel) {
  if (!ctx) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  cudaStream_t st = ctx_stream(ctx);
  const long n = d.nchi;
  std::vector<double> sc(2 * n);
  cudaMemcpyAsync(sc.data(), d.beta, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st);
  if (rel_vel) cudaMemcpyAsync(rel_vel, d.rel, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  int r = cuda_check(ctx, cudaStreamSynchronize(st));
  if (r) return r;
  if (beta)
    for (long i = 0; i < n; ++i) beta[i] = std::atan2(sc[i], sc[n + i]);
  return 0;
}

int hymor_jacobian_get(hymor_ctx* ctx, double* coef) {
  if (!ctx || !coef) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  cudaStream_t st = ctx_stream(ctx);
  double* tmp = nullptr;
  int r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&tmp, sizeof(double) * 144 * d.N, st)))) return r;
  k_planes_to_blocks<<<grid_for(d.N * 144, 256), 256, 0, st>>>(d.coef, tmp, d.N);
  r = cuda_check(ctx, cudaMemcpyAsync(coef, tmp, sizeof(double) * 144 * d.N, cudaMemcpyDeviceToHost, st));
  cudaFreeAsync(tmp, st);
  if (r) return r;
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_jacobian_set(hymor_ctx* ctx, const double* coef) {
  if (!ctx || !coef) return HYMOR_ERR_INVALID;
  int r = ensure_linear(ctx);
  if (r) return r;
  DevCtx& d = ctx_dev(ctx);
  cudaStream_t st = ctx_stream(ctx);
  double* tmp = nullptr;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&tmp, sizeof(double) * 144 * d.N, st)))) return r;
  r = cuda_check(ctx, cudaMemcpyAsync(tmp, coef, sizeof(double) * 144 * d.N, cudaMemcpyHostToDevice, st));
  k_blocks_to_planes<<<grid_for(d.N * 144, 256), 256, 0, st>>>(tmp, d.coef, d.N);
  ++d.coef_version;
  cudaFreeAsync(tmp, st);
  if (r) return r;
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_matvec_dev(hymor_ctx* ctx, int k, const double* dX, double* dY, int transpose) {
  if (!ctx || k < 1 || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  launch_matvec(d, k, dX, dY, transpose, 1.0, ctx_stream(ctx));
  return cuda_check(ctx, cudaGetLastError());
}

int hymor_matvec(hymor_ctx* ctx, int k, const double* X, double* Y, int transpose) {
  if (!ctx || k < 1 || !X || !Y) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  cudaStream_t st = ctx_stream(ctx);
  const size_t bytes = sizeof(double) * op_size(d) * (size_t)k;
  double *dx = nullptr, *dy = nullptr;
  int r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&dx, bytes, st)))) return r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&dy, bytes, st)))) return r;
  cudaMemcpyAsync(dx, X, bytes, cudaMemcpyHostToDevice, st);
  launch_matvec(d, k, dx, dy, transpose, 1.0, st);
  cudaMemcpyAsync(Y, dy, bytes, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(dx, st);
  cudaFreeAsync(dy, st);
  if ((r = cuda_check(ctx, cudaGetLastError()))) return r;
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_bench_matvec(hymor_ctx* ctx, int k, const double* dX, double* dY, int transpose, int per_vector,
                       int reps, float* ms) {
  if (!ctx || k < 1 || !dX || !dY || reps < 1 || !ms) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  cudaStream_t st = ctx_stream(ctx);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r;
  if ((r = cuda_check(ctx, cudaEventCreate(&e0)))) return r;
  if ((r = cuda_check(ctx, cudaEventCreate(&e1)))) {
    cudaEventDestroy(e0);
    return r;
  }
  const long n4 = op_size(d);
  cudaEventRecord(e0, st);
  for (int rep = 0; rep < reps; ++rep) {
    if (per_vector) {
      for (int v = 0; v < k; ++v) launch_matvec(d, 1, dX + v * n4, dY + v * n4, transpose, 1.0, st);
    } else {
      launch_matvec(d, k, dX, dY, transpose, 1.0, st);
    }
  }
  cudaEventRecord(e1, st);
  r = cuda_check(ctx, cudaEventSynchronize(e1));
  if (!r) r = cuda_check(ctx, cudaEventElapsedTime(ms, e0, e1));
  if (!r) r = cuda_check(ctx, cudaGetLastError());
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return r;
}

int hymor_expm_apply_dev(hymor_ctx* ctx, int k, double dt, int nsteps, int order, const double* dX, double* dY,
                         int transpose) {
  if (!ctx || k < 1 || nsteps < 0 || order < 1 || order > 20 || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  cudaStream_t st = ctx_stream(ctx);
  // the cooperative kernel covers the stencil operator; with the shock blocks each term
  // is a launch sequence (launch_expm_body)
  if (!d.sj.on && (long)nsteps * (order + 1) >= kExpmCoopMinLaunches)
    return expm_cooperative(ctx, k, dt, nsteps, order, dX, dY, transpose);
  const size_t n = op_size(d) * (size_t)k;
  double* work = nullptr;
  int r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&work, 3 * n * sizeof(double), st)))) return r;
  launch_expm(d, k, dt, nsteps, order, dX, dY, transpose, work, st);
  cudaFreeAsync(work, st);
  return cuda_check(ctx, cudaGetLastError());
}

int hymor_expm_apply_multi_dev(hymor_ctx* ctx, int k, const double* dts, const int32_t* nsteps, int order,
                               const double* dX, double* dY, int transpose) {
  if (!ctx || k < 1 || !dts || !nsteps || order < 1 || order > 20 || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  for (int c = 0; c < k; ++c)
    if (nsteps[c] < 0 || (c > 0 && nsteps[c] > nsteps[c - 1]))
      return ctx_fail(ctx, HYMOR_ERR_INVALID, "per-vector step counts must be non-negative and non-increasing");
  if (d.sj.on) {
    // the shock-position operator has no cooperative propagator: one vector at a time
    const long n = op_size(d);
    for (int c = 0; c < k; ++c) {
      const int r = hymor_expm_apply_dev(ctx, 1, dts[c], nsteps[c], order, dX + c * n, dY + c * n, transpose);
      if (r) return r;
    }
    return 0;
  }
  return expm_cooperative(ctx, k, 0.0, nsteps[0], order, dX, dY, transpose, dts, nsteps);
}

int hymor_expm_apply(hymor_ctx* ctx, int k, double dt, int nsteps, int order, const double* X, double* Y,
                     int transpose) {
  if (!ctx || k < 1 || !X || !Y) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  cudaStream_t st = ctx_stream(ctx);
  const size_t bytes = sizeof(double) * op_size(d) * (size_t)k;
  double *dx = nullptr, *dy = nullptr;
  int r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&dx, bytes, st)))) return r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&dy, bytes, st)))) return r;
  cudaMemcpyAsync(dx, X, bytes, cudaMemcpyHostToDevice, st);
  r = hymor_expm_apply_dev(ctx, k, dt, nsteps, order, dx, dy, transpose);
  if (!r) cudaMemcpyAsync(Y, dy, bytes, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(dx, st);
  cudaFreeAsync(dy, st);
  if (r) return r;
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

}  // extern "C"

namespace {
KrylovScratch& kscratch(hymor_ctx* ctx) { return linear_state(ctx).kry; }
int ensure_scratch(hymor_ctx* ctx, int cols, long tmp_n) {
  KrylovScratch& k = kscratch(ctx);
  if (cols > k.cols) {
    void* p;
    if (cudaMalloc(&p, sizeof(double) * (long)kDotBlocks * cols) != cudaSuccess)
      return ctx_fail(ctx, HYMOR_ERR_CUDA, "Krylov scratch allocation failed");
    ctx_allocs(ctx).push_back(p);
    k.partial = static_cast<double*>(p);
    if (cudaMalloc(&p, sizeof(double) * (2 * cols + 4)) != cudaSuccess)
      return ctx_fail(ctx, HYMOR_ERR_CUDA, "Krylov scratch allocation failed");
    ctx_allocs(ctx).push_back(p);
    k.h = static_cast<double*>(p);
    k.cols = cols;
  }
  if (tmp_n > k.tmp_n) {
    void* p;
    if (cudaMalloc(&p, sizeof(double) * tmp_n) != cudaSuccess)
      return ctx_fail(ctx, HYMOR_ERR_CUDA, "Krylov scratch allocation failed");
    ctx_allocs(ctx).push_back(p);
    k.tmp = static_cast<double*>(p);
    k.tmp_n = tmp_n;
  }
  return 0;
}
void dots(const double* A, long lda, int m, const double* w, long n, double* out, int mode, double* partial,
          cudaStream_t st) {
  k_dot_stage1<<<dim3(kDotBlocks, m), kDotThreads, 0, st>>>(A, lda, w, n, partial);
  k_dot_stage2<<<m, 32, 0, st>>>(partial, out, mode);
}
}  // namespace

extern "C" {

int hymor_dot_dev(hymor_ctx* ctx, int64_t n, int m, const double* dA, int64_t lda, const double* dw, double* out) {
  if (!ctx || n < 1 || m < 1 || !dA || !dw || !out) return HYMOR_ERR_INVALID;
  int r = ensure_scratch(ctx, m + 1, 0);
  if (r) return r;
  KrylovScratch& k = kscratch(ctx);
  cudaStream_t st = ctx_stream(ctx);
  dots(dA, lda, m, dw, n, k.h, 0, k.partial, st);
  cudaMemcpyAsync(out, k.h, sizeof(double) * m, cudaMemcpyDeviceToHost, st);
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_krylov_orthogonalize(hymor_ctx* ctx, int64_t n, int m, double* dV, int64_t ldv, double* dw, double* h,
                               int out_col) {
  if (!ctx || n < 1 || m < 0 || !dV || !dw || !h) return HYMOR_ERR_INVALID;
  int r = ensure_scratch(ctx, 2 * (m + 1), 0);
  if (r) return r;
  KrylovScratch& k = kscratch(ctx);
  cudaStream_t st = ctx_stream(ctx);
  const int gb = grid_for(n, 256);
  double* h1 = k.h;           // m
  double* nrm = k.h + 2 * (m + 1) - 1;
  if (m > 0) {
    for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, twice
      double* hp = pass == 0 ? h1 : h1 + m;
      dots(dV, ldv, m, dw, n, hp, 0, k.partial, st);
      k_gemv_sub<<<gb, 256, sizeof(double) * m, st>>>(dV, ldv, n, m, hp, dw);
    }
  }
  dots(dw, n, 1, dw, n, nrm, 0, k.partial, st);
  if (out_col >= 0) k_normalize<<<gb, 256, 0, st>>>(dw, dV + (long)out_col * ldv, n, nrm);
  std::vector<double> hh(2 * m + 1);
  if (m > 0) cudaMemcpyAsync(hh.data(), h1, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hh.data() + 2 * m, nrm, sizeof(double), cudaMemcpyDeviceToHost, st);
  if ((r = cuda_check(ctx, cudaStreamSynchronize(st)))) return r;
  for (int j = 0; j < m; ++j) h[j] = hh[j] + hh[m + j];
  h[m] = std::sqrt(hh[2 * m]);
  return cuda_check(ctx, cudaGetLastError());
}

int hymor_krylov_rotate(hymor_ctx* ctx, int64_t n, int m, int kk, double* dV, int64_t ldv, const double* Q) {
  if (!ctx || n < 1 || m < 1 || kk < 1 || kk > m || !dV || !Q) return HYMOR_ERR_INVALID;
  int r = ensure_scratch(ctx, 1, n * kk + (long)m * kk);
  if (r) return r;
  KrylovScratch& k = kscratch(ctx);
  cudaStream_t st = ctx_stream(ctx);
  double* dQ = k.tmp + n * kk;
  cudaMemcpyAsync(dQ, Q, sizeof(double) * m * kk, cudaMemcpyHostToDevice, st);
  k_rotate<<<grid_for(n, 128), 128, 0, st>>>(dV, ldv, n, m, kk, dQ, k.tmp, n);
  for (int c = 0; c < kk; ++c)
    cudaMemcpyAsync(dV + (long)c * ldv, k.tmp + (long)c * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
  if ((r = cuda_check(ctx, cudaGetLastError()))) return r;
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_linearize_b(hymor_ctx* ctx) {
  if (!ctx) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.cfg.shock_enabled) return ctx_fail(ctx, HYMOR_ERR_INVALID, "the upstream-boundary operator needs shock fitting");
  int r = ensure_linear(ctx);
  if (r || (r = ensure_b(ctx))) return r;
  cudaStream_t st = ctx_stream(ctx);
  std::vector<int> rows(d.nchi);
  cudaMemcpyAsync(rows.data(), d.cell_idx, sizeof(int) * d.nchi, cudaMemcpyDeviceToHost, st);
  if ((r = cuda_check(ctx, cudaStreamSynchronize(st)))) return r;
  if ((r = check_b_rows(ctx, rows.data(), d.nchi, d.neta))) return r;
  JacLanes* L = nullptr;
  if ((r = ensure_lanes(ctx, &L))) return r;
  launch_b_assemble(d, st, *L);
  if ((r = cuda_check(ctx, cudaGetLastError()))) return r;
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_b_get(hymor_ctx* ctx, int32_t* rows, double* bq, double* bs) {
  if (!ctx || !rows || !bq) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.bq) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no upstream-boundary operator: call hymor_linearize_b");
  cudaStream_t st = ctx_stream(ctx);
  cudaMemcpyAsync(rows, d.brows, sizeof(int) * d.nchi, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(bq, d.bq, sizeof(double) * 48 * d.nchi, cudaMemcpyDeviceToHost, st);
  if (bs) cudaMemcpyAsync(bs, d.bs, sizeof(double) * 12 * d.nchi, cudaMemcpyDeviceToHost, st);
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_b_set(hymor_ctx* ctx, const int32_t* rows, const double* bq, const double* bs) {
  if (!ctx || !rows || !bq || !bs) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  int r;
  if ((r = check_b_rows(ctx, rows, d.nchi, d.neta)) || (r = ensure_b(ctx))) return r;
  cudaStream_t st = ctx_stream(ctx);
  cudaMemcpyAsync(d.brows, rows, sizeof(int) * d.nchi, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.bq, bq, sizeof(double) * 48 * d.nchi, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d.bs, bs, sizeof(double) * 12 * d.nchi, cudaMemcpyHostToDevice, st);
  return cuda_check(ctx, cudaStreamSynchronize(st));
}

int hymor_recept_size(hymor_ctx* ctx, int nw, int64_t* n) {
  if (!ctx || nw < 0 || !n) return HYMOR_ERR_INVALID;
  *n = recept_size(ctx_dev(ctx), nw);
  return 0;
}

// the frequencies on the device for one call (freed in stream order)
static int recept_prep(hymor_ctx* ctx, int k, int nw, const double* w, const double* dX, double* dY, double** dw) {
  if (!ctx || k < 1 || nw < 1 || !w || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  if (!d.bq) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no upstream-boundary operator: call hymor_linearize_b");
  cudaStream_t st = ctx_stream(ctx);
  int r;
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)dw, sizeof(double) * nw, st)))) return r;
  return cuda_check(ctx, cudaMemcpyAsync(*dw, w, sizeof(double) * nw, cudaMemcpyHostToDevice, st));
}

int hymor_recept_apply_dev(hymor_ctx* ctx, int k, int nw, const double* w, double scale, const double* dX, double* dY,
                           int adjoint) {
  double* dw = nullptr;
  int r = recept_prep(ctx, k, nw, w, dX, dY, &dw);
  if (r) return r;
  cudaStream_t st = ctx_stream(ctx);
  launch_recept_apply(ctx_dev(ctx), k, nw, dw, dX, dY, adjoint, scale, st);
  cudaFreeAsync(dw, st);
  return cuda_check(ctx, cudaGetLastError());
}

int hymor_recept_expm_dev(hymor_ctx* ctx, int k, int nw, const double* w, double dt, int nsteps, int order,
                          const double* dX, double* dY, int adjoint) {
  if (nsteps < 0 || order < 1 || order > 20) return HYMOR_ERR_INVALID;
  double* dw = nullptr;
  int r = recept_prep(ctx, k, nw, w, dX, dY, &dw);
  if (r) return r;
  DevCtx& d = ctx_dev(ctx);
  cudaStream_t st = ctx_stream(ctx);
  double* work = nullptr;
  const long n = 2L * k * recept_size(d, nw);
  if ((r = cuda_check(ctx, cudaMallocAsync((void**)&work, sizeof(double) * 2 * n, st)))) return r;
  launch_recept_expm(d, k, nw, dw, dt, nsteps, order, dX, dY, adjoint, work, st);
  cudaFreeAsync(work, st);
  cudaFreeAsync(dw, st);
  return cuda_check(ctx, cudaGetLastError());
}

int hymor_block4_apply_ext_dev(hymor_ctx* ctx, int k, int64_t ntail, const double* dB, const double* dTail,
                               const double* dX, double* dY) {
  if (!ctx || k < 1 || ntail < 0 || !dB || (ntail && !dTail) || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  k_block4_tail<<<grid_for(d.N * k, 256), 256, 0, ctx_stream(ctx)>>>(dB, dTail, dX, dY, d.N, ntail, k);
  return cuda_check(ctx, cudaGetLastError());
}

int hymor_block4_apply_dev(hymor_ctx* ctx, int k, const double* dB, const double* dX, double* dY) {
  if (!ctx || k < 1 || !dB || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  k_block4<<<grid_for(d.N * k, 256), 256, 0, ctx_stream(ctx)>>>(dB, dX, dY, d.N, k);
  return cuda_check(ctx, cudaGetLastError());
}

}  // extern "C"
