// Device-resident eigen and transient-growth solvers behind the C ABI: hymor_eigs and
// hymor_tg_gain.
//
// The reference wraps its GPU propagation in a LinearMap and hands it to host Arpack
// (Eigenvalues/EIGENVALUES.jl:152-162, TRANSIENT_GROWTH_DOWNSTREAM.jl:96-106), which moves
// every Krylov vector host -> device -> host. Here the Krylov basis stays in HBM: the
// operator (the Taylor propagator and the per-cell Chu-norm blocks), the classical
// Gram-Schmidt (twice, deterministic device reductions) and the restart rotation run on
// the device through the library's own entry points, and only the projected matrix (at
// most ncv + 2 block square) is handled on the host (dense.h). The restart is Stewart's
// Krylov-Schur (SIAM J. Matrix Anal. Appl. 23 (2001) 601-614); block > 1 grows the basis
// `block` vectors per batched propagation (Zhou and Saad, Numer. Algorithms 47 (2008)
// 341-359), so the projected matrix is block upper Hessenberg.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "dense.h"
#include "kernels.h"

namespace hymor {
DevCtx& ctx_dev(hymor_ctx* c);
cudaStream_t ctx_stream(hymor_ctx* c);
int ctx_fail(hymor_ctx* c, int code, const char* msg);
}  // namespace hymor

using namespace hymor;
using dense::cplx;
using dense::Mat;

namespace {

int cu(hymor_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  char msg[256];
  snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
  return ctx_fail(ctx, HYMOR_ERR_CUDA, msg);
}

// A device buffer freed (after the context stream drains) when it goes out of scope.
struct DevBuf {
  hymor_ctx* ctx = nullptr;
  double* p = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  int alloc(hymor_ctx* c, size_t doubles) {
    ctx = c;
    return cu(c, cudaMalloc((void**)&p, sizeof(double) * std::max<size_t>(doubles, 1)), "Krylov buffer allocation");
  }
  ~DevBuf() {
    if (p) {
      cudaStreamSynchronize(ctx_stream(ctx));
      cudaFree(p);
    }
  }
};

// Deterministic standard normal start vectors when the caller gives none (splitmix64 and
// the Box-Muller transform).
void normal_fill(uint64_t seed, double* x, size_t n) {
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
  auto next = [&]() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (size_t i = 0; i < n; i += 2) {
    const double u1 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double r = std::sqrt(-2.0 * std::log(u1)), a = 6.283185307179586 * u2;
    x[i] = r * std::cos(a);
    if (i + 1 < n) x[i + 1] = r * std::sin(a);
  }
}

// 1 on the entries of the flow cells (j < cell_idx[i]), and on the shock-position tail.
int flow_mask(hymor_ctx* ctx, long n, std::vector<double>& mask) {
  DevCtx& d = ctx_dev(ctx);
  mask.assign(n, 1.0);
  if (!(d.cfg.shock_enabled && d.cfg.shock_feedback)) return 0;
  std::vector<int> ci(d.nchi);
  int r = cu(ctx, cudaMemcpy(ci.data(), d.cell_idx, sizeof(int) * d.nchi, cudaMemcpyDeviceToHost), "cell indices");
  if (r) return r;
  for (int j = 0; j < d.neta; ++j)
    for (int i = 0; i < d.nchi; ++i) {
      const double f = (j + 1 < ci[i]) ? 1.0 : 0.0;
      for (int v = 0; v < 4; ++v) mask[(size_t)v * d.N + i + (size_t)j * d.nchi] = f;
    }
  return 0;
}

// One Krylov-Schur solve (block size b). The caller applies the operator: while
// need_op(), apply it to the b device vectors at src() and write dst(), then call
// consume(). Ritz values are kept in decreasing modulus.
class KrylovSchur {
 public:
  long n = 0;
  int nev = 0, ncv = 0, b = 1, maxit = 0;
  bool sym = false;
  double tol = 0;
  int nops = 0, restarts = 0;
  bool converged = false, failed = false;
  std::vector<cplx> theta;     // nev Ritz values
  std::vector<double> resid;   // their residual norms
  Mat Y;                       // projected Ritz vectors of the last cycle (m x nev), real part
  Mat Yi;                      //   and imaginary part (non-symmetric)
  int mlast = 0;               // basis size of the last cycle

  int init(hymor_ctx* c, long n_, int nev_, int ncv_, int b_, int maxit_, double tol_, bool sym_, const double* hx0) {
    ctx = c;
    n = n_;
    nev = nev_;
    ncv = ncv_;
    b = b_;
    maxit = maxit_;
    tol = tol_;
    sym = sym_;
    cap = ncv + 2 * b;
    int r;
    if ((r = V.alloc(ctx, (size_t)n * cap)) || (r = W.alloc(ctx, (size_t)n * b))) return r;
    H = Mat(cap, cap);
    st = ctx_stream(ctx);
    if ((r = cu(ctx, cudaMemcpyAsync(W.p, hx0, sizeof(double) * n * b, cudaMemcpyHostToDevice, st), "start block")))
      return r;
    std::vector<double> h(cap + 2);
    for (int i = 0; i < b; ++i) {  // orthonormal start block
      if ((r = hymor_krylov_orthogonalize(ctx, n, i, V.p, n, W.p + (size_t)i * n, h.data(), i))) return r;
      if (h[i] == 0) return ctx_fail(ctx, HYMOR_ERR_NUMERIC, "Krylov start block is rank deficient");
    }
    p = 0;
    begin_cycle();
    return 0;
  }

  bool need_op() const { return !done; }
  double* src() { return V.p + (size_t)j * n; }
  double* dst() { return W.p; }
  double* basis() { return V.p; }

  // Orthogonalises the b new vectors in dst() into the basis; at the end of a cycle,
  // checks convergence and restarts.
  int consume() {
    nops += b;
    std::vector<double> h(cap + 2);
    for (int i = 0; i < b; ++i) {
      const int J = j + b + i;  // orthonormal basis vectors so far
      int r = hymor_krylov_orthogonalize(ctx, n, J, V.p, n, W.p + (size_t)i * n, h.data(), J);
      if (r) return r;
      for (int q = 0; q < J; ++q) H(q, j + i) = h[q];
      H(J, j + i) = h[J];
      if (h[J] == 0) return ctx_fail(ctx, HYMOR_ERR_NUMERIC, "Krylov breakdown (invariant subspace found)");
    }
    j += b;
    if (j < m) return 0;
    return end_cycle();
  }

  // Ritz vectors V[:, :m] Y of the wanted values: real ones (symmetric) into dOut
  // (n x nev), else the real parts followed by the imaginary parts (n x 2 nev). Overwrites
  // the basis: call last.
  int ritz_vectors(double* dOut) {
    const int k = sym ? nev : 2 * nev;
    if (k > mlast) return ctx_fail(ctx, HYMOR_ERR_INVALID, "too many Ritz vectors for the basis");
    std::vector<double> Q((size_t)mlast * k);
    for (int c = 0; c < nev; ++c)
      for (int i = 0; i < mlast; ++i) {
        Q[(size_t)c * mlast + i] = Y(i, c);
        if (!sym) Q[(size_t)(nev + c) * mlast + i] = Yi(i, c);
      }
    int r = hymor_krylov_rotate(ctx, n, mlast, k, V.p, n, Q.data());
    if (r) return r;
    return cu(ctx, cudaMemcpyAsync(dOut, V.p, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st), "Ritz vectors");
  }

 private:
  hymor_ctx* ctx = nullptr;
  cudaStream_t st = nullptr;
  DevBuf V, W;
  Mat H;
  int cap = 0, p = 0, m = 0, j = 0;
  bool done = false;

  void begin_cycle() {
    m = p + b * std::max(1, (ncv - p + b - 1) / b);
    j = p;
  }

  int end_cycle() {
    Mat Hm(m, m), B(b, m);
    for (int c = 0; c < m; ++c) {
      for (int i = 0; i < m; ++i) Hm(i, c) = H(i, c);
      for (int i = 0; i < b; ++i) B(i, c) = H(m + i, c);
    }
    mlast = m;
    const int keep0 = std::min(nev + std::max(2, (m - nev) / 2), m - b);
    Mat Q;
    Mat T;
    int keep = 0;
    if (sym) {
      Mat S(m, m);
      for (int c = 0; c < m; ++c)
        for (int i = 0; i < m; ++i) S(i, c) = 0.5 * (Hm(i, c) + Hm(c, i));
      std::vector<double> w;
      Mat Vs;
      dense::symeig(S, w, Vs);
      std::vector<int> ord(m);
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return std::abs(w[a]) > std::abs(w[c]); });
      theta.assign(nev, 0.0);
      resid.assign(nev, 0.0);
      Y = Mat(m, nev);
      for (int c = 0; c < nev; ++c) {
        theta[c] = w[ord[c]];
        for (int i = 0; i < m; ++i) Y(i, c) = Vs(i, ord[c]);
        double rn = 0;
        for (int a = 0; a < b; ++a) {
          double s = 0;
          for (int i = 0; i < m; ++i) s += B(a, i) * Vs(i, ord[c]);
          rn = std::hypot(rn, s);
        }
        resid[c] = rn;
      }
      if (check_done()) return 0;
      keep = keep0;
      T = Mat(keep, keep);
      Q = Mat(m, keep);
      for (int c = 0; c < keep; ++c) {
        T(c, c) = w[ord[c]];
        for (int i = 0; i < m; ++i) Q(i, c) = Vs(i, ord[c]);
      }
    } else {
      Mat Tf = Hm, Z = Mat::eye(m);
      dense::hessenberg(Tf, Z);
      std::vector<int> bs;
      if (!dense::schur(Tf, Z, bs)) return ctx_fail(ctx, HYMOR_ERR_NUMERIC, "projected Schur form did not converge");
      std::vector<cplx> w;
      dense::block_eigs(Tf, bs, w);
      std::vector<int> ord(m);
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return std::abs(w[a]) > std::abs(w[c]); });
      theta.assign(nev, 0.0);
      resid.assign(nev, 0.0);
      Y = Mat(m, nev);
      Yi = Mat(m, nev);
      std::vector<cplx> x;
      for (int c = 0; c < nev; ++c) {
        const int e = ord[c];
        theta[c] = w[e];
        int start = e;
        bool upper = true;
        if (bs[e] == 0) {  // second row of a 2 x 2 block: the conjugate
          start = e - 1;
          upper = false;
        }
        dense::tri_eigvec(Tf, bs, start, upper, x);
        std::vector<cplx> y(m, 0.0);
        for (int i = 0; i < m; ++i) {
          cplx s = 0;
          for (int q = 0; q < m; ++q) s += Z(i, q) * x[q];
          y[i] = s;
        }
        double nrm = 0;
        for (const cplx& v : y) nrm = std::hypot(nrm, std::abs(v));
        double rn = 0;
        for (int a = 0; a < b; ++a) {
          cplx s = 0;
          for (int i = 0; i < m; ++i) s += B(a, i) * y[i];
          rn = std::hypot(rn, std::abs(s));
        }
        resid[c] = rn / nrm;
        for (int i = 0; i < m; ++i) {
          Y(i, c) = y[i].real() / nrm;
          Yi(i, c) = y[i].imag() / nrm;
        }
      }
      if (check_done()) return 0;
      // keep the Schur vectors of the keep0 largest Ritz values (whole conjugate pairs)
      const double thr = std::abs(w[ord[keep0 - 1]]) * (1 - 1e-12);
      std::vector<char> sel(m, 0);
      for (int k = 0; k < m; k += bs[k]) sel[k] = std::abs(w[k]) >= thr;
      const int lead = dense::reorder(Tf, Z, bs, sel);
      keep = std::max(1, std::min(lead, m - b));
      if (keep < m && bs[keep] == 0) keep -= 1;  // never split a 2 x 2 block
      T = Mat(keep, keep);
      Q = Mat(m, keep);
      for (int c = 0; c < keep; ++c) {
        for (int i = 0; i < keep; ++i) T(i, c) = Tf(i, c);
        for (int i = 0; i < m; ++i) Q(i, c) = Z(i, c);
      }
    }
    // V[:, :keep] = V[:, :m] Q; the residual block V[:, m:m+b] becomes columns keep..
    int r = hymor_krylov_rotate(ctx, n, m, keep, V.p, n, Q.a.data());
    if (r) return r;
    if ((r = cu(ctx, cudaMemcpyAsync(V.p + (size_t)keep * n, V.p + (size_t)m * n, sizeof(double) * n * b,
                                     cudaMemcpyDeviceToDevice, st), "residual block")))
      return r;
    Mat Hn(cap, cap);
    for (int c = 0; c < keep; ++c) {
      for (int i = 0; i < keep; ++i) Hn(i, c) = T(i, c);
      for (int a = 0; a < b; ++a) {
        double s = 0;
        for (int i = 0; i < m; ++i) s += B(a, i) * Q(i, c);
        Hn(keep + a, c) = s;
      }
    }
    H = Hn;
    p = keep;
    ++restarts;
    begin_cycle();
    return 0;
  }

  bool check_done() {
    converged = true;
    for (int c = 0; c < nev; ++c)
      if (!(resid[c] <= tol * std::abs(theta[c]))) converged = false;
    if (converged || restarts + 1 >= maxit) {
      done = true;
      return true;
    }
    return false;
  }
};

int check_opts(hymor_ctx* ctx, const hymor_krylov_opts* o, int* ncv) {
  if (!o || o->nev < 1 || o->block < 1 || o->maxit < 1 || o->order < 1 || o->order > 20 || !(o->tol > 0))
    return ctx_fail(ctx, HYMOR_ERR_INVALID, "invalid Krylov options (nev, block, maxit >= 1; order 1..20; tol > 0)");
  *ncv = o->ncv > 0 ? o->ncv : std::max({2 * o->nev + 1, 20, o->nev + 4 * o->block});
  if (*ncv < o->nev + 2 * o->block)
    return ctx_fail(ctx, HYMOR_ERR_INVALID, "need nev + 2 block <= ncv");
  return 0;
}

int start_vectors(hymor_ctx* ctx, const hymor_krylov_opts* o, long n, const double* x0, std::vector<double>& X) {
  X.assign((size_t)n * o->block, 0.0);
  if (x0) {
    std::memcpy(X.data(), x0, sizeof(double) * n * o->block);
  } else {
    normal_fill(o->seed, X.data(), X.size());
    if (o->flow_start) {
      std::vector<double> mask;
      int r = flow_mask(ctx, n, mask);
      if (r) return r;
      for (int c = 0; c < o->block; ++c)
        for (long i = 0; i < n; ++i) X[(size_t)c * n + i] *= mask[i];
    }
  }
  return 0;
}

// Chu-norm weights of transient growth for the context's solution (CONSTRUCT_R.jl:24-133,
// CONSTRUCT_M.jl:27-94, CONSTRUCT_M_HAT.jl:25-105): per cell, C0 = R'MR (M masked by the
// flow cells) and the inverse Cholesky factor of D = R'M^R (D = K K'), row-major 4 x 4;
// on the shock-position tail C0 = 0 and K = sqrt(bt_area[i, sc_i] / 2)
// (CONSTRUCT_M_HAT.jl:77-90). Device buffers: C0, K^-1, K^-T (16 N each), tails (0, 1/K).
struct ChuWeights {
  DevBuf blk, tail;
  long N = 0, ntail = 0;
  std::vector<double> kinvT, tail_k;  // host copies for the initial conditions

  int build(hymor_ctx* ctx) {
    DevCtx& d = ctx_dev(ctx);
    N = d.N;
    ntail = op_size(d) - 4 * d.N;
    const long G = d.G;
    std::vector<double> q(4 * G), vol(N);
    std::vector<int> ci(d.nchi);
    const double* planes[4] = {d.S.rho, d.S.ru, d.S.rv, d.S.rE};
    int r;
    for (int v = 0; v < 4; ++v)
      if ((r = cu(ctx, cudaMemcpy(q.data() + v * G, planes[v], sizeof(double) * G, cudaMemcpyDeviceToHost), "state")))
        return r;
    if ((r = cu(ctx, cudaMemcpy(vol.data(), d.m.vol, sizeof(double) * N, cudaMemcpyDeviceToHost), "volumes")) ||
        (r = cu(ctx, cudaMemcpy(ci.data(), d.cell_idx, sizeof(int) * d.nchi, cudaMemcpyDeviceToHost), "cell indices")))
      return r;
    const double g = d.cfg.gamma;
    std::vector<double> hb(48 * N);
    kinvT.assign(16 * N, 0.0);
    for (int jj = 0; jj < d.neta; ++jj)
      for (int ii = 0; ii < d.nchi; ++ii) {
        const long c = ii + (long)jj * d.nchi;
        const long gi = (ii + 1) + (long)(jj + 1) * (d.nchi + 2);
        const double rho = q[gi], ru = q[G + gi], rv = q[2 * G + gi], rE = q[3 * G + gi];
        const double u = ru / rho, w = rv / rho;
        const double p = (rE - (ru * ru + rv * rv) / rho / 2) * (g - 1);
        const double a2 = g * p / rho;
        double R[4][4] = {{(g - 1) * (u * u + w * w) / 2, -u * (g - 1), -w * (g - 1), g - 1},
                          {-u / rho, 1.0 / rho, 0, 0},
                          {-w / rho, 0, 1.0 / rho, 0},
                          {(u * u + w * w) / (2 * p) - g / (g - 1) / rho, -u / p, -w / p, 1.0 / p}};
        const double mh[4] = {rho * a2 / (2 * (g * p) * (g * p)) * vol[c], rho / 2 * vol[c], rho / 2 * vol[c],
                              (g - 1) * p / (2 * g) * vol[c]};
        const double flow = (!d.cfg.shock_enabled || jj + 1 < ci[ii]) ? 1.0 : 0.0;
        double C0[4][4], D[4][4];
        for (int i = 0; i < 4; ++i)
          for (int k = 0; k < 4; ++k) {
            double s0 = 0, s1 = 0;
            for (int l = 0; l < 4; ++l) {
              s0 += R[l][i] * (mh[l] * flow) * R[l][k];
              s1 += R[l][i] * mh[l] * R[l][k];
            }
            C0[i][k] = s0;
            D[i][k] = s1;
          }
        // Cholesky D = K K' (lower K), then K^-1 (lower)
        double K[4][4] = {{0}}, Ki[4][4] = {{0}};
        for (int i = 0; i < 4; ++i)
          for (int k = 0; k <= i; ++k) {
            double s = D[i][k];
            for (int l = 0; l < k; ++l) s -= K[i][l] * K[k][l];
            if (i == k) {
              if (!(s > 0)) return ctx_fail(ctx, HYMOR_ERR_NUMERIC, "Chu-norm weight block is not positive definite");
              K[i][i] = std::sqrt(s);
            } else {
              K[i][k] = s / K[k][k];
            }
          }
        for (int k = 0; k < 4; ++k) {
          Ki[k][k] = 1.0 / K[k][k];
          for (int i = k + 1; i < 4; ++i) {
            double s = 0;
            for (int l = k; l < i; ++l) s -= K[i][l] * Ki[l][k];
            Ki[i][k] = s / K[i][i];
          }
        }
        for (int i = 0; i < 4; ++i)
          for (int k = 0; k < 4; ++k) {
            hb[c * 16 + i * 4 + k] = C0[i][k];
            hb[16 * N + c * 16 + i * 4 + k] = Ki[i][k];
            hb[32 * N + c * 16 + i * 4 + k] = Ki[k][i];
            kinvT[c * 16 + i * 4 + k] = Ki[k][i];
          }
      }
    if ((r = blk.alloc(ctx, 48 * N)) ||
        (r = cu(ctx, cudaMemcpy(blk.p, hb.data(), sizeof(double) * 48 * N, cudaMemcpyHostToDevice), "weights")))
      return r;
    std::vector<double> ht(2 * std::max<long>(ntail, 1), 0.0);
    tail_k.assign(std::max<long>(ntail, 1), 1.0);
    if (ntail) {
      std::vector<double> bta((size_t)d.nchi * (d.neta + 1));
      if ((r = cu(ctx, cudaMemcpy(bta.data(), d.m.bt_a, sizeof(double) * bta.size(), cudaMemcpyDeviceToHost),
                  "face areas")))
        return r;
      for (int i = 0; i < d.nchi; ++i) {
        tail_k[i] = 1.0 / std::sqrt(bta[i + (size_t)(ci[i] - 1) * d.nchi] / 2);
        ht[std::max<long>(ntail, 1) + i] = tail_k[i];
      }
    }
    if ((r = tail.alloc(ctx, ht.size())) ||
        (r = cu(ctx, cudaMemcpy(tail.p, ht.data(), sizeof(double) * ht.size(), cudaMemcpyHostToDevice), "tails")))
      return r;
    return 0;
  }
  // which: 0 C0, 1 K^-1, 2 K^-T on k contiguous vectors
  int apply(hymor_ctx* ctx, int which, int k, const double* x, double* y) {
    const long nt = std::max<long>(ntail, 1);
    return hymor_block4_apply_ext_dev(ctx, k, ntail, blk.p + (size_t)which * 16 * N, tail.p + (which ? nt : 0), x, y);
  }
};

}  // namespace

extern "C" {

int hymor_eigs(hymor_ctx* ctx, const hymor_krylov_opts* o, double dt, int nsteps, const double* x0, double* mu_re,
               double* mu_im, double* resid, int32_t* info, double* dvecs) {
  if (!ctx || !mu_re || !mu_im || nsteps < 0) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  int ncv, r;
  if ((r = check_opts(ctx, o, &ncv))) return r;
  if (dvecs && 2 * o->nev > ncv) return ctx_fail(ctx, HYMOR_ERR_INVALID, "eigenvectors need 2 nev <= ncv");
  const long n = op_size(d);
  std::vector<double> X;
  if ((r = start_vectors(ctx, o, n, x0, X))) return r;
  KrylovSchur ks;
  if ((r = ks.init(ctx, n, o->nev, ncv, o->block, o->maxit, o->tol, false, X.data()))) return r;
  while (ks.need_op()) {
    if ((r = hymor_expm_apply_dev(ctx, o->block, dt, nsteps, o->order, ks.src(), ks.dst(), 0))) return r;
    if ((r = ks.consume())) return r;
  }
  for (int c = 0; c < o->nev; ++c) {
    mu_re[c] = ks.theta[c].real();
    mu_im[c] = ks.theta[c].imag();
    if (resid) resid[c] = ks.resid[c];
  }
  if (info) {
    info[0] = ks.nops;
    info[1] = ks.restarts;
    info[2] = ks.converged ? 1 : 0;
  }
  if (dvecs && (r = ks.ritz_vectors(dvecs))) return r;
  return cu(ctx, cudaStreamSynchronize(ctx_stream(ctx)), "eigen solve");
}

int hymor_tg_gain(hymor_ctx* ctx, const hymor_krylov_opts* o, int nh, const double* T, const double* x0,
                  double* gains, double* resid, int32_t* info, double* dt_out, int32_t* nsteps_out, double* dvecs) {
  if (!ctx || nh < 1 || !T || !gains) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  int ncv, r;
  if ((r = check_opts(ctx, o, &ncv))) return r;
  if (nh > 1 && (o->block != 1 || dvecs))
    return ctx_fail(ctx, HYMOR_ERR_INVALID, "several horizons run one vector each (block 1) and return no modes");
  for (int h = 0; h < nh; ++h)
    if (!(T[h] > 0)) return ctx_fail(ctx, HYMOR_ERR_INVALID, "horizons must be positive");
  double dt_cfl = 0;
  if ((r = hymor_cfl_timestep(ctx, &dt_cfl))) return r;
  const long n = op_size(d);
  const int b = o->block;
  // per horizon: steps = round(T / dt_CFL), dt = T / steps (TRANSIENT_GROWTH_DOWNSTREAM.jl:40-44)
  std::vector<int> steps(nh);
  std::vector<double> dts(nh);
  for (int h = 0; h < nh; ++h) {
    steps[h] = std::max(1, (int)std::lround(T[h] / dt_cfl));
    dts[h] = T[h] / steps[h];
    if (dt_out) dt_out[h] = dts[h];
    if (nsteps_out) nsteps_out[h] = steps[h];
  }
  ChuWeights cw;
  if ((r = cw.build(ctx))) return r;
  std::vector<double> X;
  if ((r = start_vectors(ctx, o, n, x0, X))) return r;
  std::vector<std::unique_ptr<KrylovSchur>> ks(nh);
  for (int h = 0; h < nh; ++h) {
    ks[h].reset(new KrylovSchur());
    if ((r = ks[h]->init(ctx, n, o->nev, ncv, b, o->maxit, o->tol, true, X.data()))) return r;
  }
  // horizons longest first: the vectors still advancing are a prefix of each batch
  std::vector<int> order(nh);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return steps[a] > steps[c]; });
  const int kmax = std::max(nh, b);
  DevBuf b0, b1, b2;
  if ((r = b0.alloc(ctx, (size_t)n * kmax)) || (r = b1.alloc(ctx, (size_t)n * kmax)) ||
      (r = b2.alloc(ctx, (size_t)n * kmax)))
    return r;
  cudaStream_t st = ctx_stream(ctx);
  std::vector<double> kdt;
  std::vector<int32_t> kst;
  for (;;) {
    std::vector<int> act;
    for (int h : order)
      if (ks[h]->need_op()) act.push_back(h);
    if (act.empty()) break;
    const int k = nh > 1 ? (int)act.size() : b;
    const double* src = ks[act[0]]->src();
    if (nh > 1) {
      for (int c = 0; c < k; ++c)
        if ((r = cu(ctx, cudaMemcpyAsync(b0.p + (size_t)c * n, ks[act[c]]->src(), sizeof(double) * n,
                                         cudaMemcpyDeviceToDevice, st), "gather")))
          return r;
      src = b0.p;
    }
    // y -> K^-1 P' C0 P K^-T y
    if ((r = cw.apply(ctx, 2, k, src, b1.p))) return r;
    if (nh > 1) {
      kdt.resize(k);
      kst.resize(k);
      for (int c = 0; c < k; ++c) {
        kdt[c] = dts[act[c]];
        kst[c] = steps[act[c]];
      }
      if ((r = hymor_expm_apply_multi_dev(ctx, k, kdt.data(), kst.data(), o->order, b1.p, b2.p, 0)) ||
          (r = cw.apply(ctx, 0, k, b2.p, b1.p)) ||
          (r = hymor_expm_apply_multi_dev(ctx, k, kdt.data(), kst.data(), o->order, b1.p, b2.p, 1)))
        return r;
    } else {
      if ((r = hymor_expm_apply_dev(ctx, k, dts[0], steps[0], o->order, b1.p, b2.p, 0)) ||
          (r = cw.apply(ctx, 0, k, b2.p, b1.p)) ||
          (r = hymor_expm_apply_dev(ctx, k, dts[0], steps[0], o->order, b1.p, b2.p, 1)))
        return r;
    }
    if (nh > 1) {
      if ((r = cw.apply(ctx, 1, k, b2.p, b0.p))) return r;
      for (int c = 0; c < k; ++c)
        if ((r = cu(ctx, cudaMemcpyAsync(ks[act[c]]->dst(), b0.p + (size_t)c * n, sizeof(double) * n,
                                         cudaMemcpyDeviceToDevice, st), "scatter")))
          return r;
    } else if ((r = cw.apply(ctx, 1, k, b2.p, ks[0]->dst()))) {
      return r;
    }
    for (int h : act)
      if ((r = ks[h]->consume())) return r;
  }
  for (int h = 0; h < nh; ++h) {
    for (int c = 0; c < o->nev; ++c) {
      gains[(size_t)h * o->nev + c] = ks[h]->theta[c].real();
      if (resid) resid[(size_t)h * o->nev + c] = ks[h]->resid[c];
    }
    if (info) {
      info[3 * h] = ks[h]->nops;
      info[3 * h + 1] = ks[h]->restarts;
      info[3 * h + 2] = ks[h]->converged ? 1 : 0;
    }
  }
  if (dvecs) {
    // optimal initial conditions x = K^-T y (x' R'M^R x = 1)
    DevBuf ry;
    if ((r = ry.alloc(ctx, (size_t)n * o->nev)) || (r = ks[0]->ritz_vectors(ry.p)) ||
        (r = cw.apply(ctx, 2, o->nev, ry.p, dvecs)))
      return r;
  }
  return cu(ctx, cudaStreamSynchronize(st), "transient-growth solve");
}

int hymor_dense_schur(int n, const double* A, int nsel, double* T, double* Z, double* wr, double* wi, int32_t* nlead) {
  if (n < 1 || n > 1024 || !A || !T || !Z || !wr || !wi || nsel < 0 || nsel > n) return HYMOR_ERR_INVALID;
  Mat M(n, n), Q = Mat::eye(n);
  std::memcpy(M.a.data(), A, sizeof(double) * n * n);
  dense::hessenberg(M, Q);
  std::vector<int> bs;
  if (!dense::schur(M, Q, bs)) return HYMOR_ERR_NUMERIC;
  std::vector<cplx> w;
  int lead = 0;
  if (nsel > 0) {
    dense::block_eigs(M, bs, w);
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return std::abs(w[a]) > std::abs(w[c]); });
    const double thr = std::abs(w[ord[nsel - 1]]) * (1 - 1e-12);
    std::vector<char> sel(n, 0);
    for (int k = 0; k < n; k += bs[k]) sel[k] = std::abs(w[k]) >= thr;
    lead = dense::reorder(M, Q, bs, sel);
  }
  dense::block_eigs(M, bs, w);
  std::memcpy(T, M.a.data(), sizeof(double) * n * n);
  std::memcpy(Z, Q.a.data(), sizeof(double) * n * n);
  for (int i = 0; i < n; ++i) {
    wr[i] = w[i].real();
    wi[i] = w[i].imag();
  }
  if (nlead) *nlead = lead;
  return 0;
}

int hymor_dense_symeig(int n, const double* A, double* w, double* V) {
  if (n < 1 || n > 1024 || !A || !w || !V) return HYMOR_ERR_INVALID;
  Mat M(n, n), Vm;
  std::memcpy(M.a.data(), A, sizeof(double) * n * n);
  std::vector<double> ww;
  dense::symeig(M, ww, Vm);
  std::memcpy(w, ww.data(), sizeof(double) * n);
  std::memcpy(V, Vm.a.data(), sizeof(double) * n * n);
  return 0;
}

}  // extern "C"
