// Small dense eigen-solvers for the projected matrices of the Krylov-Schur drivers
// (krylov.cu): n <= a few hundred, host code, column-major storage.
//
// The reference calls Arpack (Eigenvalues/EIGENVALUES.jl:159), whose dense steps are
// LAPACK's. These are written from the textbook algorithms:
//   * Householder reduction to upper Hessenberg form;
//   * the Francis implicit double-shift QR iteration to real Schur form (Golub and Van
//     Loan, Matrix Computations, 4th ed., Algorithms 7.5.1-7.5.2), 2 x 2 blocks with
//     real eigenvalues split by one rotation;
//   * reordering of the Schur form by swaps of adjacent 1 x 1 / 2 x 2 blocks through the
//     Sylvester equation A11 X - X A22 = A12 and a QR factorisation of [-X; I] (Bai and
//     Demmel, "On swapping diagonal blocks in real Schur form", Linear Algebra Appl. 186
//     (1993) 73-95);
//   * eigenvectors of the quasi-triangular factor by complex back-substitution;
//   * the cyclic Jacobi method for symmetric matrices.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

namespace hymor {
namespace dense {

using cplx = std::complex<double>;

struct Mat {
  int r = 0, c = 0;
  std::vector<double> a;
  Mat() = default;
  Mat(int rows, int cols) : r(rows), c(cols), a((size_t)rows * cols, 0.0) {}
  double& operator()(int i, int j) { return a[(size_t)i + (size_t)j * r]; }
  double operator()(int i, int j) const { return a[(size_t)i + (size_t)j * r]; }
  static Mat eye(int n) {
    Mat m(n, n);
    for (int i = 0; i < n; ++i) m(i, i) = 1.0;
    return m;
  }
};

// Householder vector of x[0..len): (I - tau v v^T) x = beta e1 with v[0] = 1.
inline double house(double* x, int len, double* v, double* beta) {
  double alpha = x[0], xn = 0;
  for (int i = 1; i < len; ++i) xn = std::hypot(xn, x[i]);
  v[0] = 1.0;
  if (xn == 0) {
    for (int i = 1; i < len; ++i) v[i] = 0;
    *beta = alpha;
    return 0.0;
  }
  double b = -std::copysign(std::hypot(alpha, xn), alpha);
  double s = 1.0 / (alpha - b);
  for (int i = 1; i < len; ++i) v[i] = x[i] * s;
  *beta = b;
  return (b - alpha) / b;
}

// A <- P^T A P with P = I - tau v v^T acting on indices k..k+len-1; rows of the left
// product restricted to columns c0..c1, columns of the right product to rows r0..r1.
inline void apply_left(Mat& A, int k, int len, const double* v, double tau, int c0, int c1) {
  if (tau == 0) return;
  for (int j = c0; j <= c1; ++j) {
    double d = 0;
    for (int i = 0; i < len; ++i) d += v[i] * A(k + i, j);
    d *= tau;
    for (int i = 0; i < len; ++i) A(k + i, j) -= d * v[i];
  }
}
inline void apply_right(Mat& A, int k, int len, const double* v, double tau, int r0, int r1) {
  if (tau == 0) return;
  for (int i = r0; i <= r1; ++i) {
    double d = 0;
    for (int j = 0; j < len; ++j) d += A(i, k + j) * v[j];
    d *= tau;
    for (int j = 0; j < len; ++j) A(i, k + j) -= d * v[j];
  }
}

// A = Q H Q^T: A is overwritten by the upper Hessenberg H, Q (n x n) accumulates.
inline void hessenberg(Mat& A, Mat& Q) {
  const int n = A.r;
  std::vector<double> x(n), v(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int len = n - k - 1;
    for (int i = 0; i < len; ++i) x[i] = A(k + 1 + i, k);
    double beta;
    const double tau = house(x.data(), len, v.data(), &beta);
    if (tau == 0) continue;
    apply_left(A, k + 1, len, v.data(), tau, k, n - 1);
    apply_right(A, k + 1, len, v.data(), tau, 0, n - 1);
    apply_right(Q, k + 1, len, v.data(), tau, 0, n - 1);
    A(k + 1, k) = beta;
    for (int i = 1; i < len; ++i) A(k + 1 + i, k) = 0;
  }
}

// Rotation of rows/columns k, k+1 by G = [c -s; s c]: T <- G^T T G, Z <- Z G.
inline void rotate2(Mat& T, Mat& Z, int k, double c, double s) {
  const int n = T.r;
  for (int j = 0; j < n; ++j) {
    const double a = T(k, j), b = T(k + 1, j);
    T(k, j) = c * a + s * b;
    T(k + 1, j) = -s * a + c * b;
  }
  for (int i = 0; i < n; ++i) {
    const double a = T(i, k), b = T(i, k + 1);
    T(i, k) = c * a + s * b;
    T(i, k + 1) = -s * a + c * b;
  }
  for (int i = 0; i < Z.r; ++i) {
    const double a = Z(i, k), b = Z(i, k + 1);
    Z(i, k) = c * a + s * b;
    Z(i, k + 1) = -s * a + c * b;
  }
}

// A 2 x 2 diagonal block at k with real eigenvalues is made upper triangular by one
// rotation whose first column is an eigenvector. Returns true if the block is complex.
inline bool split2(Mat& T, Mat& Z, int k) {
  const double a = T(k, k), b = T(k, k + 1), c = T(k + 1, k), d = T(k + 1, k + 1);
  if (c == 0) return false;
  const double p = 0.5 * (a - d);
  const double disc = p * p + b * c;
  if (disc < 0) return true;
  const double z = p + std::copysign(std::sqrt(disc), p);
  const double lam = d + z;
  double v1 = b, v2 = lam - a;
  const double w1 = lam - d, w2 = c;
  if (std::hypot(w1, w2) > std::hypot(v1, v2)) {
    v1 = w1;
    v2 = w2;
  }
  const double nv = std::hypot(v1, v2);
  if (nv == 0) return false;
  rotate2(T, Z, k, v1 / nv, v2 / nv);
  T(k + 1, k) = 0;
  return false;
}

// Francis double-shift QR: the upper Hessenberg H becomes quasi-upper-triangular T
// (real Schur form), Z <- Z Q. bsize[k] = 1 or 2 at the first index of each diagonal
// block (0 elsewhere). Returns false if the iteration did not converge.
inline bool schur(Mat& H, Mat& Z, std::vector<int>& bsize) {
  const int n = H.r;
  const double eps = std::numeric_limits<double>::epsilon();
  double hnorm = 0;
  for (double x : H.a) hnorm = std::max(hnorm, std::abs(x));
  bsize.assign(n, 0);
  int hi = n - 1, its = 0, total = 0;
  double v[3];
  while (hi >= 0) {
    int l = hi;
    for (; l > 0; --l) {
      double s = std::abs(H(l - 1, l - 1)) + std::abs(H(l, l));
      if (s == 0) s = hnorm;
      if (std::abs(H(l, l - 1)) <= eps * s) {
        H(l, l - 1) = 0;
        break;
      }
    }
    if (l == hi) {
      bsize[hi] = 1;
      --hi;
      its = 0;
      continue;
    }
    if (l == hi - 1) {
      if (split2(H, Z, hi - 1)) {
        bsize[hi - 1] = 2;
      } else {
        bsize[hi - 1] = 1;
        bsize[hi] = 1;
      }
      hi -= 2;
      its = 0;
      continue;
    }
    if (++total > 60 * n) return false;
    ++its;
    double s, t;
    if (its % 10 == 0) {  // exceptional shift after 10 stalled steps
      const double w = std::abs(H(hi, hi - 1)) + std::abs(H(hi - 1, hi - 2));
      s = 1.5 * w;
      t = w * w;
    } else {
      s = H(hi - 1, hi - 1) + H(hi, hi);
      t = H(hi - 1, hi - 1) * H(hi, hi) - H(hi - 1, hi) * H(hi, hi - 1);
    }
    double x = H(l, l) * H(l, l) + H(l, l + 1) * H(l + 1, l) - s * H(l, l) + t;
    double y = H(l + 1, l) * (H(l, l) + H(l + 1, l + 1) - s);
    double z = H(l + 1, l) * H(l + 2, l + 1);
    for (int k = l; k <= hi - 2; ++k) {
      double xv[3] = {x, y, z}, beta;
      const double tau = house(xv, 3, v, &beta);
      const int c0 = k > l ? k - 1 : l;
      apply_left(H, k, 3, v, tau, c0, n - 1);
      apply_right(H, k, 3, v, tau, 0, std::min(k + 3, hi));
      apply_right(Z, k, 3, v, tau, 0, Z.r - 1);
      if (k > l) {
        H(k + 1, k - 1) = 0;
        H(k + 2, k - 1) = 0;
      }
      x = H(k + 1, k);
      y = H(k + 2, k);
      z = k + 3 <= hi ? H(k + 3, k) : 0.0;
    }
    {
      double xv[2] = {x, y}, beta;
      const double tau = house(xv, 2, v, &beta);
      apply_left(H, hi - 1, 2, v, tau, hi - 2, n - 1);
      apply_right(H, hi - 1, 2, v, tau, 0, hi);
      apply_right(Z, hi - 1, 2, v, tau, 0, Z.r - 1);
      H(hi, hi - 2) = 0;
    }
  }
  return true;
}

// Eigenvalues of the diagonal blocks, in T's order (a complex pair as +im, -im).
inline void block_eigs(const Mat& T, const std::vector<int>& bsize, std::vector<cplx>& w) {
  const int n = T.r;
  w.assign(n, 0.0);
  for (int k = 0; k < n;) {
    if (bsize[k] == 2) {
      const double a = T(k, k), b = T(k, k + 1), c = T(k + 1, k), d = T(k + 1, k + 1);
      const double p = 0.5 * (a - d), disc = p * p + b * c;
      const double re = 0.5 * (a + d), im = std::sqrt(std::max(0.0, -disc));
      w[k] = cplx(re, im);
      w[k + 1] = cplx(re, -im);
      k += 2;
    } else {
      w[k] = T(k, k);
      k += 1;
    }
  }
}

// Solves the small dense system M x = r (dim <= 4) by Gaussian elimination with complete
// pivoting; false if M is numerically singular.
inline bool small_solve(int m, double* M, double* r, double* x) {
  int perm[4] = {0, 1, 2, 3};
  double scale = 0;
  for (int i = 0; i < m * m; ++i) scale = std::max(scale, std::abs(M[i]));
  if (scale == 0) return false;
  for (int k = 0; k < m; ++k) {
    int pi = k, pj = k;
    double best = 0;
    for (int i = k; i < m; ++i)
      for (int j = k; j < m; ++j)
        if (std::abs(M[i * m + j]) > best) {
          best = std::abs(M[i * m + j]);
          pi = i;
          pj = j;
        }
    if (best <= 1e-14 * scale) return false;
    if (pi != k) {
      for (int j = 0; j < m; ++j) std::swap(M[pi * m + j], M[k * m + j]);
      std::swap(r[pi], r[k]);
    }
    if (pj != k) {
      for (int i = 0; i < m; ++i) std::swap(M[i * m + pj], M[i * m + k]);
      std::swap(perm[pj], perm[k]);
    }
    for (int i = k + 1; i < m; ++i) {
      const double f = M[i * m + k] / M[k * m + k];
      for (int j = k; j < m; ++j) M[i * m + j] -= f * M[k * m + j];
      r[i] -= f * r[k];
    }
  }
  double y[4];
  for (int k = m - 1; k >= 0; --k) {
    double s = r[k];
    for (int j = k + 1; j < m; ++j) s -= M[k * m + j] * y[j];
    y[k] = s / M[k * m + k];
  }
  for (int k = 0; k < m; ++k) x[perm[k]] = y[k];
  return true;
}

// Swaps the adjacent diagonal blocks of sizes p (at k) and q (at k + p) of the real Schur
// form T, Z <- Z W. Returns false (nothing changed) when the blocks share an eigenvalue.
inline bool swap_blocks(Mat& T, Mat& Z, int k, int p, int q) {
  const int n = T.r, s = p + q;
  double K[16] = {0}, rhs[4], X[4];
  // A11 X - X A22 = A12, unknowns X(i, j) at i + j p
  for (int j = 0; j < q; ++j)
    for (int i = 0; i < p; ++i) {
      const int row = i + j * p;
      rhs[row] = T(k + i, k + p + j);
      for (int l = 0; l < p; ++l) K[row * (p * q) + (l + j * p)] += T(k + i, k + l);
      for (int l = 0; l < q; ++l) K[row * (p * q) + (i + l * p)] -= T(k + p + l, k + p + j);
    }
  if (!small_solve(p * q, K, rhs, X)) return false;
  // orthogonal W whose first q columns span [-X; I_q]: Householder QR of that s x q matrix
  Mat M(s, q), W = Mat::eye(s);
  for (int j = 0; j < q; ++j) {
    for (int i = 0; i < p; ++i) M(i, j) = -X[i + j * p];
    M(p + j, j) = 1.0;
  }
  double x[4], v[4], beta;
  for (int j = 0; j < q; ++j) {
    const int len = s - j;
    for (int i = 0; i < len; ++i) x[i] = M(j + i, j);
    const double tau = house(x, len, v, &beta);
    apply_left(M, j, len, v, tau, j, q - 1);
    apply_right(W, j, len, v, tau, 0, s - 1);
  }
  // T <- W^T T W on rows/columns k..k+s-1, Z <- Z W
  std::vector<double> tmp((size_t)std::max(n, Z.r) * s);
  for (int jj = k; jj < n; ++jj) {  // rows k..k+s-1 (entries left of k are zero)
    for (int a = 0; a < s; ++a) {
      double d = 0;
      for (int b = 0; b < s; ++b) d += W(b, a) * T(k + b, jj);
      tmp[a] = d;
    }
    for (int a = 0; a < s; ++a) T(k + a, jj) = tmp[a];
  }
  for (int i = 0; i < k + s; ++i) {
    for (int a = 0; a < s; ++a) {
      double d = 0;
      for (int b = 0; b < s; ++b) d += T(i, k + b) * W(b, a);
      tmp[a] = d;
    }
    for (int a = 0; a < s; ++a) T(i, k + a) = tmp[a];
  }
  for (int i = 0; i < Z.r; ++i) {
    for (int a = 0; a < s; ++a) {
      double d = 0;
      for (int b = 0; b < s; ++b) d += Z(i, k + b) * W(b, a);
      tmp[a] = d;
    }
    for (int a = 0; a < s; ++a) Z(i, k + a) = tmp[a];
  }
  for (int j = 0; j < q; ++j)
    for (int i = q; i < s; ++i) T(k + i, k + j) = 0;
  return true;
}

// Moves the selected blocks (sel per block start) to the top of the Schur form, keeping
// their relative order. bsize is updated; returns the number of leading rows that hold
// selected blocks (fewer than asked if a swap failed).
inline int reorder(Mat& T, Mat& Z, std::vector<int>& bsize, const std::vector<char>& sel_at) {
  const int n = T.r;
  std::vector<int> sz;
  std::vector<char> sel;
  for (int k = 0; k < n; k += bsize[k]) {
    sz.push_back(bsize[k]);
    sel.push_back(sel_at[k]);
  }
  const int nb = (int)sz.size();
  int lead = 0;
  bool ok = true;
  for (int b = 0; b < nb && ok; ++b) {
    if (!sel[b]) continue;
    int j = b;
    while (j > 0 && !sel[j - 1]) {
      int start = 0;
      for (int t = 0; t < j - 1; ++t) start += sz[t];
      if (!swap_blocks(T, Z, start, sz[j - 1], sz[j])) {
        ok = false;
        break;
      }
      std::swap(sz[j - 1], sz[j]);
      std::swap(sel[j - 1], sel[j]);
      --j;
    }
  }
  bsize.assign(n, 0);
  for (int b = 0, k = 0; b < nb; k += sz[b], ++b) {
    bsize[k] = sz[b];
    if (sel[b] && lead == k) lead += sz[b];
  }
  return lead;
}

// Unit eigenvector (complex, length n) of the quasi-triangular T for the eigenvalue of
// the block at k (for a 2 x 2 block, the eigenvalue with positive imaginary part when
// upper is true, else its conjugate), by back-substitution.
inline void tri_eigvec(const Mat& T, const std::vector<int>& bsize, int k, bool upper, std::vector<cplx>& x) {
  const int n = T.r;
  x.assign(n, 0.0);
  double tn = 0;
  for (double a : T.a) tn = std::max(tn, std::abs(a));
  const double small = std::max(tn, 1e-300) * std::numeric_limits<double>::epsilon();
  cplx lam;
  if (bsize[k] == 2) {
    const double a = T(k, k), b = T(k, k + 1), c = T(k + 1, k), d = T(k + 1, k + 1);
    const double p = 0.5 * (a - d), disc = p * p + b * c;
    lam = cplx(0.5 * (a + d), (upper ? 1.0 : -1.0) * std::sqrt(std::max(0.0, -disc)));
    cplx v1 = b, v2 = lam - a;
    const cplx w1 = lam - d, w2 = c;
    if (std::abs(w1) + std::abs(w2) > std::abs(v1) + std::abs(v2)) {
      v1 = w1;
      v2 = w2;
    }
    x[k] = v1;
    x[k + 1] = v2;
  } else {
    lam = T(k, k);
    x[k] = 1.0;
  }
  // blocks above k, bottom to top
  std::vector<int> starts;
  for (int s = 0; s < k; s += bsize[s]) starts.push_back(s);
  const int top = k + bsize[k];
  for (int bi = (int)starts.size() - 1; bi >= 0; --bi) {
    const int s = starts[bi];
    if (bsize[s] == 1) {
      cplx r = 0;
      for (int j = s + 1; j < top; ++j) r -= T(s, j) * x[j];
      cplx dg = T(s, s) - lam;
      if (std::abs(dg) < small) dg = small;
      x[s] = r / dg;
    } else {
      cplx r0 = 0, r1 = 0;
      for (int j = s + 2; j < top; ++j) {
        r0 -= T(s, j) * x[j];
        r1 -= T(s + 1, j) * x[j];
      }
      const cplx a = T(s, s) - lam, b = T(s, s + 1), c = T(s + 1, s), d = T(s + 1, s + 1) - lam;
      cplx det = a * d - b * c;
      if (std::abs(det) < small * small) det = small * small;
      x[s] = (r0 * d - b * r1) / det;
      x[s + 1] = (a * r1 - c * r0) / det;
    }
    // rescale against overflow
    double mx = 0;
    for (int j = s; j < top; ++j) mx = std::max(mx, std::abs(x[j]));
    if (mx > 1e100)
      for (int j = s; j < top; ++j) x[j] /= mx;
  }
  double nrm = 0;
  for (const cplx& v : x) nrm = std::hypot(nrm, std::abs(v));
  if (nrm > 0)
    for (cplx& v : x) v /= nrm;
}

// Symmetric eigen-decomposition by the cyclic Jacobi method: A = V diag(w) V^T.
inline void symeig(Mat A, std::vector<double>& w, Mat& V) {
  const int n = A.r;
  V = Mat::eye(n);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        tot += A(i, j) * A(i, j);
        if (i != j) off += A(i, j) * A(i, j);
      }
    if (off <= 1e-32 * tot || off == 0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (apq == 0) continue;
        const double theta = (A(q, q) - A(p, p)) / (2 * apq);
        const double t = std::copysign(1.0, theta) / (std::abs(theta) + std::sqrt(theta * theta + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        A(p, q) = A(q, p) = 0;
        for (int k = 0; k < n; ++k) {
          const double vkp = V(k, p), vkq = V(k, q);
          V(k, p) = c * vkp - s * vkq;
          V(k, q) = s * vkp + c * vkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = A(i, i);
}

}  // namespace dense
}  // namespace hymor
