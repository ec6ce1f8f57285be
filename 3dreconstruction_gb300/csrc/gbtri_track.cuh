// Per-track triangulation math shared by the FP64 parity kernels and the
// FP32 production kernel of gbtri.cu.  The functions are host-callable too,
// so that the CPU tests can run the same code against the reference's
// outputs.
#pragma once
#include <cmath>
#include <cuda_runtime.h>

namespace gbba {

// Inverse of a symmetric 3x3 given as [00, 01, 02, 11, 12, 22] (cofactors);
// false when the determinant is zero or not finite.
template <typename T>
__host__ __device__ __forceinline__ bool inv3t(const T A[6], T Ai[6]) {  // symmetric packed [00,01,02,11,12,22]
  const T c00 = A[3] * A[5] - A[4] * A[4], c01 = A[2] * A[4] - A[1] * A[5], c02 = A[1] * A[4] - A[2] * A[3];
  const T det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  if (!(fabs((double)det) > 0) || !((det - det) == T(0))) return false;  // zero, or not finite
  const T id = T(1) / det;
  Ai[0] = c00 * id;
  Ai[1] = c01 * id;
  Ai[2] = c02 * id;
  Ai[3] = (A[0] * A[5] - A[2] * A[2]) * id;
  Ai[4] = (A[1] * A[2] - A[0] * A[4]) * id;
  Ai[5] = (A[0] * A[3] - A[1] * A[1]) * id;
  return true;
}

// Smallest right singular vector of a 4x4 matrix by one-sided Jacobi (the
// nullspace of TriangulateDLT's design, libs/base/include/mvg/math/numeric.h:
// 228-240, in the same arithmetic as the reference's JacobiSVD to 1e-15).
__host__ __device__ inline void jacobi_nullspace4(double A[4][4], double x[4]) {
  double V[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int i = 0; i < 3; ++i)
      for (int j = i + 1; j < 4; ++j) {
        double a = 0, b = 0, g = 0;
        for (int r = 0; r < 4; ++r) {
          a += A[r][i] * A[r][i];
          b += A[r][j] * A[r][j];
          g += A[r][i] * A[r][j];
        }
        if (g == 0.0 || fabs(g) <= 1e-15 * sqrt(a * b)) continue;
        rotated = true;
        const double zeta = (b - a) / (2.0 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        for (int r = 0; r < 4; ++r) {
          const double ui = A[r][i], uj = A[r][j];
          A[r][i] = c * ui - s * uj;
          A[r][j] = s * ui + c * uj;
          const double vi = V[r][i], vj = V[r][j];
          V[r][i] = c * vi - s * vj;
          V[r][j] = s * vi + c * vj;
        }
      }
    if (!rotated) break;
  }
  int best = 0;
  double bn = 1e300;
  for (int i = 0; i < 4; ++i) {
    const double nrm = A[0][i] * A[0][i] + A[1][i] * A[1][i] + A[2][i] * A[2][i] + A[3][i] * A[3][i];
    if (nrm < bn) {
      bn = nrm;
      best = i;
    }
  }
  for (int r = 0; r < 4; ++r) x[r] = V[r][best];
}

// ------------------------------------------------ N-view nullspace of any track length
// TriangulateNView (triangulation_nview.cpp:8-24) takes the smallest right
// singular vector v = [X; alpha] of the 3n x (4+n) design whose view-i rows
// are [-P_i | x~_i e_i] (x~ = (x, y, 1)), and returns its head X.  The same
// vector is found here in O(n) work and O(1) state per track:
//   1. A Householder reflection H_i of view i's three rows maps x~_i to
//      c_i e_0 (|c_i| = |x~_i|).  Row 0 becomes [-h_i^T | c_i e_i] with
//      h_i = (H_i P_i)_0; rows 1-2, [-(H_i P_i)_{1,2} | 0], no longer involve
//      alpha and are rotated (Givens) into a 4x4 upper-triangular R.  Both
//      steps are orthogonal, so the singular vectors are unchanged.
//   2. Eliminating alpha (alpha_i = c_i h_i^T X / (c_i^2 - lambda)) leaves
//      the generalized problem  R^T R X = lambda G(lambda) X  with
//      G(lambda) = I + sum_i h_i h_i^T / (c_i^2 - lambda) (SPD), whose
//      smallest root lambda = sigma_min^2 is the fixed point of
//      lambda <- sigma_min(R L^-T)^2, G = L L^T.  lambda << c_i^2, so the
//      iteration contracts fast; three passes are used.
//   3. X = L^-T y for the smallest right singular vector y of R L^-T
//      (one-sided Jacobi on a 4x4), then [X; alpha] is scaled to unit norm.
// TriangulateNViewAlgebraic (:35-46) is the 2n x 4 design
// [[0,-1,y] P_i; [1,0,-x] P_i]: its rows go straight into R, and X is the
// smallest right singular vector of R.  Everything is templated on the
// arithmetic type: FP64 for the parity path, FP32 for the production path.

// Rotate `row` into the upper-triangular R (Givens).
template <typename T>
__host__ __device__ __forceinline__ void givens_in(T R[4][4], T row[4]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const T a = R[j][j], b = row[j];
    if (b == T(0)) continue;
    const T r = sqrt(a * a + b * b);
    const T c = a / r, s = b / r;
#pragma unroll
    for (int k = j; k < 4; ++k) {
      const T u = R[j][k], v = row[k];
      R[j][k] = c * u + s * v;
      row[k] = c * v - s * u;
    }
  }
}

// Householder reduction of one view (P row-major 3x4, pixel (x, y)):
// h = (H P)_0, g1 = (H P)_1, g2 = (H P)_2, c with H x~ = c e_0.
template <typename T>
__host__ __device__ __forceinline__ void view_house(const T* __restrict__ P, T x, T y, T h[4], T g1[4], T g2[4], T* c) {
  const T nx = sqrt(x * x + y * y + T(1));
  const T sg = x >= T(0) ? T(1) : T(-1);
  const T v0 = x + sg * nx, v1 = y, v2 = T(1);
  const T beta = T(2) / (v0 * v0 + v1 * v1 + v2 * v2);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T w = beta * (v0 * P[k] + v1 * P[4 + k] + v2 * P[8 + k]);
    h[k] = P[k] - v0 * w;
    g1[k] = P[4 + k] - v1 * w;
    g2[k] = P[8 + k] - v2 * w;
  }
  *c = -sg * nx;
}

// Smallest right singular vector of a 4x4 matrix B (one-sided Jacobi on its
// columns, V accumulated); returns sigma_min^2.
template <typename T>
__host__ __device__ __forceinline__ T min_right_singular4(T B[4][4], T y[4]) {
  T V[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) V[i][j] = i == j ? T(1) : T(0);
  const T tol = sizeof(T) == 8 ? T(1e-15) : T(1e-7);
  for (int sweep = 0; sweep < 30; ++sweep) {
    bool rotated = false;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i + 1; j < 4; ++j) {
        T a = 0, b = 0, g = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          a += B[r][i] * B[r][i];
          b += B[r][j] * B[r][j];
          g += B[r][i] * B[r][j];
        }
        if (g == T(0) || fabs(g) <= tol * sqrt(a * b)) continue;
        rotated = true;
        const T zeta = (b - a) / (T(2) * g);
        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T cs = T(1) / sqrt(T(1) + t * t), sn = cs * t;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const T ui = B[r][i], uj = B[r][j];
          B[r][i] = cs * ui - sn * uj;
          B[r][j] = sn * ui + cs * uj;
          const T vi = V[r][i], vj = V[r][j];
          V[r][i] = cs * vi - sn * vj;
          V[r][j] = sn * vi + cs * vj;
        }
      }
    if (!rotated) break;
  }
  int best = 0;
  T bn = T(0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const T nrm = B[0][i] * B[0][i] + B[1][i] * B[1][i] + B[2][i] * B[2][i] + B[3][i] * B[3][i];
    if (i == 0 || nrm < bn) {
      bn = nrm;
      best = i;
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) y[r] = V[r][best];
  return bn;
}

// Index of (i, j), i <= j, in a packed symmetric 4x4.
__host__ __device__ __forceinline__ constexpr int sym4(int i, int j) { return i <= j ? i * 4 - i * (i - 1) / 2 + (j - i) : j * 4 - j * (j - 1) / 2 + (i - j); }

// Generalized 4x4 step: with G = L L^T, the smallest right singular vector y
// of R L^-T gives X = L^-T y; returns sigma_min^2 (the next lambda).
template <typename T>
__host__ __device__ __forceinline__ T nview_solve4(const T R[4][4], const T G[10], T X[4]) {
  T L[4][4], Li[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) L[i][j] = Li[i][j] = T(0);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    T d = G[sym4(j, j)];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= L[j][k] * L[j][k];
    L[j][j] = sqrt(d);
#pragma unroll
    for (int i = j + 1; i < 4; ++i) {
      T v = G[sym4(i, j)];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= L[i][k] * L[j][k];
      L[i][j] = v / L[j][j];
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    Li[j][j] = T(1) / L[j][j];
#pragma unroll
    for (int i = j + 1; i < 4; ++i) {
      T v = T(0);
#pragma unroll
      for (int k = j; k < i; ++k) v -= L[i][k] * Li[k][j];
      Li[i][j] = v / L[i][i];
    }
  }
  T B[4][4], y[4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T v = T(0);
#pragma unroll
      for (int k = 0; k < 4; ++k) v += R[i][k] * Li[j][k];
      B[i][j] = v;
    }
  const T lam = min_right_singular4<T>(B, y);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    T v = T(0);
#pragma unroll
    for (int j = 0; j < 4; ++j) v += Li[j][i] * y[j];
    X[i] = v;
  }
  return lam;
}

// [X; alpha] scaled to unit norm, |alpha|^2 = X^T Q X.
template <typename T>
__host__ __device__ __forceinline__ void nview_normalize(const T Q[10], T X[4]) {
  T an = T(0), xn = T(0);
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    xn += X[a] * X[a];
#pragma unroll
    for (int b = 0; b < 4; ++b) an += X[a] * Q[sym4(a, b)] * X[b];
  }
  const T inv = T(1) / sqrt(xn + an);
#pragma unroll
  for (int i = 0; i < 4; ++i) X[i] *= inv;
}

// TriangulateNView of one track.  view(j, &P, &x, &y) gives view j's
// projection matrix (row-major 3x4) and pixel.  X: the head of the unit
// vector [X; alpha].
//
// kExact (the FP64 parity path): every fixed-point pass re-reads the views
// and accumulates G(lambda) = I + sum h h^T / (c^2 - lambda) exactly.
// Otherwise (the FP32 production path) one pass over the views accumulates
// the moments G_m = sum h h^T / c^(2m), m = 1..3, and every pass uses
//   G(lambda) = I + G_1 + lambda G_2 + lambda^2 G_3,
//   Q(lambda) = sum c^2 h h^T / (c^2 - lambda)^2 = G_1 + 2 lambda G_2 + 3 lambda^2 G_3,
// whose truncation error (lambda / c^2)^3 is far below FP32 rounding
// (lambda is a squared residual, c^2 >= 1 and ~1e6 in pixels).
template <typename T, bool kExact = true, typename Views>
__host__ __device__ void nview_track(const Views& view, int n, T X[4]) {
  T R[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) R[i][j] = T(0);
  T lam = T(0), Q[10];
#pragma unroll
  for (int i = 0; i < 4; ++i) X[i] = T(0);
  if (!kExact) {
    T M1[10], M2[10], M3[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) M1[i] = M2[i] = M3[i] = T(0);
    for (int j = 0; j < n; ++j) {
      const T* P;
      T px, py;
      view(j, &P, &px, &py);
      T h[4], g1[4], g2[4], c;
      view_house<T>(P, px, py, h, g1, g2, &c);
      givens_in<T>(R, g1);
      givens_in<T>(R, g2);
      const T w1 = T(1) / (c * c), w2 = w1 * w1, w3 = w2 * w1;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a; b < 4; ++b) {
          const T hh = h[a] * h[b];
          M1[sym4(a, b)] += w1 * hh;
          M2[sym4(a, b)] += w2 * hh;
          M3[sym4(a, b)] += w3 * hh;
        }
    }
    for (int pass = 0; pass < 3; ++pass) {
      T G[10];
#pragma unroll
      for (int i = 0; i < 10; ++i) {
        G[i] = M1[i] + lam * (M2[i] + lam * M3[i]);
        Q[i] = M1[i] + lam * (T(2) * M2[i] + T(3) * lam * M3[i]);
      }
      G[sym4(0, 0)] += T(1);
      G[sym4(1, 1)] += T(1);
      G[sym4(2, 2)] += T(1);
      G[sym4(3, 3)] += T(1);
      lam = nview_solve4<T>(R, G, X);
    }
    nview_normalize<T>(Q, X);
    return;
  }
  for (int pass = 0; pass < 3; ++pass) {
    T G[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) G[i] = T(0), Q[i] = T(0);
    G[sym4(0, 0)] = G[sym4(1, 1)] = G[sym4(2, 2)] = G[sym4(3, 3)] = T(1);
    for (int j = 0; j < n; ++j) {
      const T* P;
      T px, py;
      view(j, &P, &px, &py);
      T h[4], g1[4], g2[4], c;
      view_house<T>(P, px, py, h, g1, g2, &c);
      if (pass == 0) {
        givens_in<T>(R, g1);
        givens_in<T>(R, g2);
      }
      const T w = T(1) / (c * c - lam);
      const T q = c * c * w * w;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a; b < 4; ++b) {
          G[sym4(a, b)] += w * h[a] * h[b];
          Q[sym4(a, b)] += q * h[a] * h[b];
        }
    }
    lam = nview_solve4<T>(R, G, X);
  }
  // |alpha|^2 = X^T Q X with Q = sum c^2 h h^T / (c^2 - lambda)^2
  nview_normalize<T>(Q, X);
}

// TriangulateNViewAlgebraic of one track: unit X.
template <typename T, typename Views>
__host__ __device__ void algebraic_track(const Views& view, int n, T X[4]) {
  T R[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) R[i][j] = T(0);
  for (int j = 0; j < n; ++j) {
    const T* P;
    T px, py;
    view(j, &P, &px, &py);
    T a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a[k] = -P[4 + k] + py * P[8 + k];
      b[k] = P[k] - px * P[8 + k];
    }
    givens_in<T>(R, a);
    givens_in<T>(R, b);
  }
  min_right_singular4<T>(R, X);
}

// Triangulation::compute(3) (triangulation_nview.cpp:62-121): three
// weighted linear solves, weights 1/z from the previous estimate.
template <typename T, typename Views>
__host__ __device__ bool iterative_track(const Views& view, int n, T Xc[3]) {
  Xc[0] = Xc[1] = Xc[2] = T(0);
  bool ok = true;
  for (int it = 0; it < 3; ++it) {
    T A[6] = {0, 0, 0, 0, 0, 0}, r[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
      const T* Pi;
      T px, py;
      view(i, &Pi, &px, &py);
      const T wi = it == 0 ? T(1) : T(1) / (Pi[8] * Xc[0] + Pi[9] * Xc[1] + Pi[10] * Xc[2] + Pi[11]);
      T v1[3], v2[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        v1[j] = wi * (Pi[j] - px * Pi[8 + j]);
        v2[j] = wi * (Pi[4 + j] - py * Pi[8 + j]);
        r[j] += wi * (v1[j] * (px * Pi[11] - Pi[3]) + v2[j] * (py * Pi[11] - Pi[7]));
      }
      A[0] += v1[0] * v1[0] + v2[0] * v2[0];
      A[1] += v1[0] * v1[1] + v2[0] * v2[1];
      A[2] += v1[0] * v1[2] + v2[0] * v2[2];
      A[3] += v1[1] * v1[1] + v2[1] * v2[1];
      A[4] += v1[1] * v1[2] + v2[1] * v2[2];
      A[5] += v1[2] * v1[2] + v2[2] * v2[2];
    }
    T Ai[6];
    ok = inv3t<T>(A, Ai);
    Xc[0] = Ai[0] * r[0] + Ai[1] * r[1] + Ai[2] * r[2];
    Xc[1] = Ai[1] * r[0] + Ai[3] * r[1] + Ai[4] * r[2];
    Xc[2] = Ai[2] * r[0] + Ai[4] * r[1] + Ai[5] * r[2];
  }
  return ok;
}

}  // namespace gbba
