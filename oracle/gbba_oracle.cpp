// CPU oracle for the GB300 bundle-adjustment / triangulation engine.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++ on the host, the
// algorithms of the reference path so that the CUDA implementation can be
// checked against it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline load it; the product library never links or calls it.
//
// Parity of this restatement is pinned against the reference itself: the
// reference's own ceres/Eigen code is compiled from its sources by
// oracle/Makefile (target `ref`) and tests/golden/make_golden.py records its
// outputs as fixtures in tests/golden/, which the CPU tests compare with.
//
// What is restated (reference file:line):
//   - ceres::AngleAxisRotatePoint            3rdparty/ceres/include/ceres/rotation.h:566-625
//   - ComputeResidual / ErrorFunc_Refine_Camera_3DPoints / PinholeReprojectionError_*
//                                            libs/sfm/include/mvg/sfm/pinhole_ceres_functor.h:24-54,
//                                            pinhole_brown_rt_ceres_functor.h:60-107,
//                                            sfm_bundle_adjustment_helper_tonly.h:11-76
//   - ApplyRadialDistortionIntrinsics        libs/camera/include/mvg/camera/brown_pinhole_camera.h:15-41
//   - AutoDiff (forward-mode dual numbers)   include/ceres/jet.h:171-227, internal/autodiff.h:231
//   - HuberLoss + Corrector                  internal/ceres/loss_function.cc:47-61, corrector.cc:41-155
//   - cost = 1/2 rho                         internal/ceres/residual_block.cc:160-166
//   - Jacobi scaling                         internal/ceres/trust_region_minimizer.cc:103-108
//   - LM step / radius update                internal/ceres/levenberg_marquardt_strategy.cc:65-160
//   - trust region loop + terminations       internal/ceres/trust_region_minimizer.cc:110-716
//   - Schur elimination + back substitution  internal/ceres/schur_eliminator_impl.h:173-370
//   - dense Cholesky of S                    internal/ceres/schur_complement_solver.cc:180-222
//   - TriangulateDLT / Nullspace             libs/multiview/src/triangulation.cpp:10-29,
//                                            libs/base/include/mvg/math/numeric.h:228-240
//   - TriangulateNView(/Algebraic), Triangulation::compute/error
//                                            libs/multiview/src/triangulation_nview.cpp:8-121
//   - BundleAdjustment's problem assembly    libs/sfm/src/sfm_incremental_engine.cpp:1250-1393,
//     over the engine's std::map state, with RotationMatrixToAngleAxis
//                                            include/ceres/rotation.h:266-370
//   - AC-RANSAC model scoring (residuals, sort, bestNFA)
//                                            libs/feature/include/mvg/feature/estimator_acransac.h:40-200
#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <set>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gbba.h"
#include "../include/gbtri.h"
#include "../include/gbsfm.h"

namespace {

// ------------------------------------------------------------------ dual numbers
template <int N>
struct Jet {
  double a;
  double v[N];
  Jet() : a(0) { for (int i = 0; i < N; ++i) v[i] = 0; }
  explicit Jet(double x) : a(x) { for (int i = 0; i < N; ++i) v[i] = 0; }
  Jet(double x, int k) : a(x) { for (int i = 0; i < N; ++i) v[i] = 0; v[k] = 1; }
};
template <int N> Jet<N> operator+(const Jet<N>& f, const Jet<N>& g) { Jet<N> h(f.a + g.a); for (int i = 0; i < N; ++i) h.v[i] = f.v[i] + g.v[i]; return h; }
template <int N> Jet<N> operator-(const Jet<N>& f, const Jet<N>& g) { Jet<N> h(f.a - g.a); for (int i = 0; i < N; ++i) h.v[i] = f.v[i] - g.v[i]; return h; }
template <int N> Jet<N> operator-(const Jet<N>& f) { Jet<N> h(-f.a); for (int i = 0; i < N; ++i) h.v[i] = -f.v[i]; return h; }
template <int N> Jet<N> operator*(const Jet<N>& f, const Jet<N>& g) { Jet<N> h(f.a * g.a); for (int i = 0; i < N; ++i) h.v[i] = f.a * g.v[i] + f.v[i] * g.a; return h; }
template <int N> Jet<N> operator/(const Jet<N>& f, const Jet<N>& g) {
  const double ig = 1.0 / g.a, q = f.a * ig;
  Jet<N> h(q); for (int i = 0; i < N; ++i) h.v[i] = (f.v[i] - q * g.v[i]) * ig; return h;
}
template <int N> Jet<N> operator*(double s, const Jet<N>& f) { Jet<N> h(s * f.a); for (int i = 0; i < N; ++i) h.v[i] = s * f.v[i]; return h; }
template <int N> Jet<N> operator/(double s, const Jet<N>& g) { return Jet<N>(s) / g; }
template <int N> Jet<N>& operator+=(Jet<N>& f, const Jet<N>& g) { f = f + g; return f; }
template <int N> Jet<N> sqrt(const Jet<N>& f) { const double s = std::sqrt(f.a); Jet<N> h(s); const double d = 0.5 / s; for (int i = 0; i < N; ++i) h.v[i] = d * f.v[i]; return h; }
template <int N> Jet<N> cos(const Jet<N>& f) { Jet<N> h(std::cos(f.a)); const double d = -std::sin(f.a); for (int i = 0; i < N; ++i) h.v[i] = d * f.v[i]; return h; }
template <int N> Jet<N> sin(const Jet<N>& f) { Jet<N> h(std::sin(f.a)); const double d = std::cos(f.a); for (int i = 0; i < N; ++i) h.v[i] = d * f.v[i]; return h; }
template <int N> double Scalar(const Jet<N>& f) { return f.a; }
inline double Scalar(double f) { return f; }
template <typename T> T Lift(double x) { return T(x); }

// ------------------------------------------------------------------ functors
template <typename T>
void AngleAxisRotate(const T w[3], const T p[3], T out[3]) {
  const T theta2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (Scalar(theta2) > std::numeric_limits<double>::epsilon()) {
    using std::cos; using std::sin; using std::sqrt;
    const T theta = sqrt(theta2);
    const T c = cos(theta), s = sin(theta);
    const T ith = 1.0 / theta;
    const T u[3] = {w[0] * ith, w[1] * ith, w[2] * ith};
    const T uxp[3] = {u[1] * p[2] - u[2] * p[1], u[2] * p[0] - u[0] * p[2], u[0] * p[1] - u[1] * p[0]};
    const T k = (u[0] * p[0] + u[1] * p[1] + u[2] * p[2]) * (T(1.0) - c);
    for (int i = 0; i < 3; ++i) out[i] = p[i] * c + uxp[i] * s + u[i] * k;
  } else {
    const T wxp[3] = {w[1] * p[2] - w[2] * p[1], w[2] * p[0] - w[0] * p[2], w[0] * p[1] - w[1] * p[0]};
    for (int i = 0; i < 3; ++i) out[i] = p[i] + wxp[i];
  }
}

int ModelK(int model) { return model == GBBA_PINHOLE_F ? 1 : model == GBBA_RADIAL_K3 ? 6 : 8; }

template <typename T>
void Residual(int model, const T* K, const T* E, const T* X, const double* obs, T* r) {
  T p[3];
  AngleAxisRotate(E, X, p);
  p[0] = p[0] + E[3]; p[1] = p[1] + E[4]; p[2] = p[2] + E[5];
  const T x = p[0] / p[2], y = p[1] / p[2];
  if (model == GBBA_PINHOLE_F) {
    r[0] = K[0] * x - T(obs[0]);
    r[1] = K[0] * y - T(obs[1]);
    return;
  }
  const T r2 = x * x + y * y, r4 = r2 * r2, r6 = r4 * r2;
  const T rc = T(1) + K[3] * r2 + K[4] * r4 + K[5] * r6;
  T xd = x * rc, yd = y * rc;
  if (model == GBBA_BROWN_T2) {
    xd = xd + T(2) * K[6] * x * y + K[7] * (r2 + T(2) * x * x);
    yd = yd + T(2) * K[7] * x * y + K[6] * (r2 + T(2) * y * y);
  }
  r[0] = K[1] + K[0] * xd - T(obs[0]);
  r[1] = K[2] + K[0] * yd - T(obs[1]);
}

struct Loss {
  int type; double a, b;
  // ceres HuberLoss::Evaluate (loss_function.cc:47-61); TrivialLoss otherwise.
  void Eval(double s, double rho[3]) const {
    if (type == GBBA_LOSS_HUBER && s > b) {
      const double r = std::sqrt(s);
      rho[0] = 2.0 * a * r - b;
      rho[1] = std::max(std::numeric_limits<double>::min(), a / r);
      rho[2] = -rho[1] / (2.0 * s);
    } else {
      rho[0] = s; rho[1] = 1.0; rho[2] = 0.0;
    }
  }
};

// Per-observation evaluation: robustified cost, corrected residual and the
// corrected full Jacobian row pair over [extrinsic(6) | intrinsic(k) | point(3)].
template <int N>
void EvalObs(int model, const double* K, const double* E, const double* X, const double* obs,
             const Loss& loss, double* cost, double* r_raw, double* r_c, double* J /* [2][N] or NULL */) {
  const int k = ModelK(model);
  if (J == NULL) {
    double r[2];
    Residual<double>(model, K, E, X, obs, r);
    const double s = r[0] * r[0] + r[1] * r[1];
    double rho[3];
    loss.Eval(s, rho);
    *cost = (loss.type == GBBA_LOSS_SQUARED) ? 0.5 * s : 0.5 * rho[0];
    if (r_raw) { r_raw[0] = r[0]; r_raw[1] = r[1]; }
    if (r_c) { const double sc = (loss.type == GBBA_LOSS_SQUARED) ? 1.0 : std::sqrt(rho[1]); r_c[0] = r[0] * sc; r_c[1] = r[1] * sc; }
    return;
  }
  Jet<N> je[6], jk[8], jx[3], jr[2];
  for (int i = 0; i < 6; ++i) je[i] = Jet<N>(E[i], i);
  for (int i = 0; i < k; ++i) jk[i] = Jet<N>(K[i], 6 + i);
  for (int i = 0; i < 3; ++i) jx[i] = Jet<N>(X[i], 6 + k + i);
  Residual<Jet<N> >(model, jk, je, jx, obs, jr);
  const double r[2] = {jr[0].a, jr[1].a};
  const double s = r[0] * r[0] + r[1] * r[1];
  double rho[3];
  loss.Eval(s, rho);
  double sc = 1.0;
  if (loss.type == GBBA_LOSS_SQUARED) {
    *cost = 0.5 * s;
  } else {
    *cost = 0.5 * rho[0];
    // Corrector (corrector.cc:41-155).  For Huber rho'' <= 0 everywhere, so
    // both residual and Jacobian are scaled by sqrt(rho').
    sc = std::sqrt(rho[1]);
  }
  if (r_raw) { r_raw[0] = r[0]; r_raw[1] = r[1]; }
  if (r_c) { r_c[0] = r[0] * sc; r_c[1] = r[1] * sc; }
  for (int row = 0; row < 2; ++row)
    for (int c = 0; c < N; ++c) J[row * N + c] = jr[row].v[c] * sc;
}

typedef void (*EvalFn)(int, const double*, const double*, const double*, const double*, const Loss&, double*, double*, double*, double*);
EvalFn PickEval(int model) {
  if (model == GBBA_PINHOLE_F) return &EvalObs<10>;
  if (model == GBBA_RADIAL_K3) return &EvalObs<15>;
  return &EvalObs<17>;
}

double Now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

// ------------------------------------------------------------------ BA state
struct BA {
  const gbba_problem* P;
  int model, k, nb;  // nb = 6 + k + 3 jacobian row width
  int64_t nc, ni, np, no;
  Loss loss;
  EvalFn eval;
  // column maps: -1 = held, else index among the reduced (camera-side) columns
  std::vector<int64_t> ext_col, intr_col;
  int64_t n_red;      // camera-side variable columns (size of S)
  int64_t n_pt_cols;  // 3 * np
  // observations grouped by point
  std::vector<int64_t> pt_off, pt_obs;
  // x = parameters (copies)
  std::vector<double> ext, intr, pts;
  // per obs
  std::vector<double> J, rc;  // J [no][2][nb], corrected residual [no][2]
  // scaling over reduced columns: camera-side [n_red] then points [3 np]
  std::vector<double> scale_c, scale_p;
};

void InitBA(BA& b, const gbba_problem* P, const gbba_options* o) {
  b.P = P;
  b.model = P->camera_model;
  b.k = ModelK(b.model);
  b.nb = 6 + b.k + 3;
  b.nc = P->num_cameras; b.ni = P->num_intrinsics; b.np = P->num_points; b.no = P->num_observations;
  b.loss.type = o->loss_type; b.loss.a = o->loss_scale; b.loss.b = o->loss_scale * o->loss_scale;
  b.eval = PickEval(b.model);
  b.ext.assign(P->extrinsics, P->extrinsics + 6 * b.nc);
  b.intr.assign(P->intrinsics, P->intrinsics + b.k * b.ni);
  b.pts.assign(P->points, P->points + 3 * b.np);
  // Which blocks are used at all (ceres drops parameter blocks without residuals).
  std::vector<char> cam_used(b.nc, 0), intr_used(b.ni, 0);
  for (int64_t i = 0; i < b.no; ++i) { cam_used[P->camera_index[i]] = 1; intr_used[P->intrinsic_index[i]] = 1; }
  b.ext_col.assign(6 * b.nc, -1);
  b.intr_col.assign(b.k * b.ni, -1);
  int64_t col = 0;
  for (int64_t c = 0; c < b.nc; ++c) {
    if (!cam_used[c] || (P->camera_constant && P->camera_constant[c])) continue;
    for (int j = 0; j < 6; ++j) if (!(P->extrinsic_fixed_mask & (1u << j))) b.ext_col[6 * c + j] = col++;
  }
  for (int64_t i = 0; i < b.ni; ++i) {
    if (!intr_used[i] || (P->intrinsic_constant && P->intrinsic_constant[i])) continue;
    for (int j = 0; j < b.k; ++j) if (!(P->intrinsic_fixed_mask & (1u << j))) b.intr_col[b.k * i + j] = col++;
  }
  b.n_red = col;
  b.n_pt_cols = 3 * b.np;
  b.pt_off.assign(b.np + 1, 0);
  for (int64_t i = 0; i < b.no; ++i) b.pt_off[P->point_index[i] + 1]++;
  for (int64_t p = 0; p < b.np; ++p) b.pt_off[p + 1] += b.pt_off[p];
  b.pt_obs.resize(b.no);
  std::vector<int64_t> fill(b.pt_off.begin(), b.pt_off.end() - 1);
  for (int64_t i = 0; i < b.no; ++i) b.pt_obs[fill[P->point_index[i]]++] = i;
  b.J.resize((size_t)b.no * 2 * b.nb);
  b.rc.resize((size_t)b.no * 2);
}

// Cost (and optionally J, corrected residuals) at parameters (E, K, X).
// Returns false if any value is non-finite (ceres treats that as a failed evaluation).
bool Evaluate(BA& b, const double* E, const double* K, const double* X, double* cost, bool with_jacobian) {
  const gbba_problem* P = b.P;
  double total = 0.0;
  bool ok = true;
#pragma omp parallel for reduction(+ : total) reduction(&& : ok) schedule(static)
  for (int64_t i = 0; i < b.no; ++i) {
    double c;
    const double* e = E + 6 * (int64_t)P->camera_index[i];
    const double* kk = K + b.k * (int64_t)P->intrinsic_index[i];
    const double* x = X + 3 * (int64_t)P->point_index[i];
    b.eval(b.model, kk, e, x, P->observations + 2 * i, b.loss, &c, NULL, with_jacobian ? &b.rc[2 * i] : NULL,
           with_jacobian ? &b.J[(size_t)i * 2 * b.nb] : NULL);
    total += c;
    ok = ok && std::isfinite(c);
  }
  *cost = total;
  return ok && std::isfinite(total);
}

// Column of an observation's jacobian entry `c` (0..nb-1) among the reduced
// camera columns, or -1 (point columns are handled separately).
inline int64_t CamCol(const BA& b, int64_t obs, int c) {
  if (c < 6) return b.ext_col[6 * (int64_t)b.P->camera_index[obs] + c];
  return b.intr_col[b.k * (int64_t)b.P->intrinsic_index[obs] + (c - 6)];
}

// Squared column norms of the (corrected) Jacobian: camera-side and points.
void ColumnNorms(const BA& b, std::vector<double>& cam, std::vector<double>& pt, bool scaled) {
  cam.assign(b.n_red, 0.0);
  pt.assign(b.n_pt_cols, 0.0);
  for (int64_t i = 0; i < b.no; ++i) {
    const double* J = &b.J[(size_t)i * 2 * b.nb];
    for (int c = 0; c < 6 + b.k; ++c) {
      const int64_t col = CamCol(b, i, c);
      if (col < 0) continue;
      const double s = scaled ? b.scale_c[col] : 1.0;
      cam[col] += (J[c] * s) * (J[c] * s) + (J[b.nb + c] * s) * (J[b.nb + c] * s);
    }
    const int64_t p = b.P->point_index[i];
    for (int c = 0; c < 3; ++c) {
      const double s = scaled ? b.scale_p[3 * p + c] : 1.0;
      const double j0 = J[6 + b.k + c] * s, j1 = J[b.nb + 6 + b.k + c] * s;
      pt[3 * p + c] += j0 * j0 + j1 * j1;
    }
  }
}

// Scale the stored Jacobian columns in place (ceres ScaleColumns).
void ScaleJacobian(BA& b) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < b.no; ++i) {
    double* J = &b.J[(size_t)i * 2 * b.nb];
    for (int c = 0; c < 6 + b.k; ++c) {
      const int64_t col = CamCol(b, i, c);
      const double s = col < 0 ? 0.0 : b.scale_c[col];
      J[c] *= s; J[b.nb + c] *= s;
    }
    const int64_t p = b.P->point_index[i];
    for (int c = 0; c < 3; ++c) { J[6 + b.k + c] *= b.scale_p[3 * p + c]; J[b.nb + 6 + b.k + c] *= b.scale_p[3 * p + c]; }
  }
}

// Dense Cholesky (lower, in place, row-major n x n); false if not positive definite.
bool Cholesky(std::vector<double>& A, int64_t n) {
  const int64_t NB = 64;
  for (int64_t k0 = 0; k0 < n; k0 += NB) {
    const int64_t k1 = std::min(n, k0 + NB);
    for (int64_t j = k0; j < k1; ++j) {  // factor the panel columns
      double d = A[j * n + j];
      for (int64_t t = k0; t < j; ++t) d -= A[j * n + t] * A[j * n + t];
      if (!(d > 0.0) || !std::isfinite(d)) return false;
      d = std::sqrt(d);
      A[j * n + j] = d;
#pragma omp parallel for schedule(static)
      for (int64_t i = j + 1; i < n; ++i) {
        double v = A[i * n + j];
        for (int64_t t = k0; t < j; ++t) v -= A[i * n + t] * A[j * n + t];
        A[i * n + j] = v / d;
      }
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t i = k1; i < n; ++i)  // trailing update (lower triangle)
      for (int64_t j = k1; j <= i; ++j) {
        double v = 0.0;
        for (int64_t t = k0; t < k1; ++t) v += A[i * n + t] * A[j * n + t];
        A[i * n + j] -= v;
      }
  }
  return true;
}

void CholSolve(const std::vector<double>& L, int64_t n, std::vector<double>& x) {
  for (int64_t i = 0; i < n; ++i) { double v = x[i]; for (int64_t t = 0; t < i; ++t) v -= L[i * n + t] * x[t]; x[i] = v / L[i * n + i]; }
  for (int64_t i = n - 1; i >= 0; --i) { double v = x[i]; for (int64_t t = i + 1; t < n; ++t) v -= L[t * n + i] * x[t]; x[i] = v / L[i * n + i]; }
}

// 3x3 symmetric positive definite inverse by Cholesky (ceres: ete.llt().solve(I)).
bool Inverse3(const double A[9], double Ai[9]) {
  const double l00 = std::sqrt(A[0]);
  if (!(l00 > 0)) return false;
  const double l10 = A[3] / l00, l20 = A[6] / l00;
  const double d1 = A[4] - l10 * l10;
  if (!(d1 > 0)) return false;
  const double l11 = std::sqrt(d1), l21 = (A[7] - l20 * l10) / l11;
  const double d2 = A[8] - l20 * l20 - l21 * l21;
  if (!(d2 > 0)) return false;
  const double l22 = std::sqrt(d2);
  for (int c = 0; c < 3; ++c) {
    double e[3] = {c == 0 ? 1.0 : 0.0, c == 1 ? 1.0 : 0.0, c == 2 ? 1.0 : 0.0};
    const double y0 = e[0] / l00, y1 = (e[1] - l10 * y0) / l11, y2 = (e[2] - l20 * y0 - l21 * y1) / l22;
    const double x2 = y2 / l22, x1 = (y1 - l21 * x2) / l11, x0 = (y0 - l10 * x1 - l20 * x2) / l00;
    Ai[0 * 3 + c] = x0; Ai[1 * 3 + c] = x1; Ai[2 * 3 + c] = x2;
  }
  return true;
}

// Solve (J^T J + D^T D) y = J^T r by Schur complement on the point blocks;
// step = -y.  Returns false on linear solver failure.
bool SchurSolve(BA& b, const std::vector<double>& Dc2, const std::vector<double>& Dp2,
                std::vector<double>& step_c, std::vector<double>& step_p) {
  const int64_t n = b.n_red;
  const int nb = b.nb, kc = 6 + b.k;
  std::vector<double> S((size_t)n * n, 0.0), rhs(n, 0.0);
  std::vector<double> Einv((size_t)b.np * 9), gp((size_t)b.np * 3);
  bool ok = true;
  // Per point: ete = D^2 + sum E'E, g = sum E'r, inverse (schur_eliminator_impl.h:240-275).
#pragma omp parallel for schedule(static) reduction(&& : ok)
  for (int64_t p = 0; p < b.np; ++p) {
    double ete[9] = {0}, g[3] = {0};
    ete[0] = Dp2[3 * p]; ete[4] = Dp2[3 * p + 1]; ete[8] = Dp2[3 * p + 2];
    for (int64_t q = b.pt_off[p]; q < b.pt_off[p + 1]; ++q) {
      const int64_t o = b.pt_obs[q];
      const double* J = &b.J[(size_t)o * 2 * nb];
      const double* r = &b.rc[2 * o];
      for (int row = 0; row < 2; ++row) {
        const double* e = J + row * nb + kc;
        for (int i = 0; i < 3; ++i) { g[i] += e[i] * r[row]; for (int j = 0; j < 3; ++j) ete[3 * i + j] += e[i] * e[j]; }
      }
    }
    ok = ok && Inverse3(ete, &Einv[9 * p]);
    for (int i = 0; i < 3; ++i) gp[3 * p + i] = g[i];
  }
  if (!ok) return false;
  // S = diag(Dc^2) + sum F'F - sum_p (F'E) ete^-1 (E'F); rhs = F'r - (F'E) ete^-1 g.
  // Rows are partitioned over threads so that every S entry has one writer.
#pragma omp parallel
  {
    int tid = 0, nt = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num(); nt = omp_get_num_threads();
#endif
    const int64_t r0 = n * tid / nt, r1 = n * (tid + 1) / nt;
    for (int64_t i = r0; i < r1; ++i) S[(size_t)i * n + i] += Dc2[i];
    std::vector<double> Ya, Yb;  // F'E (kc x 3) for obs a, b
    for (int64_t p = 0; p < b.np; ++p) {
      const double* Ei = &Einv[9 * p];
      for (int64_t qa = b.pt_off[p]; qa < b.pt_off[p + 1]; ++qa) {
        const int64_t oa = b.pt_obs[qa];
        const double* Ja = &b.J[(size_t)oa * 2 * nb];
        int64_t cola[16];
        bool any = false;
        for (int c = 0; c < kc; ++c) { cola[c] = CamCol(b, oa, c); any = any || (cola[c] >= r0 && cola[c] < r1); }
        if (!any) continue;
        // Y_a = F_a' E_a ete^-1  (kc x 3), and F_a' r_a
        double FE[16][3], Y[16][3];
        for (int c = 0; c < kc; ++c)
          for (int j = 0; j < 3; ++j) FE[c][j] = Ja[c] * Ja[kc + j] + Ja[nb + c] * Ja[nb + kc + j];
        for (int c = 0; c < kc; ++c)
          for (int j = 0; j < 3; ++j) Y[c][j] = FE[c][0] * Ei[0 * 3 + j] + FE[c][1] * Ei[1 * 3 + j] + FE[c][2] * Ei[2 * 3 + j];
        const double* ra = &b.rc[2 * oa];
        for (int c = 0; c < kc; ++c) {
          const int64_t ca = cola[c];
          if (ca < r0 || ca >= r1) continue;
          rhs[ca] += Ja[c] * ra[0] + Ja[nb + c] * ra[1];
          rhs[ca] -= Y[c][0] * gp[3 * p] + Y[c][1] * gp[3 * p + 1] + Y[c][2] * gp[3 * p + 2];
          // F_a' F_a (same observation)
          for (int d = 0; d < kc; ++d) {
            const int64_t cb = cola[d];
            if (cb < 0) continue;
            S[(size_t)ca * n + cb] += Ja[c] * Ja[d] + Ja[nb + c] * Ja[nb + d];
          }
          // - Y_a (E_b' F_b) over all observations b of the point
          for (int64_t qb = b.pt_off[p]; qb < b.pt_off[p + 1]; ++qb) {
            const int64_t ob = b.pt_obs[qb];
            const double* Jb = &b.J[(size_t)ob * 2 * nb];
            for (int d = 0; d < kc; ++d) {
              const int64_t cb = CamCol(b, ob, d);
              if (cb < 0) continue;
              double v = 0.0;
              for (int j = 0; j < 3; ++j) v += Y[c][j] * (Jb[kc + j] * Jb[d] + Jb[nb + kc + j] * Jb[nb + d]);
              S[(size_t)ca * n + cb] -= v;
            }
          }
        }
      }
    }
  }
  std::vector<double> z = rhs;
  if (n > 0) {
    if (!Cholesky(S, n)) return false;
    CholSolve(S, n, z);
  }
  for (int64_t i = 0; i < n; ++i) if (!std::isfinite(z[i])) return false;
  // Back substitution: y_p = ete^-1 (E'r - E'F z)  (schur_eliminator_impl.h:301-370)
  step_c.assign(n, 0.0);
  step_p.assign(3 * b.np, 0.0);
  for (int64_t i = 0; i < n; ++i) step_c[i] = -z[i];
  bool finite = true;
#pragma omp parallel for schedule(static) reduction(&& : finite)
  for (int64_t p = 0; p < b.np; ++p) {
    double g[3] = {gp[3 * p], gp[3 * p + 1], gp[3 * p + 2]};
    for (int64_t q = b.pt_off[p]; q < b.pt_off[p + 1]; ++q) {
      const int64_t o = b.pt_obs[q];
      const double* J = &b.J[(size_t)o * 2 * nb];
      double fz[2] = {0, 0};
      for (int c = 0; c < kc; ++c) { const int64_t col = CamCol(b, o, c); if (col < 0) continue; fz[0] += J[c] * z[col]; fz[1] += J[nb + c] * z[col]; }
      for (int j = 0; j < 3; ++j) g[j] -= J[kc + j] * fz[0] + J[nb + kc + j] * fz[1];
    }
    const double* Ei = &Einv[9 * p];
    for (int i = 0; i < 3; ++i) {
      const double y = Ei[3 * i] * g[0] + Ei[3 * i + 1] * g[1] + Ei[3 * i + 2] * g[2];
      step_p[3 * p + i] = -y;
      finite = finite && std::isfinite(y);
    }
  }
  return finite;
}

// Apply delta (reduced scaled step already multiplied by the scale) to x.
void Plus(const BA& b, const std::vector<double>& dc, const std::vector<double>& dp,
          std::vector<double>& E, std::vector<double>& K, std::vector<double>& X) {
  E = b.ext; K = b.intr; X = b.pts;
  for (int64_t i = 0; i < 6 * b.nc; ++i) if (b.ext_col[i] >= 0) E[i] += dc[b.ext_col[i]];
  for (int64_t i = 0; i < b.k * b.ni; ++i) if (b.intr_col[i] >= 0) K[i] += dc[b.intr_col[i]];
  for (int64_t i = 0; i < 3 * b.np; ++i) X[i] += dp[i];
}

// Norm of the minimizer's parameter vector: ceres keeps non-constant blocks
// at their global size (a SubsetParameterization block keeps all of its
// coordinates); held extrinsic coordinates are constant functor data in the
// reference (PinholeReprojectionError_t) and are not part of it.
double XNorm(const BA& b) {
  double s = 0.0;
  for (int64_t i = 0; i < 6 * b.nc; ++i) if (b.ext_col[i] >= 0) s += b.ext[i] * b.ext[i];
  for (int64_t g = 0; g < b.ni; ++g) {
    bool var = false;
    for (int j = 0; j < b.k; ++j) var = var || b.intr_col[b.k * g + j] >= 0;
    if (var) for (int j = 0; j < b.k; ++j) s += b.intr[b.k * g + j] * b.intr[b.k * g + j];
  }
  for (int64_t i = 0; i < 3 * b.np; ++i) s += b.pts[i] * b.pts[i];
  return std::sqrt(s);
}

double GradientMaxNorm(const BA& b) {
  // gradient of the robustified problem in local (unscaled) coordinates
  std::vector<double> gc(b.n_red, 0.0), gpt(3 * b.np, 0.0);
  for (int64_t i = 0; i < b.no; ++i) {
    const double* J = &b.J[(size_t)i * 2 * b.nb];
    const double* r = &b.rc[2 * i];
    for (int c = 0; c < 6 + b.k; ++c) { const int64_t col = CamCol(b, i, c); if (col >= 0) gc[col] += J[c] * r[0] + J[b.nb + c] * r[1]; }
    const int64_t p = b.P->point_index[i];
    for (int c = 0; c < 3; ++c) gpt[3 * p + c] += J[6 + b.k + c] * r[0] + J[b.nb + 6 + b.k + c] * r[1];
  }
  double m = 0.0;
  for (double v : gc) m = std::max(m, std::fabs(v));
  for (double v : gpt) m = std::max(m, std::fabs(v));
  return m;
}

}  // namespace

extern "C" {

// Restatement of ceres::Solve(TrustRegionMinimizer + LevenbergMarquardtStrategy
// + Schur complement) on a host problem.  Writes the refined parameters back
// when the solution is usable.  iteration_costs (may be NULL) receives the
// ceres Summary::iterations[i].cost sequence (at most max_costs entries).
int oracle_ba_solve(const gbba_problem* P, const gbba_options* o, gbba_summary* S,
                    double* iteration_costs, int max_costs, int num_threads) {
#ifdef _OPENMP
  if (num_threads > 0) omp_set_num_threads(num_threads);
#endif
  const double t0 = Now();
  std::memset(S, 0, sizeof(*S));
  BA b;
  InitBA(b, P, o);
  S->reduced_system_size = b.n_red;
  int ncost = 0;
  auto push_cost = [&](double c) { if (iteration_costs && ncost < max_costs) iteration_costs[ncost] = c; ++ncost; };

  double cost;
  if (!Evaluate(b, b.ext.data(), b.intr.data(), b.pts.data(), &cost, true)) {
    S->termination_type = GBBA_FAILURE; S->usable = 0; return GBBA_ERROR_NUMERICAL;
  }
  S->initial_cost = cost;
  push_cost(cost);
  double grad_max = GradientMaxNorm(b);
  auto finish = [&](int term) {
    S->termination_type = term;
    S->usable = (term != GBBA_FAILURE) ? 1 : 0;
    S->final_cost = cost;
    S->num_iterations = S->num_successful_steps + S->num_unsuccessful_steps;
    if (S->usable) {
      std::copy(b.ext.begin(), b.ext.end(), P->extrinsics);
      std::copy(b.intr.begin(), b.intr.end(), P->intrinsics);
      std::copy(b.pts.begin(), b.pts.end(), P->points);
    }
    S->total_time_s = Now() - t0;
    return (int)GBBA_SUCCESS;
  };
  if (grad_max <= o->gradient_tolerance) return finish(GBBA_CONVERGENCE);

  // Jacobi scaling, computed once from the initial Jacobian (trust_region_minimizer.cc:238-243).
  {
    std::vector<double> cn, pn;
    b.scale_c.assign(b.n_red, 1.0); b.scale_p.assign(3 * b.np, 1.0);
    if (o->jacobi_scaling) {
      ColumnNorms(b, cn, pn, false);
      for (int64_t i = 0; i < b.n_red; ++i) b.scale_c[i] = 1.0 / (1.0 + std::sqrt(cn[i]));
      for (int64_t i = 0; i < 3 * b.np; ++i) b.scale_p[i] = 1.0 / (1.0 + std::sqrt(pn[i]));
    }
    ScaleJacobian(b);
  }

  double radius = o->initial_trust_region_radius, decrease_factor = 2.0;
  bool reuse_diagonal = false;
  std::vector<double> diag_c, diag_p;
  int invalid_steps = 0, iteration = 0;
  double x_norm = XNorm(b);
  std::vector<double> step_c, step_p, dc, dp, E2, K2, X2;
  while (true) {
    if (iteration >= o->max_num_iterations) return finish(GBBA_NO_CONVERGENCE);
    const double ts = Now();
    // LevenbergMarquardtStrategy::ComputeStep
    if (!reuse_diagonal) {
      ColumnNorms(b, diag_c, diag_p, false);  // the stored J is already scaled
      for (double& v : diag_c) v = std::min(std::max(v, o->min_lm_diagonal), o->max_lm_diagonal);
      for (double& v : diag_p) v = std::min(std::max(v, o->min_lm_diagonal), o->max_lm_diagonal);
    }
    std::vector<double> Dc2(b.n_red), Dp2(3 * b.np);
    for (int64_t i = 0; i < b.n_red; ++i) { const double d = std::sqrt(diag_c[i] / radius); Dc2[i] = d * d; }
    for (int64_t i = 0; i < 3 * b.np; ++i) { const double d = std::sqrt(diag_p[i] / radius); Dp2[i] = d * d; }
    const bool solved = SchurSolve(b, Dc2, Dp2, step_c, step_p);
    reuse_diagonal = true;
    S->linear_solver_time_s += Now() - ts;
    ++iteration;
    double model_cost_change = 0.0;
    bool valid = false;
    if (solved) {
      // model_cost_change = -m'(r + m/2), m = J step  (trust_region_minimizer.cc:336-345)
      double mcc = 0.0;
#pragma omp parallel for reduction(+ : mcc) schedule(static)
      for (int64_t i = 0; i < b.no; ++i) {
        const double* J = &b.J[(size_t)i * 2 * b.nb];
        double m[2] = {0, 0};
        for (int c = 0; c < 6 + b.k; ++c) { const int64_t col = CamCol(b, i, c); if (col < 0) continue; m[0] += J[c] * step_c[col]; m[1] += J[b.nb + c] * step_c[col]; }
        const int64_t p = b.P->point_index[i];
        for (int c = 0; c < 3; ++c) { m[0] += J[6 + b.k + c] * step_p[3 * p + c]; m[1] += J[b.nb + 6 + b.k + c] * step_p[3 * p + c]; }
        mcc += -(m[0] * (b.rc[2 * i] + m[0] / 2.0) + m[1] * (b.rc[2 * i + 1] + m[1] / 2.0));
      }
      model_cost_change = mcc;
      valid = model_cost_change >= 0.0;
    }
    bool success = false;
    double relative_decrease = 0.0;
    if (!valid) {
      if (++invalid_steps >= o->max_num_consecutive_invalid_steps) return finish(GBBA_FAILURE);
    } else {
      invalid_steps = 0;
      dc.resize(b.n_red); dp.resize(3 * b.np);
      for (int64_t i = 0; i < b.n_red; ++i) dc[i] = step_c[i] * b.scale_c[i];
      for (int64_t i = 0; i < 3 * b.np; ++i) dp[i] = step_p[i] * b.scale_p[i];
      Plus(b, dc, dp, E2, K2, X2);
      double new_cost;
      const double tr = Now();
      if (!Evaluate(b, E2.data(), K2.data(), X2.data(), &new_cost, false)) new_cost = std::numeric_limits<double>::max();
      S->residual_time_s += Now() - tr;
      double step_norm2 = 0.0;
      for (double v : dc) step_norm2 += v * v;
      for (double v : dp) step_norm2 += v * v;
      if (std::sqrt(step_norm2) <= o->parameter_tolerance * (x_norm + o->parameter_tolerance))
        return finish(GBBA_CONVERGENCE);
      const double cost_change = cost - new_cost;
      if (std::fabs(cost_change) <= o->function_tolerance * cost) return finish(GBBA_CONVERGENCE);
      relative_decrease = cost_change / model_cost_change;
      success = relative_decrease > o->min_relative_decrease;
    }
    if (success) {
      ++S->num_successful_steps;
      radius = radius / std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * relative_decrease - 1.0, 3));
      radius = std::min(o->max_trust_region_radius, radius);
      decrease_factor = 2.0;
      reuse_diagonal = false;
      b.ext = E2; b.intr = K2; b.pts = X2;
      x_norm = XNorm(b);
      const double tj = Now();
      if (!Evaluate(b, b.ext.data(), b.intr.data(), b.pts.data(), &cost, true)) return finish(GBBA_FAILURE);
      grad_max = GradientMaxNorm(b);
      ScaleJacobian(b);
      S->jacobian_time_s += Now() - tj;
    } else {
      ++S->num_unsuccessful_steps;
      if (valid) { radius = radius / decrease_factor; decrease_factor *= 2.0; reuse_diagonal = true; }
      else { radius = radius / decrease_factor; decrease_factor *= 2.0; reuse_diagonal = true; }  // StepIsInvalid == StepRejected(0)
    }
    push_cost(cost);
    if (success) {
      if (grad_max <= o->gradient_tolerance) return finish(GBBA_CONVERGENCE);
    } else if (radius < o->min_trust_region_radius) {
      return finish(GBBA_CONVERGENCE);
    }
  }
}

// Restatement of ceres::Problem::Evaluate on the problem (no constant blocks):
// cost, raw residuals [no][2], corrected Jacobian blocks, gradient laid out as
// [extrinsics | intrinsics | points].
int oracle_ba_evaluate(const gbba_problem* P, int loss_type, double loss_scale, double* cost,
                       double* residuals, double* jac_e, double* jac_i, double* jac_p, double* gradient) {
  const int model = P->camera_model, k = ModelK(model), nb = 6 + k + 3;
  Loss loss; loss.type = loss_type; loss.a = loss_scale; loss.b = loss_scale * loss_scale;
  EvalFn f = PickEval(model);
  const int64_t nc = P->num_cameras, ni = P->num_intrinsics, no = P->num_observations;
  double total = 0.0;
  if (gradient) std::memset(gradient, 0, sizeof(double) * (6 * nc + k * ni + 3 * P->num_points));
  std::vector<double> J(2 * nb);
  for (int64_t i = 0; i < no; ++i) {
    double c, rr[2], rc[2];
    const double* e = P->extrinsics + 6 * (int64_t)P->camera_index[i];
    const double* kk = P->intrinsics + k * (int64_t)P->intrinsic_index[i];
    const double* x = P->points + 3 * (int64_t)P->point_index[i];
    f(model, kk, e, x, P->observations + 2 * i, loss, &c, rr, rc, J.data());
    total += c;
    if (residuals) { residuals[2 * i] = rr[0]; residuals[2 * i + 1] = rr[1]; }
    for (int row = 0; row < 2; ++row) {
      for (int j = 0; j < 6; ++j) if (jac_e) jac_e[(i * 2 + row) * 6 + j] = J[row * nb + j];
      for (int j = 0; j < k; ++j) if (jac_i) jac_i[(i * 2 + row) * k + j] = J[row * nb + 6 + j];
      for (int j = 0; j < 3; ++j) if (jac_p) jac_p[(i * 2 + row) * 3 + j] = J[row * nb + 6 + k + j];
    }
    if (gradient) {
      double* ge = gradient + 6 * (int64_t)P->camera_index[i];
      double* gi = gradient + 6 * nc + k * (int64_t)P->intrinsic_index[i];
      double* gx = gradient + 6 * nc + k * ni + 3 * (int64_t)P->point_index[i];
      for (int j = 0; j < 6; ++j) ge[j] += J[j] * rc[0] + J[nb + j] * rc[1];
      for (int j = 0; j < k; ++j) gi[j] += J[6 + j] * rc[0] + J[nb + 6 + j] * rc[1];
      for (int j = 0; j < 3; ++j) gx[j] += J[6 + k + j] * rc[0] + J[nb + 6 + k + j] * rc[1];
    }
  }
  if (cost) *cost = total;
  return 0;
}

}  // extern "C"

// ====================================================================== triangulation
namespace {

// Smallest right singular vector of A (m x n, row-major) by one-sided
// (Hestenes) Jacobi; the reference uses Eigen::JacobiSVD with ComputeFullV
// and takes V's last column (numeric.h:228-240).  Returns the smallest singular value.
double NullspaceJacobi(const double* A, int m, int n, double* x) {
  std::vector<double> U(A, A + (size_t)m * n), V((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int i = 0; i < n - 1; ++i)
      for (int j = i + 1; j < n; ++j) {
        double a = 0, bb = 0, g = 0;
        for (int r = 0; r < m; ++r) { const double ui = U[(size_t)r * n + i], uj = U[(size_t)r * n + j]; a += ui * ui; bb += uj * uj; g += ui * uj; }
        if (g == 0.0 || std::fabs(g) <= 1e-15 * std::sqrt(a * bb)) continue;
        rotated = true;
        const double zeta = (bb - a) / (2.0 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int r = 0; r < m; ++r) { double& ui = U[(size_t)r * n + i]; double& uj = U[(size_t)r * n + j]; const double vi = ui, vj = uj; ui = c * vi - s * vj; uj = s * vi + c * vj; }
        for (int r = 0; r < n; ++r) { double& vi_ = V[(size_t)r * n + i]; double& vj_ = V[(size_t)r * n + j]; const double vi = vi_, vj = vj_; vi_ = c * vi - s * vj; vj_ = s * vi + c * vj; }
      }
    if (!rotated) break;
  }
  int best = 0;
  double bestn = std::numeric_limits<double>::max();
  for (int i = 0; i < n; ++i) {
    double s = 0;
    for (int r = 0; r < m; ++r) s += U[(size_t)r * n + i] * U[(size_t)r * n + i];
    if (s < bestn) { bestn = s; best = i; }
  }
  for (int r = 0; r < n; ++r) x[r] = V[(size_t)r * n + best];
  return std::sqrt(bestn);
}

void Project(const double* P, const double* X3, double* x) {
  double h[3];
  for (int r = 0; r < 3; ++r) h[r] = P[4 * r] * X3[0] + P[4 * r + 1] * X3[1] + P[4 * r + 2] * X3[2] + P[4 * r + 3];
  x[0] = h[0] / h[2]; x[1] = h[1] / h[2];
}

bool Inverse3General(const double A[9], double Ai[9]) {
  const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  if (!(std::fabs(det) > 0) || !std::isfinite(det)) return false;
  const double id = 1.0 / det;
  Ai[0] = c00 * id; Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id; Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = c01 * id; Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id; Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = c02 * id; Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id; Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  return true;
}

}  // namespace

extern "C" {

int oracle_tri_dlt2(int64_t n, const double* P1, const double* P2, int64_t p_stride,
                    const double* x1, const double* x2, double* Xh, double* Xe) {
  for (int64_t t = 0; t < n; ++t) {
    const double* A = P1 + t * p_stride;
    const double* B = P2 + t * p_stride;
    double D[16], X[4];
    for (int i = 0; i < 4; ++i) {
      D[0 * 4 + i] = x1[2 * t] * A[8 + i] - A[i];
      D[1 * 4 + i] = x1[2 * t + 1] * A[8 + i] - A[4 + i];
      D[2 * 4 + i] = x2[2 * t] * B[8 + i] - B[i];
      D[3 * 4 + i] = x2[2 * t + 1] * B[8 + i] - B[4 + i];
    }
    NullspaceJacobi(D, 4, 4, X);
    if (Xh) for (int i = 0; i < 4; ++i) Xh[4 * t + i] = X[i];
    if (Xe) for (int i = 0; i < 3; ++i) Xe[3 * t + i] = X[i] / X[3];
  }
  return 0;
}

int oracle_tri_nview(int method, const double* P, int64_t num_cameras, const int64_t* offs,
                     const uint32_t* cam, const double* xy, int64_t num_tracks, double* X, double* err) {
  (void)num_cameras;
  for (int64_t t = 0; t < num_tracks; ++t) {
    const int64_t b = offs[t];
    const int n = (int)(offs[t + 1] - b);
    if (method == 0) {  // TriangulateNView: [-P_i | x~_i e_i]
      const int m = 3 * n, nc = 4 + n;
      std::vector<double> D((size_t)m * nc, 0.0), v(nc);
      for (int i = 0; i < n; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        for (int r = 0; r < 3; ++r) for (int c = 0; c < 4; ++c) D[(size_t)(3 * i + r) * nc + c] = -Pi[4 * r + c];
        D[(size_t)(3 * i + 0) * nc + 4 + i] = xy[2 * (b + i)];
        D[(size_t)(3 * i + 1) * nc + 4 + i] = xy[2 * (b + i) + 1];
        D[(size_t)(3 * i + 2) * nc + 4 + i] = 1.0;
      }
      NullspaceJacobi(D.data(), m, nc, v.data());
      for (int i = 0; i < 4; ++i) X[4 * t + i] = v[i];
    } else if (method == 1) {  // algebraic: rows [0,-1,y]P and [1,0,-x]P
      std::vector<double> D((size_t)2 * n * 4);
      for (int i = 0; i < n; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        const double x = xy[2 * (b + i)], y = xy[2 * (b + i) + 1];
        for (int c = 0; c < 4; ++c) {
          D[(size_t)(2 * i) * 4 + c] = -Pi[4 + c] + y * Pi[8 + c];
          D[(size_t)(2 * i + 1) * 4 + c] = Pi[c] - x * Pi[8 + c];
        }
      }
      double v[4];
      NullspaceJacobi(D.data(), 2 * n, 4, v);
      for (int i = 0; i < 4; ++i) X[4 * t + i] = v[i];
    } else {  // Triangulation::compute(3) + error()
      std::vector<double> w(n, 1.0);
      double Xc[3] = {0, 0, 0};
      for (int it = 0; it < 3; ++it) {
        double AtA[9] = {0}, Atb[3] = {0};
        for (int i = 0; i < n; ++i) {
          const double* Pi = P + 12 * (int64_t)cam[b + i];
          const double px = xy[2 * (b + i)], py = xy[2 * (b + i) + 1], wi = w[i];
          double v1[3], v2[3];
          for (int j = 0; j < 3; ++j) {
            v1[j] = wi * (Pi[j] - px * Pi[8 + j]);
            v2[j] = wi * (Pi[4 + j] - py * Pi[8 + j]);
            Atb[j] += wi * (v1[j] * (px * Pi[11] - Pi[3]) + v2[j] * (py * Pi[11] - Pi[7]));
          }
          for (int kk = 0; kk < 3; ++kk)
            for (int j = 0; j <= kk; ++j) {
              const double v = v1[j] * v1[kk] + v2[j] * v2[kk];
              AtA[3 * j + kk] += v;
              if (j < kk) AtA[3 * kk + j] += v;
            }
        }
        double Ai[9];
        Inverse3General(AtA, Ai);
        for (int r = 0; r < 3; ++r) Xc[r] = Ai[3 * r] * Atb[0] + Ai[3 * r + 1] * Atb[1] + Ai[3 * r + 2] * Atb[2];
        for (int i = 0; i < n; ++i) {
          const double* Pi = P + 12 * (int64_t)cam[b + i];
          const double z = Pi[8] * Xc[0] + Pi[9] * Xc[1] + Pi[10] * Xc[2] + Pi[11];
          w[i] = 1.0 / z;
        }
      }
      for (int r = 0; r < 3; ++r) X[3 * t + r] = Xc[r];
      if (err) {
        double e = 0;
        for (int i = 0; i < n; ++i) {
          double x[2];
          Project(P + 12 * (int64_t)cam[b + i], Xc, x);
          const double dx = xy[2 * (b + i)] - x[0], dy = xy[2 * (b + i) + 1] - x[1];
          e += std::sqrt(dx * dx + dy * dy);
        }
        err[t] = e;
      }
    }
  }
  return 0;
}

// FP64 twin of the FP32 production triangulation (gbtri_nview_batched_f32):
// unit-weight linear solve of the reference's 3x3 system, then `gn_steps`
// Gauss-Newton steps on the reprojection error; status / min depth as there.
int oracle_tri_linear_gn(const double* P, const int64_t* offs, const uint32_t* cam, const double* xy,
                         int64_t num_tracks, int gn_steps, double* X, uint8_t* status, double* min_depth) {
  for (int64_t t = 0; t < num_tracks; ++t) {
    const int64_t b = offs[t];
    const int n = (int)(offs[t + 1] - b);
    double Xc[3] = {0, 0, 0};
    uint8_t st = GBTRI_TRACK_OK;
    if (n < 2) st = GBTRI_TRACK_DEGENERATE;
    if (st == GBTRI_TRACK_OK) {
      double AtA[9] = {0}, Atb[3] = {0};
      for (int i = 0; i < n; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        const double px = xy[2 * (b + i)], py = xy[2 * (b + i) + 1];
        double v1[3], v2[3];
        for (int j = 0; j < 3; ++j) { v1[j] = Pi[j] - px * Pi[8 + j]; v2[j] = Pi[4 + j] - py * Pi[8 + j]; }
        const double b1 = px * Pi[11] - Pi[3], b2 = py * Pi[11] - Pi[7];
        for (int j = 0; j < 3; ++j) {
          Atb[j] += v1[j] * b1 + v2[j] * b2;
          for (int kk = 0; kk < 3; ++kk) AtA[3 * j + kk] += v1[j] * v1[kk] + v2[j] * v2[kk];
        }
      }
      double Ai[9];
      if (!Inverse3General(AtA, Ai)) st = GBTRI_TRACK_DEGENERATE;
      else for (int r = 0; r < 3; ++r) Xc[r] = Ai[3 * r] * Atb[0] + Ai[3 * r + 1] * Atb[1] + Ai[3 * r + 2] * Atb[2];
    }
    for (int s = 0; s < gn_steps && st == GBTRI_TRACK_OK; ++s) {
      double H[9] = {0}, g[3] = {0};
      for (int i = 0; i < n; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        double h[3];
        for (int r = 0; r < 3; ++r) h[r] = Pi[4 * r] * Xc[0] + Pi[4 * r + 1] * Xc[1] + Pi[4 * r + 2] * Xc[2] + Pi[4 * r + 3];
        const double iz = 1.0 / h[2];
        const double u = h[0] * iz, v = h[1] * iz;
        const double ru = u - xy[2 * (b + i)], rv = v - xy[2 * (b + i) + 1];
        double Ju[3], Jv[3];
        for (int j = 0; j < 3; ++j) { Ju[j] = (Pi[j] - u * Pi[8 + j]) * iz; Jv[j] = (Pi[4 + j] - v * Pi[8 + j]) * iz; }
        for (int j = 0; j < 3; ++j) {
          g[j] += Ju[j] * ru + Jv[j] * rv;
          for (int kk = 0; kk < 3; ++kk) H[3 * j + kk] += Ju[j] * Ju[kk] + Jv[j] * Jv[kk];
        }
      }
      double Hi[9];
      if (!Inverse3General(H, Hi)) { st = GBTRI_TRACK_DEGENERATE; break; }
      for (int r = 0; r < 3; ++r) Xc[r] -= Hi[3 * r] * g[0] + Hi[3 * r + 1] * g[1] + Hi[3 * r + 2] * g[2];
    }
    double md = std::numeric_limits<double>::max();
    for (int i = 0; i < n; ++i) {
      const double* Pi = P + 12 * (int64_t)cam[b + i];
      md = std::min(md, Pi[8] * Xc[0] + Pi[9] * Xc[1] + Pi[10] * Xc[2] + Pi[11]);
    }
    if (st == GBTRI_TRACK_OK && !(md > 0)) st = GBTRI_TRACK_BEHIND_CAMERA;
    for (int r = 0; r < 3; ++r) X[3 * t + r] = Xc[r];
    if (status) status[t] = st;
    if (min_depth) min_depth[t] = n > 0 ? md : 0.0;
  }
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------- engine BA assembly

// ceres::RotationMatrixToQuaternion (Shoemake, rotation.h:312-350) and
// QuaternionToAngleAxis (:266-306) on a column-major matrix, as the engine
// passes Eigen's Mat3::data().
static void oracle_rotation_to_angle_axis(const double* Rc, double* aa) {
  auto R = [&](int i, int j) { return Rc[3 * j + i]; };
  double q[4];
  const double trace = R(0, 0) + R(1, 1) + R(2, 2);
  if (trace >= 0.0) {
    double t = std::sqrt(trace + 1.0);
    q[0] = 0.5 * t;
    t = 0.5 / t;
    q[1] = (R(2, 1) - R(1, 2)) * t;
    q[2] = (R(0, 2) - R(2, 0)) * t;
    q[3] = (R(1, 0) - R(0, 1)) * t;
  } else {
    int i = R(1, 1) > R(0, 0) ? 1 : 0;
    if (R(2, 2) > R(i, i)) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double t = std::sqrt(R(i, i) - R(j, j) - R(k, k) + 1.0);
    q[i + 1] = 0.5 * t;
    t = 0.5 / t;
    q[0] = (R(k, j) - R(j, k)) * t;
    q[j + 1] = (R(j, i) + R(i, j)) * t;
    q[k + 1] = (R(k, i) + R(i, k)) * t;
  }
  const double s2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  double kk = 2.0;
  if (s2 > 0.0) {
    const double st = std::sqrt(s2), ct = q[0];
    kk = 2.0 * (ct < 0.0 ? std::atan2(-st, -ct) : std::atan2(st, ct)) / st;
  }
  for (int a = 0; a < 3; ++a) aa[a] = q[a + 1] * kk;
}

struct OracleEngineCamera {
  double R[9];  // column-major, as Eigen stores rotation_matrix_
  double t[3];
};

extern "C" {

// The engine's maps are built from the dense state (not timed); then the
// assembly loop of BundleAdjustment runs `repeats` times over them and its
// mean wall time goes to *seconds.  The last run's problem is written in the
// gbsfm_ba_arrays layout; counts[0..2] = cameras, observations, locked block.
int oracle_sfm_pack_maps(const gbsfm_engine_state* st, int64_t first_added, double* ext, double* intr, double* pts,
                         double* obs, uint32_t* cam_idx, uint32_t* intr_idx, uint32_t* pt_idx, int64_t* counts,
                         int repeats, double* seconds) {
  std::map<size_t, OracleEngineCamera> map_Camera;
  std::map<size_t, std::vector<std::pair<float, float> > > map_features;
  std::map<size_t, std::vector<size_t> > map_images_id_per_intrinsic_group;
  std::map<size_t, std::vector<double> > map_intrinsics_per_group;
  std::map<size_t, std::vector<double> > map_3d_points;
  std::map<size_t, std::map<size_t, size_t> > map_reconstructed;
  for (int64_t g = 0; g < st->num_intrinsic_groups; ++g)
    map_intrinsics_per_group[(size_t)g] = std::vector<double>(st->group_intrinsics + 6 * g,
                                                               st->group_intrinsics + 6 * g + 6);
  for (int64_t i = 0; i < st->num_images; ++i) {
    map_images_id_per_intrinsic_group[st->intrinsic_group[i]].push_back((size_t)i);
    std::vector<std::pair<float, float> >& f = map_features[(size_t)i];
    for (int64_t k = st->feature_offsets[i]; k < st->feature_offsets[i + 1]; ++k)
      f.push_back(std::make_pair(st->features[2 * k], st->features[2 * k + 1]));
    if (!st->reconstructed[i]) continue;
    const gbsfm_camera& c = st->cameras[i];
    OracleEngineCamera e;
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) e.R[3 * k + r] = c.R[3 * r + k];
    for (int r = 0; r < 3; ++r) e.t[r] = c.t[r];
    map_Camera[(size_t)i] = e;
  }
  for (int64_t t = 0; t < st->num_points; ++t) {
    map_3d_points[(size_t)t] = std::vector<double>(st->points + 3 * t, st->points + 3 * t + 3);
    std::map<size_t, size_t>& tr = map_reconstructed[(size_t)t];
    for (int64_t e = st->track_offsets[t]; e < st->track_offsets[t + 1]; ++e)
      tr[st->track_image[e]] = st->track_feature[e];
  }

  std::vector<double> parameters, observations;
  std::vector<size_t> point_index, cam_ext, cam_intr;
  size_t num_cameras = 0, num_intrinsic = 0;
  int64_t locked = -1;
  const auto t0 = std::chrono::steady_clock::now();
  for (int rep = 0; rep < std::max(1, repeats); ++rep) {
    parameters.clear();
    observations.clear();
    point_index.clear();
    cam_ext.clear();
    cam_intr.clear();
    num_cameras = map_Camera.size();
    num_intrinsic = map_images_id_per_intrinsic_group.size();
    size_t measurements = 0;
    for (auto it = map_3d_points.begin(); it != map_3d_points.end(); ++it)
      measurements += map_reconstructed[it->first].size();
    point_index.reserve(measurements);
    cam_ext.reserve(measurements);
    cam_intr.reserve(measurements);
    observations.reserve(2 * measurements);
    parameters.reserve(6 * num_cameras + 6 * num_intrinsic + 3 * map_3d_points.size());
    std::set<size_t> set_camIndex;
    std::map<size_t, size_t> ext_number, intr_number;
    size_t cpt = 0;
    for (auto it = map_Camera.begin(); it != map_Camera.end(); ++it, ++cpt) {
      set_camIndex.insert(it->first);
      ext_number.insert(std::make_pair(it->first, cpt));
      double aa[3];
      oracle_rotation_to_angle_axis(it->second.R, aa);
      for (int a = 0; a < 3; ++a) parameters.push_back(aa[a]);
      for (int a = 0; a < 3; ++a) parameters.push_back(it->second.t[a]);
    }
    for (auto it = map_intrinsics_per_group.begin(); it != map_intrinsics_per_group.end(); ++it)
      for (int j = 0; j < 6; ++j) parameters.push_back(it->second[j]);
    cpt = 0;
    for (auto it = map_images_id_per_intrinsic_group.begin(); it != map_images_id_per_intrinsic_group.end();
         ++it, ++cpt)
      for (size_t k = 0; k < it->second.size(); ++k) intr_number.insert(std::make_pair(it->second[k], cpt));
    for (auto it = map_3d_points.begin(); it != map_3d_points.end(); ++it)
      for (int j = 0; j < 3; ++j) parameters.push_back(it->second[j]);
    cpt = 0;
    for (auto it = map_3d_points.begin(); it != map_3d_points.end(); ++it, ++cpt) {
      const std::map<size_t, size_t>& tr = map_reconstructed[it->first];
      for (auto e = tr.begin(); e != tr.end(); ++e) {
        if (set_camIndex.find(e->first) == set_camIndex.end()) continue;
        const std::pair<float, float>& f = map_features[e->first][e->second];
        observations.push_back(f.first);
        observations.push_back(f.second);
        point_index.push_back(cpt);
        cam_ext.push_back(ext_number[e->first]);
        cam_intr.push_back(intr_number[e->first]);
      }
    }
    locked = -1;
    if (first_added >= 0 && !ext_number.empty()) {
      const size_t k = ext_number[(size_t)first_added];
      if (k < cam_ext.size()) locked = (int64_t)cam_ext[k];
    }
  }
  *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / std::max(1, repeats);
  const size_t nc = num_cameras, ng = num_intrinsic;
  if (ext) std::memcpy(ext, parameters.data(), sizeof(double) * 6 * nc);
  if (intr) std::memcpy(intr, parameters.data() + 6 * nc, sizeof(double) * 6 * ng);
  if (pts) std::memcpy(pts, parameters.data() + 6 * (nc + ng), sizeof(double) * 3 * st->num_points);
  if (obs) std::memcpy(obs, observations.data(), sizeof(double) * observations.size());
  for (size_t o = 0; o < point_index.size(); ++o) {
    if (cam_idx) cam_idx[o] = (uint32_t)cam_ext[o];
    if (intr_idx) intr_idx[o] = (uint32_t)cam_intr[o];
    if (pt_idx) pt_idx[o] = (uint32_t)point_index[o];
  }
  counts[0] = (int64_t)nc;
  counts[1] = (int64_t)point_index.size();
  counts[2] = locked;
  return 0;
}


// AC-RANSAC scoring of a batch of models as the reference's main loop does
// it, model after model (estimator_acransac.h:170-200): residuals
// (ResectionSquaredResidualError, sfm_robust.h:197-204), std::sort of
// (error, index) pairs, bestNFA (:75-97) with the float logcombi tables
// (:40-65).  Returns the mean seconds per model in *seconds.
static double oracle_logcombi(size_t k, size_t n) {
  if (k >= n || k <= 0) return 0.0;
  if (n - k < k) k = n - k;
  double r = 0.0;
  for (size_t i = 1; i <= k; i++) r += std::log10((double)(n - i + 1)) - std::log10((double)i);
  return r;
}

int oracle_acransac_score(int sample_size, int max_models, double logalpha0, double mult_error, double max_threshold,
                          int64_t n, const double* x2d, const double* x3d, int64_t num_models, const double* models,
                          double* nfa, int32_t* num_inliers, double* error_max, uint32_t* order, double* seconds) {
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<float> logc_n(n + 1), logc_k(n + 1);
  for (int64_t k = 0; k <= n; ++k) logc_n[k] = (float)oracle_logcombi((size_t)k, (size_t)n);
  for (int64_t m = 0; m <= n; ++m) logc_k[m] = (float)oracle_logcombi((size_t)sample_size, (size_t)m);
  const double loge0 = std::log10((double)max_models * (double)(n - sample_size));
  std::vector<std::pair<double, size_t> > e((size_t)n);
  for (int64_t h = 0; h < num_models; ++h) {
    const double* P = models + 12 * h;
    for (int64_t i = 0; i < n; ++i) {
      const double* X = x3d + 3 * i;
      double hx[3];
      for (int r = 0; r < 3; ++r) hx[r] = P[4 * r] * X[0] + P[4 * r + 1] * X[1] + P[4 * r + 2] * X[2] + P[4 * r + 3];
      const double dx = hx[0] / hx[2] - x2d[2 * i], dy = hx[1] / hx[2] - x2d[2 * i + 1];
      e[(size_t)i] = std::make_pair(dx * dx + dy * dy, (size_t)i);
    }
    std::sort(e.begin(), e.end());
    double best = std::numeric_limits<double>::infinity();
    int64_t best_k = sample_size;
    for (int64_t k = sample_size + 1; k <= n && e[k - 1].first <= max_threshold; ++k) {
      const double logalpha = logalpha0 + mult_error * std::log10(e[k - 1].first + std::numeric_limits<float>::min());
      const double v = loge0 + logalpha * (double)(k - sample_size) + logc_n[k] + logc_k[k];
      if (v < best) {
        best = v;
        best_k = k;
      }
    }
    nfa[h] = best;
    num_inliers[h] = (int32_t)best_k;
    error_max[h] = best_k > sample_size ? e[best_k - 1].first : std::numeric_limits<double>::infinity();
    if (order)
      for (int64_t i = 0; i < n; ++i) order[h * n + i] = (uint32_t)e[(size_t)i].second;
  }
  *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() /
             (double)std::max<int64_t>(1, num_models);
  return 0;
}

}  // extern "C"
