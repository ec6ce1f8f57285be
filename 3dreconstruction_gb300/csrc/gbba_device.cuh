// Device math of the reprojection residual and its hand-written Jacobian.
//
// Forward:  p = R(w) X + t  (ceres::AngleAxisRotatePoint, 3rdparty/ceres/
//           include/ceres/rotation.h:566-625, including its first-order branch
//           for theta^2 <= DBL_EPSILON), x = p0/p2, y = p1/p2, then the camera
//           model of libs/sfm/include/mvg/sfm/pinhole_ceres_functor.h:24-54 or
//           libs/camera/include/mvg/camera/brown_pinhole_camera.h:15-41 (+ the
//           commented-out tangential terms of :35-36 for BROWN_T2).
// Adjoint:  the chain  dr/d(x,y) . d(x,y)/dp . [dp/dw | I | R]  written out by
//           hand; it replaces ceres AutoDiff (include/ceres/autodiff_cost_
//           function.h:202-211) and is recomputed from the parameters on every
//           use, nothing is stored between kernels.
// Loss:     ceres::HuberLoss (internal/ceres/loss_function.cc:47-61) through
//           the Corrector (internal/ceres/corrector.cc:41-155): for Huber
//           rho'' <= 0, so residual and Jacobian are both scaled by sqrt(rho').
#pragma once
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace gbba {

enum { kPinholeF = 0, kRadialK3 = 1, kBrownT2 = 2 };

template <int M> struct Model;
template <> struct Model<kPinholeF> { static constexpr int K = 1; };
template <> struct Model<kRadialK3> { static constexpr int K = 6; };
template <> struct Model<kBrownT2> { static constexpr int K = 8; };

template <typename T> __device__ __forceinline__ T dsqrt(T x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }

template <typename T> __device__ __forceinline__ void dsincos(T x, T* s, T* c);
template <> __device__ __forceinline__ void dsincos<double>(double x, double* s, double* c) { sincos(x, s, c); }
template <> __device__ __forceinline__ void dsincos<float>(float x, float* s, float* c) { sincosf(x, s, c); }

// p = R(w) X  with R, and dp/dw when kJac.
template <typename T, bool kJac>
__device__ __forceinline__ void rotate(const T w[3], const T X[3], T p[3], T R[3][3], T dpdw[3][3]) {
  const T th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (th2 > T(DBL_EPSILON)) {
    const T th = dsqrt(th2);
    T s, c;
    dsincos(th, &s, &c);
    const T ith = T(1) / th;
    const T u[3] = {w[0] * ith, w[1] * ith, w[2] * ith};
    const T uxX[3] = {u[1] * X[2] - u[2] * X[1], u[2] * X[0] - u[0] * X[2], u[0] * X[1] - u[1] * X[0]};
    const T udX = u[0] * X[0] + u[1] * X[1] + u[2] * X[2];
    const T omc = T(1) - c;
    const T tmp = udX * omc;
#pragma unroll
    for (int i = 0; i < 3; ++i) p[i] = X[i] * c + uxX[i] * s + u[i] * tmp;
    if (kJac) {
      // R = c I + s [u]x + (1-c) u u^T
      R[0][0] = c + omc * u[0] * u[0];       R[0][1] = -s * u[2] + omc * u[0] * u[1]; R[0][2] = s * u[1] + omc * u[0] * u[2];
      R[1][0] = s * u[2] + omc * u[1] * u[0]; R[1][1] = c + omc * u[1] * u[1];       R[1][2] = -s * u[0] + omc * u[1] * u[2];
      R[2][0] = -s * u[1] + omc * u[2] * u[0]; R[2][1] = s * u[0] + omc * u[2] * u[1]; R[2][2] = c + omc * u[2] * u[2];
      // d/dw_k with dtheta/dw_k = u_k and du_i/dw_k = (delta_ik - u_i u_k)/theta
      const T eX[3][3] = {{T(0), X[2], -X[1]}, {-X[2], T(0), X[0]}, {X[1], -X[0], T(0)}};  // column k = e_k x X
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T duX = ith * (X[k] - u[k] * udX);  // (du/dw_k) . X
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const T du_ik = ith * ((i == k ? T(1) : T(0)) - u[i] * u[k]);
          const T dcross = ith * (eX[i][k] - u[k] * uxX[i]);  // ((du/dw_k) x X)_i
          dpdw[i][k] = -s * u[k] * X[i] + dcross * s + uxX[i] * c * u[k] + du_ik * tmp + u[i] * omc * duX +
                       u[i] * udX * s * u[k];
        }
      }
    }
  } else {
    // first-order branch: R p = p + w x p
    p[0] = X[0] + (w[1] * X[2] - w[2] * X[1]);
    p[1] = X[1] + (w[2] * X[0] - w[0] * X[2]);
    p[2] = X[2] + (w[0] * X[1] - w[1] * X[0]);
    if (kJac) {
      R[0][0] = T(1);  R[0][1] = -w[2]; R[0][2] = w[1];
      R[1][0] = w[2];  R[1][1] = T(1);  R[1][2] = -w[0];
      R[2][0] = -w[1]; R[2][1] = w[0];  R[2][2] = T(1);
      dpdw[0][0] = T(0);  dpdw[0][1] = X[2];  dpdw[0][2] = -X[1];
      dpdw[1][0] = -X[2]; dpdw[1][1] = T(0);  dpdw[1][2] = X[0];
      dpdw[2][0] = X[1];  dpdw[2][1] = -X[0]; dpdw[2][2] = T(0);
    }
  }
}

// Camera model applied to the camera-frame point p: residual, and with kJac
// the intrinsic block Jk and D = d r / d p.
template <int M, typename T, bool kJac>
__device__ __forceinline__ void camera_residual(const T* __restrict__ Kp, const T p[3], T ox, T oy, T r[2],
                                                T Jk[2][Model<M>::K], T D[2][3]) {
  const T iz = T(1) / p[2];
  const T x = p[0] * iz, y = p[1] * iz;
  T A[2][2];  // d r / d(x, y)
  if (M == kPinholeF) {
    const T f = Kp[0];
    r[0] = f * x - ox;
    r[1] = f * y - oy;
    if (kJac) {
      A[0][0] = f; A[0][1] = T(0); A[1][0] = T(0); A[1][1] = f;
      Jk[0][0] = x;
      Jk[1][0] = y;
    }
  } else {
    const T f = Kp[0], k1 = Kp[3], k2 = Kp[4], k3 = Kp[5];
    const T r2 = x * x + y * y, r4 = r2 * r2, r6 = r4 * r2;
    const T rc = T(1) + k1 * r2 + k2 * r4 + k3 * r6;
    T xd = x * rc, yd = y * rc;
    T t1 = T(0), t2 = T(0);
    if (M == kBrownT2) {
      t1 = Kp[6];
      t2 = Kp[7];
      xd = xd + T(2) * t1 * x * y + t2 * (r2 + T(2) * x * x);
      yd = yd + T(2) * t2 * x * y + t1 * (r2 + T(2) * y * y);
    }
    r[0] = Kp[1] + f * xd - ox;
    r[1] = Kp[2] + f * yd - oy;
    if (kJac) {
      const T drc = k1 + T(2) * k2 * r2 + T(3) * k3 * r4;  // d rc / d r2
      T a00 = rc + T(2) * x * x * drc, a01 = T(2) * x * y * drc;
      T a10 = T(2) * x * y * drc, a11 = rc + T(2) * y * y * drc;
      if (M == kBrownT2) {
        a00 += T(2) * t1 * y + T(6) * t2 * x;
        a01 += T(2) * t1 * x + T(2) * t2 * y;
        a10 += T(2) * t2 * y + T(2) * t1 * x;
        a11 += T(2) * t2 * x + T(6) * t1 * y;
      }
      A[0][0] = f * a00; A[0][1] = f * a01; A[1][0] = f * a10; A[1][1] = f * a11;
      Jk[0][0] = xd;        Jk[1][0] = yd;
      Jk[0][1] = T(1);      Jk[1][1] = T(0);
      Jk[0][2] = T(0);      Jk[1][2] = T(1);
      Jk[0][3] = f * x * r2; Jk[1][3] = f * y * r2;
      Jk[0][4] = f * x * r4; Jk[1][4] = f * y * r4;
      Jk[0][5] = f * x * r6; Jk[1][5] = f * y * r6;
      if (M == kBrownT2) {
        Jk[0][6] = f * T(2) * x * y;           Jk[1][6] = f * (r2 + T(2) * y * y);
        Jk[0][7] = f * (r2 + T(2) * x * x);    Jk[1][7] = f * T(2) * x * y;
      }
    }
  }
  if (kJac) {
    // d r / d p = A . [[iz, 0, -x iz], [0, iz, -y iz]]
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      D[i][0] = A[i][0] * iz;
      D[i][1] = A[i][1] * iz;
      D[i][2] = -(A[i][0] * x + A[i][1] * y) * iz;
    }
  }
}

// Residual (and Jacobian blocks when kJac) of one observation.
//   Je [2][6]: d r / d(w, t);  Jk [2][K]: d r / d intrinsics;  Jx [2][3]: d r / d X
template <int M, typename T, bool kJac>
__device__ __forceinline__ void residual(const T* __restrict__ Kp, const T E[6], const T X[3], T ox, T oy,
                                         T r[2], T Je[2][6], T Jk[2][Model<M>::K], T Jx[2][3], T* depth) {
  T p[3], R[3][3], dpdw[3][3];
  rotate<T, kJac>(E, X, p, R, dpdw);
  p[0] += E[3];
  p[1] += E[4];
  p[2] += E[5];
  if (depth) *depth = p[2];
  T D[2][3];
  camera_residual<M, T, kJac>(Kp, p, ox, oy, r, Jk, D);
  if (kJac) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Je[i][k] = D[i][0] * dpdw[0][k] + D[i][1] * dpdw[1][k] + D[i][2] * dpdw[2][k];
        Je[i][3 + k] = D[i][k];
        Jx[i][k] = D[i][0] * R[0][k] + D[i][1] * R[1][k] + D[i][2] * R[2][k];
      }
    }
  }
}

// Camera pose as 12 values: R(w) row-major (the matrix form of the rotation
// that rotate() applies, with the same first-order branch) and t.
template <typename T>
__device__ __forceinline__ void pose_matrix(const T E[6], T pose[12]) {
  const T w[3] = {E[0], E[1], E[2]};
  const T th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (th2 > T(DBL_EPSILON)) {
    const T th = dsqrt(th2);
    T s, c;
    dsincos(th, &s, &c);
    const T ith = T(1) / th;
    const T u[3] = {w[0] * ith, w[1] * ith, w[2] * ith};
    const T omc = T(1) - c;
    pose[0] = c + omc * u[0] * u[0];        pose[1] = -s * u[2] + omc * u[0] * u[1]; pose[2] = s * u[1] + omc * u[0] * u[2];
    pose[3] = s * u[2] + omc * u[1] * u[0]; pose[4] = c + omc * u[1] * u[1];        pose[5] = -s * u[0] + omc * u[1] * u[2];
    pose[6] = -s * u[1] + omc * u[2] * u[0]; pose[7] = s * u[0] + omc * u[2] * u[1]; pose[8] = c + omc * u[2] * u[2];
  } else {
    pose[0] = T(1);  pose[1] = -w[2]; pose[2] = w[1];
    pose[3] = w[2];  pose[4] = T(1);  pose[5] = -w[0];
    pose[6] = -w[1]; pose[7] = w[0];  pose[8] = T(1);
  }
  pose[9] = E[3];
  pose[10] = E[4];
  pose[11] = E[5];
}

// Residual only, from a precomputed pose: p = R X + t.  Equal to residual()
// up to rounding (the rotation is applied as a matrix instead of through
// the Rodrigues terms), without a sine or cosine per observation.
template <int M, typename T>
__device__ __forceinline__ void residual_pose(const T* __restrict__ Kp, const T* __restrict__ pose, const T X[3], T ox,
                                              T oy, T r[2]) {
  T p[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) p[i] = pose[3 * i] * X[0] + pose[3 * i + 1] * X[1] + pose[3 * i + 2] * X[2] + pose[9 + i];
  T Jk[2][Model<M>::K], D[2][3];
  camera_residual<M, T, false>(Kp, p, ox, oy, r, Jk, D);
}

// Huber / squared loss: returns the cost 1/2 rho(s) and the Corrector scale sqrt(rho').
template <typename T>
__device__ __forceinline__ T robust(int loss_type, T a, T s, T* sqrt_rho1) {
  if (loss_type == 1 && s > a * a) {
    const T rs = dsqrt(s);
    T rho1 = a / rs;
    if (sizeof(T) == 8) rho1 = fmax((double)rho1, DBL_MIN);
    else rho1 = fmaxf((float)rho1, FLT_MIN);
    *sqrt_rho1 = dsqrt(rho1);
    return T(0.5) * (T(2) * a * rs - a * a);
  }
  *sqrt_rho1 = T(1);
  return T(0.5) * s;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- deterministic fixed-point sums of FP64 terms: a pass records the
// largest |term| of each sum (ordered bits under atomicMax), lin_exp picks a
// power-of-two scale for which n such terms stay below 2^62, and lin_fx
// rounds each scaled term to an integer (integer sums do not depend on the
// order of the adds).
// Scale exponent for a largest term m (ordered bits) and n terms: the sum's
// bound m n times 2^e stays within 2^62.  kNonFinite marks a column with a
// non-finite term.
constexpr int kFxNonFinite = 4000;
__device__ __forceinline__ int lin_exp(unsigned long long mbits, double n) {
  if (mbits == ~0ull) return kFxNonFinite;
  const double m = __longlong_as_double((long long)mbits);
  if (!(m > 0.0)) return 0;
  int e;
  frexp(m * n, &e);  // m n < 2^e
  return 62 - e;
}
// v 2^k rounded to an integer with integer operations (|v| 2^k < 2^62 by
// the choice of k); any rounding rule serves, the sum is exact.
__device__ __forceinline__ long long lin_fx(double v, int k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)(b >> 52) & 0x7ff;
  if (ex == 0 || ex == 0x7ff || k >= kFxNonFinite) return 0;
  const long long m = (long long)((b & 0xfffffffffffffull) | 0x10000000000000ull);
  const int sh = ex - 1075 + k;  // |v| 2^k = m 2^sh, m < 2^53, sh <= 9
  const int rs = min(max(-sh, 0), 63);
  const long long ml = m << max(min(sh, 9), 0);
  const long long r = rs ? (ml + (1ll << (rs - 1))) >> rs : ml;
  return (b >> 63) ? -r : r;
}
}  // namespace gbba
