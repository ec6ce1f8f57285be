// Batched triangulation (include/gbtri.h).
//
// FP64 parity paths restate the reference functions on the GPU:
//   TriangulateDLT      libs/multiview/src/triangulation.cpp:10-29
//   TriangulateNView    libs/multiview/src/triangulation_nview.cpp:8-24
//   ...Algebraic        libs/multiview/src/triangulation_nview.cpp:35-46
//   Triangulation::compute / error   :48-121
// The nullspace (libs/base/include/mvg/math/numeric.h:228-240 takes the last
// right singular vector of Eigen::JacobiSVD) is computed by one-sided
// (Hestenes) Jacobi: rotations orthogonalise the columns, V accumulates them,
// and the column of smallest norm gives the singular vector.
//
// FP32 production path: per track, the reference's linear system of
// Triangulation::compute with unit weights, then Gauss-Newton steps on the
// reprojection error; the block's observations are staged in shared memory
// with coalesced loads and the camera table lives in shared memory.
#include <cstring>

#include "gbba_internal.h"

namespace gbba {

// ---------------------------------------------------------------- FP64 DLT (4x4)
__device__ void jacobi_nullspace4(double A[4][4], double x[4]) {
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

__global__ void k_dlt2(int64_t n, const double* P1, const double* P2, int64_t ps, const double* x1, const double* x2,
                       double* Xh, double* Xe) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double* A = P1 + t * ps;
    const double* B = P2 + t * ps;
    double D[4][4], X[4];
    for (int i = 0; i < 4; ++i) {
      D[0][i] = x1[2 * t] * A[8 + i] - A[i];
      D[1][i] = x1[2 * t + 1] * A[8 + i] - A[4 + i];
      D[2][i] = x2[2 * t] * B[8 + i] - B[i];
      D[3][i] = x2[2 * t + 1] * B[8 + i] - B[4 + i];
    }
    jacobi_nullspace4(D, X);
    if (Xh)
      for (int i = 0; i < 4; ++i) Xh[4 * t + i] = X[i];
    if (Xe)
      for (int i = 0; i < 3; ++i) Xe[3 * t + i] = X[i] / X[3];
  }
}

// ------------------------------------------------- FP64 N-view / algebraic (warp per track)
// A is column-major in shared memory: column c at A + c * ldr, ldr >= rows.
__device__ void warp_jacobi_nullspace(double* A, int ldr, int m, int n, double* V, double* x) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < n * n; idx += 32) V[idx] = (idx / n == idx % n) ? 1.0 : 0.0;  // V column-major n x n
  __syncwarp();
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int i = 0; i < n - 1; ++i)
      for (int j = i + 1; j < n; ++j) {
        double a = 0, b = 0, g = 0;
        const double* ci = A + (size_t)i * ldr;
        const double* cj = A + (size_t)j * ldr;
        for (int r = lane; r < m; r += 32) {
          a += ci[r] * ci[r];
          b += cj[r] * cj[r];
          g += ci[r] * cj[r];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          a += __shfl_xor_sync(0xffffffffu, a, o);
          b += __shfl_xor_sync(0xffffffffu, b, o);
          g += __shfl_xor_sync(0xffffffffu, g, o);
        }
        if (g == 0.0 || fabs(g) <= 1e-15 * sqrt(a * b)) continue;
        rotated = true;
        const double zeta = (b - a) / (2.0 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        double* wi = A + (size_t)i * ldr;
        double* wj = A + (size_t)j * ldr;
        for (int r = lane; r < m; r += 32) {
          const double ui = wi[r], uj = wj[r];
          wi[r] = c * ui - s * uj;
          wj[r] = s * ui + c * uj;
        }
        double* vi = V + (size_t)i * n;
        double* vj = V + (size_t)j * n;
        for (int r = lane; r < n; r += 32) {
          const double a0 = vi[r], a1 = vj[r];
          vi[r] = c * a0 - s * a1;
          vj[r] = s * a0 + c * a1;
        }
        __syncwarp();
      }
    if (!rotated) break;
  }
  // column of smallest norm
  double bn = 1e300;
  int best = 0;
  for (int c = 0; c < n; ++c) {
    double s = 0;
    for (int r = lane; r < m; r += 32) s += A[(size_t)c * ldr + r] * A[(size_t)c * ldr + r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (s < bn) {
      bn = s;
      best = c;
    }
  }
  for (int r = lane; r < n; r += 32) x[r] = V[(size_t)best * n + r];
  __syncwarp();
}

constexpr int kMaxViews = 32;  // GBTRI_NVIEW limit per track (3*32 rows x 36 columns)

__global__ void __launch_bounds__(32) k_nview64(int method, const double* P, const int64_t* offs, const uint32_t* cam,
                                                const double* xy, int64_t nt, double* X) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x;
  for (int64_t t = blockIdx.x; t < nt; t += gridDim.x) {
    const int64_t b = offs[t];
    const int n = (int)(offs[t + 1] - b);
    double* A;
    int m, nc, ldr;
    if (method == 0) {
      m = 3 * n;
      nc = 4 + n;
      ldr = 3 * kMaxViews;
    } else {
      m = 2 * n;
      nc = 4;
      ldr = 3 * kMaxViews;
    }
    A = sm;
    double* V = sm + (size_t)ldr * (4 + kMaxViews);
    double* x = V + (size_t)(4 + kMaxViews) * (4 + kMaxViews);
    for (int idx = lane; idx < ldr * nc; idx += 32) A[idx] = 0.0;
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      const double* Pi = P + 12 * (int64_t)cam[b + i];
      const double px = xy[2 * (b + i)], py = xy[2 * (b + i) + 1];
      if (method == 0) {  // [-P_i | x~_i e_i]
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 4; ++c) A[(size_t)c * ldr + 3 * i + r] = -Pi[4 * r + c];
        A[(size_t)(4 + i) * ldr + 3 * i + 0] = px;
        A[(size_t)(4 + i) * ldr + 3 * i + 1] = py;
        A[(size_t)(4 + i) * ldr + 3 * i + 2] = 1.0;
      } else {  // rows [0,-1,y] P and [1,0,-x] P
        for (int c = 0; c < 4; ++c) {
          A[(size_t)c * ldr + 2 * i] = -Pi[4 + c] + py * Pi[8 + c];
          A[(size_t)c * ldr + 2 * i + 1] = Pi[c] - px * Pi[8 + c];
        }
      }
    }
    __syncwarp();
    warp_jacobi_nullspace(A, ldr, m, nc, V, x);
    if (lane < 4) X[4 * t + lane] = x[lane];
    __syncwarp();
  }
}

// ------------------------------------------------------- FP64 iterated linear (thread per track)
__device__ bool inv3(const double A[9], double Ai[9]) {
  const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  if (!(fabs(det) > 0) || !isfinite(det)) return false;
  const double id = 1.0 / det;
  Ai[0] = c00 * id;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = c01 * id;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = c02 * id;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  return true;
}

__global__ void k_iterative64(const double* P, const int64_t* offs, const uint32_t* cam, const double* xy, int64_t nt,
                              double* X, double* err) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = offs[t];
    const int n = (int)(offs[t + 1] - b);
    double Xc[3] = {0, 0, 0};
    double w[kMaxViews];  // weights; tracks longer than kMaxViews reuse the last slot's rule below
    for (int i = 0; i < kMaxViews; ++i) w[i] = 1.0;
    for (int it = 0; it < 3; ++it) {
      double AtA[9] = {0}, Atb[3] = {0};
      for (int i = 0; i < n; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        const double px = xy[2 * (b + i)], py = xy[2 * (b + i) + 1];
        double wi;
        if (it == 0) wi = 1.0;
        else if (i < kMaxViews) wi = w[i];
        else wi = 1.0 / (Pi[8] * Xc[0] + Pi[9] * Xc[1] + Pi[10] * Xc[2] + Pi[11]);
        double v1[3], v2[3];
        for (int j = 0; j < 3; ++j) {
          v1[j] = wi * (Pi[j] - px * Pi[8 + j]);
          v2[j] = wi * (Pi[4 + j] - py * Pi[8 + j]);
          Atb[j] += wi * (v1[j] * (px * Pi[11] - Pi[3]) + v2[j] * (py * Pi[11] - Pi[7]));
        }
        for (int k = 0; k < 3; ++k)
          for (int j = 0; j <= k; ++j) {
            const double v = v1[j] * v1[k] + v2[j] * v2[k];
            AtA[3 * j + k] += v;
            if (j < k) AtA[3 * k + j] += v;
          }
      }
      double Ai[9];
      inv3(AtA, Ai);
      for (int r = 0; r < 3; ++r) Xc[r] = Ai[3 * r] * Atb[0] + Ai[3 * r + 1] * Atb[1] + Ai[3 * r + 2] * Atb[2];
      for (int i = 0; i < n && i < kMaxViews; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        w[i] = 1.0 / (Pi[8] * Xc[0] + Pi[9] * Xc[1] + Pi[10] * Xc[2] + Pi[11]);
      }
    }
    for (int r = 0; r < 3; ++r) X[3 * t + r] = Xc[r];
    if (err) {
      double e = 0;
      for (int i = 0; i < n; ++i) {
        const double* Pi = P + 12 * (int64_t)cam[b + i];
        double h[3];
        for (int r = 0; r < 3; ++r) h[r] = Pi[4 * r] * Xc[0] + Pi[4 * r + 1] * Xc[1] + Pi[4 * r + 2] * Xc[2] + Pi[4 * r + 3];
        const double dx = xy[2 * (b + i)] - h[0] / h[2], dy = xy[2 * (b + i) + 1] - h[1] / h[2];
        e += sqrt(dx * dx + dy * dy);
      }
      err[t] = e;
    }
  }
}

// ------------------------------------------------------- Gauss-Newton (templated)
template <typename T>
__device__ __forceinline__ bool inv3t(const T A[6], T Ai[6]) {  // symmetric packed [00,01,02,11,12,22]
  const T c00 = A[3] * A[5] - A[4] * A[4], c01 = A[2] * A[4] - A[1] * A[5], c02 = A[1] * A[4] - A[2] * A[3];
  const T det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  if (!(fabs((double)det) > 0) || !isfinite((double)det)) return false;
  const T id = T(1) / det;
  Ai[0] = c00 * id;
  Ai[1] = c01 * id;
  Ai[2] = c02 * id;
  Ai[3] = (A[0] * A[5] - A[2] * A[2]) * id;
  Ai[4] = (A[1] * A[2] - A[0] * A[4]) * id;
  Ai[5] = (A[0] * A[3] - A[1] * A[1]) * id;
  return true;
}

template <typename T>
__device__ __forceinline__ void gn_accumulate(const T* Pi, const T X[3], T px, T py, T H[6], T g[3]) {
  T h[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) h[r] = Pi[4 * r] * X[0] + Pi[4 * r + 1] * X[1] + Pi[4 * r + 2] * X[2] + Pi[4 * r + 3];
  const T iz = T(1) / h[2];
  const T u = h[0] * iz, v = h[1] * iz;
  const T ru = u - px, rv = v - py;
  T Ju[3], Jv[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Ju[j] = (Pi[j] - u * Pi[8 + j]) * iz;
    Jv[j] = (Pi[4 + j] - v * Pi[8 + j]) * iz;
  }
  H[0] += Ju[0] * Ju[0] + Jv[0] * Jv[0];
  H[1] += Ju[0] * Ju[1] + Jv[0] * Jv[1];
  H[2] += Ju[0] * Ju[2] + Jv[0] * Jv[2];
  H[3] += Ju[1] * Ju[1] + Jv[1] * Jv[1];
  H[4] += Ju[1] * Ju[2] + Jv[1] * Jv[2];
  H[5] += Ju[2] * Ju[2] + Jv[2] * Jv[2];
#pragma unroll
  for (int j = 0; j < 3; ++j) g[j] += Ju[j] * ru + Jv[j] * rv;
}

template <typename T>
__device__ __forceinline__ void gn_apply(const T Hi[6], const T g[3], T X[3]) {
  X[0] -= Hi[0] * g[0] + Hi[1] * g[1] + Hi[2] * g[2];
  X[1] -= Hi[1] * g[0] + Hi[3] * g[1] + Hi[4] * g[2];
  X[2] -= Hi[2] * g[0] + Hi[4] * g[1] + Hi[5] * g[2];
}

__global__ void k_refine_gn64(const double* P, const int64_t* offs, const uint32_t* cam, const double* xy, int64_t nt,
                              int steps, double* X) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = offs[t];
    const int n = (int)(offs[t + 1] - b);
    double Xc[3] = {X[3 * t], X[3 * t + 1], X[3 * t + 2]};
    for (int s = 0; s < steps && n >= 2; ++s) {
      double H[6] = {0}, g[3] = {0}, Hi[6];
      for (int i = 0; i < n; ++i)
        gn_accumulate<double>(P + 12 * (int64_t)cam[b + i], Xc, xy[2 * (b + i)], xy[2 * (b + i) + 1], H, g);
      if (!inv3t<double>(H, Hi)) break;
      gn_apply<double>(Hi, g, Xc);
    }
    for (int r = 0; r < 3; ++r) X[3 * t + r] = Xc[r];
  }
}

// FP32 production kernel: 128 tracks per block, observations staged in shared memory.
constexpr int kTriThreads = 128;
constexpr int kTriStage = 4096;  // observations staged per block (12 B each)
constexpr int kTriCams = 1024;   // camera table kept in shared memory up to this size

__global__ void __launch_bounds__(kTriThreads) k_tri_f32(const float* __restrict__ P, int64_t ncam,
                                                         const uint32_t* __restrict__ offs, const uint32_t* __restrict__ cam,
                                                         const float2* __restrict__ xy, int64_t nt, int gn_steps,
                                                         float* __restrict__ X, uint8_t* __restrict__ status,
                                                         float* __restrict__ min_depth) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* sP = reinterpret_cast<float*>(smraw);                                   // [ncam_s][12]
  const int ncam_s = ncam <= kTriCams ? (int)ncam : 0;
  float2* sxy = reinterpret_cast<float2*>(smraw + (size_t)ncam_s * 12 * sizeof(float));
  uint32_t* scam = reinterpret_cast<uint32_t*>(sxy + kTriStage);
  for (int i = threadIdx.x; i < ncam_s * 12; i += kTriThreads) sP[i] = P[i];
  const int64_t t0 = (int64_t)blockIdx.x * kTriThreads;
  const int64_t t1 = min(nt, t0 + kTriThreads);
  const uint32_t ob = offs[t0], oe = offs[t1];
  const bool staged = (oe - ob) <= (uint32_t)kTriStage;
  if (staged) {
    for (uint32_t i = threadIdx.x; i < oe - ob; i += kTriThreads) {
      sxy[i] = xy[ob + i];
      scam[i] = cam[ob + i];
    }
  }
  __syncthreads();
  const int64_t t = t0 + threadIdx.x;
  if (t >= nt) return;
  const uint32_t b = offs[t], e = offs[t + 1];
  const int n = (int)(e - b);
  auto cam_of = [&](uint32_t o) -> const float* {
    const uint32_t c = staged ? scam[o - ob] : cam[o];
    return ncam_s ? sP + 12 * c : P + 12 * (int64_t)c;
  };
  auto xy_of = [&](uint32_t o) -> float2 { return staged ? sxy[o - ob] : xy[o]; };
  float Xc[3] = {0.f, 0.f, 0.f};
  uint8_t st = n >= 2 ? 0 : 1;
  if (st == 0) {
    float A[6] = {0, 0, 0, 0, 0, 0}, r[3] = {0, 0, 0}, Ai[6];
    for (uint32_t o = b; o < e; ++o) {
      const float* Pi = cam_of(o);
      const float2 p = xy_of(o);
      float v1[3], v2[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        v1[j] = Pi[j] - p.x * Pi[8 + j];
        v2[j] = Pi[4 + j] - p.y * Pi[8 + j];
      }
      const float b1 = p.x * Pi[11] - Pi[3], b2 = p.y * Pi[11] - Pi[7];
      A[0] += v1[0] * v1[0] + v2[0] * v2[0];
      A[1] += v1[0] * v1[1] + v2[0] * v2[1];
      A[2] += v1[0] * v1[2] + v2[0] * v2[2];
      A[3] += v1[1] * v1[1] + v2[1] * v2[1];
      A[4] += v1[1] * v1[2] + v2[1] * v2[2];
      A[5] += v1[2] * v1[2] + v2[2] * v2[2];
#pragma unroll
      for (int j = 0; j < 3; ++j) r[j] += v1[j] * b1 + v2[j] * b2;
    }
    if (inv3t<float>(A, Ai)) {
      Xc[0] = Ai[0] * r[0] + Ai[1] * r[1] + Ai[2] * r[2];
      Xc[1] = Ai[1] * r[0] + Ai[3] * r[1] + Ai[4] * r[2];
      Xc[2] = Ai[2] * r[0] + Ai[4] * r[1] + Ai[5] * r[2];
    } else {
      st = 1;
    }
  }
  for (int s = 0; s < gn_steps && st == 0; ++s) {
    float H[6] = {0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0}, Hi[6];
    for (uint32_t o = b; o < e; ++o) {
      const float2 p = xy_of(o);
      gn_accumulate<float>(cam_of(o), Xc, p.x, p.y, H, g);
    }
    if (!inv3t<float>(H, Hi)) {
      st = 1;
      break;
    }
    gn_apply<float>(Hi, g, Xc);
  }
  float md = 3.402823466e38f;
  for (uint32_t o = b; o < e; ++o) {
    const float* Pi = cam_of(o);
    md = fminf(md, Pi[8] * Xc[0] + Pi[9] * Xc[1] + Pi[10] * Xc[2] + Pi[11]);
  }
  if (st == 0 && !(md > 0.f)) st = 2;
  X[3 * t] = Xc[0];
  X[3 * t + 1] = Xc[1];
  X[3 * t + 2] = Xc[2];
  if (status) status[t] = st;
  if (min_depth) min_depth[t] = n > 0 ? md : 0.f;
}

size_t tri_f32_smem(int64_t ncam) {
  const int ncam_s = ncam <= kTriCams ? (int)ncam : 0;
  return (size_t)ncam_s * 12 * sizeof(float) + (size_t)kTriStage * (sizeof(float2) + sizeof(uint32_t));
}

}  // namespace gbba

using namespace gbba;

namespace {

template <typename F>
gbba_status tri_guard(gbba_handle* h, F&& f) {
  if (!h) return GBBA_ERROR_INVALID_ARGUMENT;
  try {
    GBBA_CUDA(cudaSetDevice(h->device));
    h->active = h->stream;
    return f();
  } catch (const Error& e) {
    if (std::getenv("GBBA_VERBOSE")) fprintf(stderr, "gbtri: %s\n", e.what.c_str());
    cudaGetLastError();
    return e.status;
  }
}

// Device view of an input array: the caller's pointer (device memory) or a
// staged copy (host memory).
template <typename T>
const T* in_view(gbba_handle* h, const T* p, size_t count, int memory) {
  if (!p || memory == GBBA_MEMORY_DEVICE) return p;
  T* d = h->arena.take<T>(count);
  if (count) GBBA_CUDA(cudaMemcpyAsync(d, p, count * sizeof(T), cudaMemcpyHostToDevice, h->active));
  return d;
}
template <typename T>
T* out_view(gbba_handle* h, T* p, size_t count, int memory) {
  if (!p || memory == GBBA_MEMORY_DEVICE) return p;
  return h->arena.take<T>(count);
}
template <typename T>
void out_back(gbba_handle* h, T* user, const T* dev, size_t count, int memory) {
  if (!user || memory == GBBA_MEMORY_DEVICE || count == 0) return;
  GBBA_CUDA(cudaMemcpyAsync(user, dev, count * sizeof(T), cudaMemcpyDeviceToHost, h->active));
}

// Device check of CSR offsets: offs[0] == 0, non-decreasing; returns the total
// and the longest track.  info = {error, max_len, total_lo, total_hi}.
template <typename Off>
__global__ void k_check_offsets(const Off* offs, int64_t nt, unsigned int* info) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = (int64_t)offs[t], b = (int64_t)offs[t + 1];
    if (b < a || (t == 0 && a != 0)) atomicExch(&info[0], 1u);
    else atomicMax(&info[1], (unsigned int)(b - a > 0x7fffffff ? 0x7fffffff : b - a));
    if (t == nt - 1) {
      info[2] = (unsigned int)(b & 0xffffffff);
      info[3] = (unsigned int)(b >> 32);
    }
  }
}

template <typename Off>
void check_offsets(gbba_handle* h, const Off* offs, int64_t nt, int memory, int64_t* total, int* max_len) {
  if (memory == GBBA_MEMORY_DEVICE) {
    unsigned int* info = nullptr;
    GBBA_CUDA(cudaMallocAsync((void**)&info, 4 * sizeof(unsigned int), h->active));
    GBBA_CUDA(cudaMemsetAsync(info, 0, 4 * sizeof(unsigned int), h->active));
    k_check_offsets<Off><<<std::max(1, std::min<int>((int)ceil_div(nt, 256), h->sm_count * 8)), 256, 0, h->active>>>(offs, nt, info);
    check_launch(h);
    unsigned int hi[4];
    GBBA_CUDA(cudaMemcpyAsync(hi, info, sizeof(hi), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaFreeAsync(info, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    GBBA_REQUIRE(hi[0] == 0, GBBA_ERROR_INVALID_ARGUMENT, "track_offsets must start at 0 and be non-decreasing");
    *max_len = (int)hi[1];
    *total = (int64_t)hi[2] | ((int64_t)hi[3] << 32);
    return;
  }
  std::vector<Off> ho(nt + 1);
  std::memcpy(ho.data(), offs, sizeof(Off) * (nt + 1));
  GBBA_REQUIRE(ho[0] == 0, GBBA_ERROR_INVALID_ARGUMENT, "track_offsets[0] must be 0");
  int ml = 0;
  for (int64_t t = 0; t < nt; ++t) {
    GBBA_REQUIRE(ho[t + 1] >= ho[t], GBBA_ERROR_INVALID_ARGUMENT, "track_offsets must be non-decreasing");
    ml = std::max<int>(ml, (int)(ho[t + 1] - ho[t]));
  }
  *total = (int64_t)ho[nt];
  *max_len = ml;
}

__global__ void k_check_cam(const uint32_t* cam, int64_t n, int64_t ncam, int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (cam[i] >= ncam) atomicExch(err, 1);
}

void check_cams(gbba_handle* h, const uint32_t* dcam, int64_t n, int64_t ncam) {
  int* err = h->arena.take<int>(1);
  GBBA_CUDA(cudaMemsetAsync(err, 0, sizeof(int), h->active));
  if (n > 0) {
    k_check_cam<<<std::max(1, std::min<int>((int)ceil_div(n, 256), h->sm_count * 8)), 256, 0, h->active>>>(dcam, n, ncam, err);
    check_launch(h);
  }
  int herr = 0;
  GBBA_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, h->active));
  GBBA_CUDA(cudaStreamSynchronize(h->active));
  GBBA_REQUIRE(herr == 0, GBBA_ERROR_INVALID_ARGUMENT, "camera_index out of range");
}

}  // namespace

extern "C" {

gbba_status gbtri_dlt2_batched(gbba_handle* h, int64_t n, const double* P1, const double* P2, int64_t p_stride,
                               const double* x1, const double* x2, double* X_homogeneous, double* X_euclidean,
                               int32_t memory) {
  if (n < 0 || !P1 || !P2 || !x1 || !x2 || (p_stride != 0 && p_stride != 12)) return GBBA_ERROR_INVALID_ARGUMENT;
  return tri_guard(h, [&]() {
    if (n == 0) return GBBA_SUCCESS;
    h->arena.reset();
    const size_t np_ = p_stride ? 12 * (size_t)n : 12;
    h->arena.reserve(sizeof(double) * (2 * np_ + 4 * n + 7 * n) + 16 * 256);
    const double* dP1 = in_view(h, P1, np_, memory);
    const double* dP2 = in_view(h, P2, np_, memory);
    const double* dx1 = in_view(h, x1, 2 * n, memory);
    const double* dx2 = in_view(h, x2, 2 * n, memory);
    double* dXh = out_view(h, X_homogeneous, 4 * n, memory);
    double* dXe = out_view(h, X_euclidean, 3 * n, memory);
    k_dlt2<<<std::max(1, std::min<int>((int)ceil_div(n, 128), h->sm_count * 16)), 128, 0, h->active>>>(
        n, dP1, dP2, p_stride, dx1, dx2, dXh, dXe);
    check_launch(h);
    out_back(h, X_homogeneous, dXh, 4 * n, memory);
    out_back(h, X_euclidean, dXe, 3 * n, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    return GBBA_SUCCESS;
  });
}

gbba_status gbtri_nview_batched(gbba_handle* h, int32_t method, const double* P, int64_t num_cameras,
                                const int64_t* track_offsets, const uint32_t* camera_index, const double* xy,
                                int64_t num_tracks, double* X, double* error, int32_t memory) {
  if (method < 0 || method > 2 || num_tracks < 0 || num_cameras < 0 || !P || !track_offsets || !X)
    return GBBA_ERROR_INVALID_ARGUMENT;
  return tri_guard(h, [&]() {
    if (num_tracks == 0) return GBBA_SUCCESS;
    int64_t no = 0;
    int max_len = 0;
    check_offsets(h, track_offsets, num_tracks, memory, &no, &max_len);
    GBBA_REQUIRE(method != GBTRI_NVIEW || max_len <= kMaxViews, GBBA_ERROR_TOO_LARGE,
                 "TriangulateNView path limited to 32 views per track");
    GBBA_REQUIRE(method != GBTRI_NVIEW_ALGEBRAIC || max_len <= 48, GBBA_ERROR_TOO_LARGE,
                 "algebraic N-view path limited to 48 views per track");
    h->arena.reset();
    const int xo = method == 2 ? 3 : 4;
    h->arena.reserve(sizeof(double) * (12 * num_cameras + 2 * no + (xo + 1) * num_tracks) + sizeof(int64_t) * (num_tracks + 1) +
                     sizeof(uint32_t) * no + 16 * 256);
    const double* dP = in_view(h, P, 12 * (size_t)num_cameras, memory);
    const int64_t* doff = in_view(h, track_offsets, num_tracks + 1, memory);
    const uint32_t* dcam = in_view(h, camera_index, no, memory);
    const double* dxy = in_view(h, xy, 2 * no, memory);
    double* dX = out_view(h, X, xo * num_tracks, memory);
    double* derr = out_view(h, error, num_tracks, memory);
    check_cams(h, dcam, no, num_cameras);
    if (method == GBTRI_ITERATIVE) {
      k_iterative64<<<std::max(1, std::min<int>((int)ceil_div(num_tracks, 128), h->sm_count * 16)), 128, 0, h->active>>>(
          dP, doff, dcam, dxy, num_tracks, dX, derr);
    } else {
      const size_t smem = sizeof(double) * ((size_t)3 * kMaxViews * (4 + kMaxViews) + (4 + kMaxViews) * (4 + kMaxViews) + 64);
      static PerDeviceOnce once;
      once.run([&] { GBBA_CUDA(cudaFuncSetAttribute(k_nview64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); });
      k_nview64<<<(unsigned)std::min<int64_t>(num_tracks, (int64_t)h->sm_count * 32), 32, smem, h->active>>>(
          method, dP, doff, dcam, dxy, num_tracks, dX);
    }
    check_launch(h);
    out_back(h, X, dX, xo * num_tracks, memory);
    if (method == GBTRI_ITERATIVE) out_back(h, error, derr, num_tracks, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    return GBBA_SUCCESS;
  });
}

gbba_status gbtri_nview_batched_f32(gbba_handle* h, const float* P, int64_t num_cameras, const uint32_t* track_offsets,
                                    const uint32_t* camera_index, const float* xy, int64_t num_tracks, int32_t gn_steps,
                                    float* X, uint8_t* status, float* min_depth, int32_t memory) {
  if (num_tracks < 0 || num_cameras < 0 || gn_steps < 0 || !P || !track_offsets || !X) return GBBA_ERROR_INVALID_ARGUMENT;
  if (num_tracks >= 0xFFFFFFFFLL) return GBBA_ERROR_TOO_LARGE;
  return tri_guard(h, [&]() {
    if (num_tracks == 0) return GBBA_SUCCESS;
    int64_t no = 0;
    int max_len = 0;
    check_offsets(h, track_offsets, num_tracks, memory, &no, &max_len);
    h->arena.reset();
    h->arena.reserve(sizeof(float) * (12 * num_cameras + 2 * no + 4 * num_tracks) + sizeof(uint32_t) * (num_tracks + 1 + no) +
                     num_tracks + 16 * 256);
    const float* dP = in_view(h, P, 12 * (size_t)num_cameras, memory);
    const uint32_t* doff = in_view(h, track_offsets, num_tracks + 1, memory);
    const uint32_t* dcam = in_view(h, camera_index, no, memory);
    const float* dxy = in_view(h, xy, 2 * no, memory);
    float* dX = out_view(h, X, 3 * num_tracks, memory);
    uint8_t* dst = out_view(h, status, num_tracks, memory);
    float* dmd = out_view(h, min_depth, num_tracks, memory);
    check_cams(h, dcam, no, num_cameras);
    const size_t smem = tri_f32_smem(num_cameras);
    static PerDeviceOnce once;
    once.run([] {
      GBBA_CUDA(cudaFuncSetAttribute(k_tri_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tri_f32_smem(kTriCams)));
    });
    k_tri_f32<<<(unsigned)ceil_div(num_tracks, kTriThreads), kTriThreads, smem, h->active>>>(
        dP, num_cameras, doff, dcam, reinterpret_cast<const float2*>(dxy), num_tracks, gn_steps, dX, dst, dmd);
    check_launch(h);
    out_back(h, X, dX, 3 * num_tracks, memory);
    out_back(h, status, dst, num_tracks, memory);
    out_back(h, min_depth, dmd, num_tracks, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    return GBBA_SUCCESS;
  });
}

gbba_status gbtri_refine_gn(gbba_handle* h, const double* P, int64_t num_cameras, const int64_t* track_offsets,
                            const uint32_t* camera_index, const double* xy, int64_t num_tracks, int32_t steps, double* X,
                            int32_t memory) {
  if (num_tracks < 0 || steps < 0 || !P || !track_offsets || !X) return GBBA_ERROR_INVALID_ARGUMENT;
  return tri_guard(h, [&]() {
    if (num_tracks == 0) return GBBA_SUCCESS;
    int64_t no = 0;
    int max_len = 0;
    check_offsets(h, track_offsets, num_tracks, memory, &no, &max_len);
    h->arena.reset();
    h->arena.reserve(sizeof(double) * (12 * num_cameras + 2 * no + 3 * num_tracks) + sizeof(int64_t) * (num_tracks + 1) +
                     sizeof(uint32_t) * no + 16 * 256);
    const double* dP = in_view(h, P, 12 * (size_t)num_cameras, memory);
    const int64_t* doff = in_view(h, track_offsets, num_tracks + 1, memory);
    const uint32_t* dcam = in_view(h, camera_index, no, memory);
    const double* dxy = in_view(h, xy, 2 * no, memory);
    double* dX = const_cast<double*>(in_view(h, (const double*)X, 3 * num_tracks, memory));
    check_cams(h, dcam, no, num_cameras);
    k_refine_gn64<<<std::max(1, std::min<int>((int)ceil_div(num_tracks, 128), h->sm_count * 16)), 128, 0, h->active>>>(
        dP, doff, dcam, dxy, num_tracks, steps, dX);
    check_launch(h);
    out_back(h, X, dX, 3 * num_tracks, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    return GBBA_SUCCESS;
  });
}

}  // extern "C"
