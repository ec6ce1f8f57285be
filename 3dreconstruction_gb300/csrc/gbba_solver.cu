// Levenberg-Marquardt bundle adjustment on one GPU.
//
// One solve replaces the ceres::Solve call of the reference call sites
// (libs/sfm/src/sfm_incremental_engine.cpp:1395-1473 and
// libs/sfm/src/sfm_global_engine.cpp:1142-1174, 1546-1594, 1756-1802) with the
// same trust-region semantics:
//   - Jacobi column scaling fixed from the initial Jacobian
//       (3rdparty/ceres/internal/ceres/trust_region_minimizer.cc:103-108, 238-243);
//   - LM diagonal D = sqrt(clamp(diag(J^T J), 1e-6, 1e32) / radius), reused
//       after a rejected step (levenberg_marquardt_strategy.cc:65-145);
//   - step from the Schur complement on the point blocks
//       (schur_eliminator_impl.h:173-370) and a dense Cholesky of S;
//   - model cost change, relative decrease, radius update and the
//       parameter / function / gradient tolerance terminations
//       (trust_region_minimizer.cc:327-345, 489-580, 650-716;
//       levenberg_marquardt_strategy.cc:147-160).
//
// Device data layout (all resident in HBM for the whole solve):
//   params     extrinsics [Nc][6], intrinsics [Ni][k], points [Np][3]  FP64, twice
//              (current and candidate x + delta)
//   obs        (x,y) FP64 pairs, camera / intrinsic index u32, sorted by point
//              with CSR offsets pt_off[Np+1]
//   S          n_pad x n_pad (lower triangle) in the compute type, rhs [n_pad]
//   per point  V^-1 (6, symmetric), g_p (3)
//   per obs    W = F^T E and W V^-1 ((6+k) x 3 each) scratch for the pair products
// Kernels are templated on the camera model M and the compute type T
// (double: the plain FP64 path; float: the mixed path, whose residuals and
// cost stay FP64).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>

#include "gbba_device.cuh"
#include "gbba_internal.h"

namespace gbba {

template <typename T>
void dense_cholesky_solve(gbba_handle* h, T* S, int64_t n_pad, T* b, T* x, T* Linv_all, int* flag, cudaStream_t st);

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int model_k(int m) { return m == kPinholeF ? 1 : m == kRadialK3 ? 6 : 8; }

// ------------------------------------------------------------------ setup kernels
__global__ void k_validate(const uint32_t* cam, const uint32_t* icam, const uint32_t* pt, int64_t no, int64_t nc,
                           int64_t ni, int64_t np, int* err, uint32_t* counts, uint8_t* cam_used, uint8_t* intr_used) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < no; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cam[i], g = icam[i], p = pt[i];
    if (c >= nc || g >= ni || p >= np) {
      atomicExch(err, 1);
      continue;
    }
    atomicAdd(&counts[p], 1u);
    cam_used[c] = 1;
    intr_used[g] = 1;
  }
}

// Exclusive scan of counts[0..n) into off[0..n] (off[n] = total); one block
// per 1024-chunk then a sequential carry over chunk sums.
__global__ void k_scan_chunks(const uint32_t* in, uint32_t* out, uint32_t* chunk_sums, int64_t n) {
  __shared__ uint32_t s[1024];
  const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
  uint32_t v = i < n ? in[i] : 0u;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint32_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;  // exclusive within chunk
  if (threadIdx.x == 1023) chunk_sums[blockIdx.x] = s[1023];
}
__global__ void k_scan_carry(uint32_t* chunk_sums, int64_t nchunks, uint32_t* total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    uint32_t run = 0;
    for (int64_t c = 0; c < nchunks; ++c) {
      const uint32_t v = chunk_sums[c];
      chunk_sums[c] = run;
      run += v;
    }
    *total = run;
  }
}
__global__ void k_scan_add(uint32_t* out, const uint32_t* chunk_sums, int64_t n) {
  const int64_t i = blockIdx.x * 1024LL + threadIdx.x;
  if (i < n) out[i] += chunk_sums[blockIdx.x];
}

__global__ void k_scatter(const uint32_t* pt, int64_t no, const uint32_t* off, uint32_t* fill, uint32_t* perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < no; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t p = pt[i];
    const uint32_t pos = off[p] + atomicAdd(&fill[p], 1u);
    perm[pos] = (uint32_t)i;
  }
}
// Restore input order inside each point's segment (deterministic result).
__global__ void k_segment_sort(uint32_t* perm, const uint32_t* off, int64_t np) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = off[p], e = off[p + 1];
    for (uint32_t i = b + 1; i < e; ++i) {
      const uint32_t v = perm[i];
      uint32_t j = i;
      while (j > b && perm[j - 1] > v) {
        perm[j] = perm[j - 1];
        --j;
      }
      perm[j] = v;
    }
  }
}
__global__ void k_gather(const uint32_t* perm, int64_t no, const double* obs_in, const uint32_t* cam_in,
                         const uint32_t* icam_in, const uint32_t* pt_in, double2* obs, uint32_t* cam, uint32_t* icam,
                         uint32_t* pt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < no; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = perm[i];
    obs[i] = make_double2(obs_in[2 * (int64_t)s], obs_in[2 * (int64_t)s + 1]);
    cam[i] = cam_in[s];
    icam[i] = icam_in[s];
    pt[i] = pt_in[s];
  }
}

// ------------------------------------------------------------------ shared argument block
struct Prob {
  const double* ext;
  const double* intr;
  const double* pts;
  const double2* obs;
  const uint32_t* cam;
  const uint32_t* icam;
  const uint32_t* pt;
  const uint32_t* pt_off;
  const int32_t* ext_col;
  const int32_t* intr_col;
  int64_t nc, ni, np, no;
  int loss_type;
  double loss_a;
};

template <int M, typename T>
struct ObsJac {
  static constexpr int K = Model<M>::K;
  static constexpr int B = 6 + K;
  double r[2];      // corrected residual (FP64)
  T Jc[2][B];       // corrected [extrinsic | intrinsic] block (scaled when requested)
  T Jp[2][3];       // corrected point block
  int32_t col[B];   // reduced column of each camera-side coordinate (-1 = held)
};

// Residual and Jacobian of observation o, robustified (Corrector) and, with
// kScale, multiplied by the Jacobi column scaling.
template <int M, typename T, bool kScale>
__device__ __forceinline__ void obs_jacobian(const Prob& P, int64_t o, const double* __restrict__ scale_c,
                                             const double* __restrict__ scale_p, ObsJac<M, T>& J, double* cost) {
  constexpr int K = Model<M>::K;
  const uint32_t c = P.cam[o], g = P.icam[o], p = P.pt[o];
  const double2 ob = P.obs[o];
  double Ed[6], Kd[K], Xd[3];
#pragma unroll
  for (int i = 0; i < 6; ++i) Ed[i] = __ldg(&P.ext[6 * (int64_t)c + i]);
#pragma unroll
  for (int i = 0; i < K; ++i) Kd[i] = __ldg(&P.intr[K * (int64_t)g + i]);
#pragma unroll
  for (int i = 0; i < 3; ++i) Xd[i] = __ldg(&P.pts[3 * (int64_t)p + i]);
  T Je[2][6], Jk[2][K], Jx[2][3];
  double r[2];
  if constexpr (sizeof(T) == 8) {
    residual<M, T, true>(Kd, Ed, Xd, ob.x, ob.y, r, Je, Jk, Jx, (T*)nullptr);
  } else {
    double dJe[2][6], dJk[2][K], dJx[2][3];
    residual<M, double, false>(Kd, Ed, Xd, ob.x, ob.y, r, dJe, dJk, dJx, (double*)nullptr);
    T Ef[6], Kf[K], Xf[3], rf[2];
#pragma unroll
    for (int i = 0; i < 6; ++i) Ef[i] = (T)Ed[i];
#pragma unroll
    for (int i = 0; i < K; ++i) Kf[i] = (T)Kd[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) Xf[i] = (T)Xd[i];
    residual<M, T, true>(Kf, Ef, Xf, (T)ob.x, (T)ob.y, rf, Je, Jk, Jx, (T*)nullptr);
  }
  double sr1;
  *cost = robust<double>(P.loss_type, P.loss_a, r[0] * r[0] + r[1] * r[1], &sr1);
  J.r[0] = r[0] * sr1;
  J.r[1] = r[1] * sr1;
  const T s = (T)sr1;
#pragma unroll
  for (int j = 0; j < 6; ++j) J.col[j] = __ldg(&P.ext_col[6 * (int64_t)c + j]);
#pragma unroll
  for (int j = 0; j < K; ++j) J.col[6 + j] = __ldg(&P.intr_col[K * (int64_t)g + j]);
#pragma unroll
  for (int j = 0; j < ObsJac<M, T>::B; ++j) {
    T sc = s;
    if (kScale) sc = J.col[j] >= 0 ? (T)(scale_c[J.col[j]] * sr1) : T(0);
#pragma unroll
    for (int i = 0; i < 2; ++i) J.Jc[i][j] = (j < 6 ? Je[i][j] : Jk[i][j - 6]) * sc;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const T sc = kScale ? (T)(scale_p[3 * (int64_t)p + j] * sr1) : s;
#pragma unroll
    for (int i = 0; i < 2; ++i) J.Jp[i][j] = Jx[i][j] * sc;
  }
}

// Squared column norms and gradient (unscaled, corrected) at the current x.
template <int M, typename T>
__global__ void __launch_bounds__(256) k_linearize(Prob P, double* __restrict__ cn_c, double* __restrict__ cn_p,
                                                   double* __restrict__ g_c, double* __restrict__ g_p) {
  constexpr int B = ObsJac<M, T>::B;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.no; o += (int64_t)gridDim.x * blockDim.x) {
    ObsJac<M, T> J;
    double cost;
    obs_jacobian<M, T, false>(P, o, nullptr, nullptr, J, &cost);
#pragma unroll
    for (int j = 0; j < B; ++j) {
      if (J.col[j] < 0) continue;
      const double a = J.Jc[0][j], b = J.Jc[1][j];
      atomicAdd(&cn_c[J.col[j]], a * a + b * b);
      atomicAdd(&g_c[J.col[j]], a * J.r[0] + b * J.r[1]);
    }
    const int64_t p = P.pt[o];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double a = J.Jp[0][j], b = J.Jp[1][j];
      atomicAdd(&cn_p[3 * p + j], a * a + b * b);
      atomicAdd(&g_p[3 * p + j], a * J.r[0] + b * J.r[1]);
    }
  }
}

// scale (first linearization only), LM diagonal and max |gradient|.
__global__ void k_scale_diag(int64_t n, const double* cn, const double* g, double* scale, double* diag, int first,
                             int jacobi, double dmin, double dmax, unsigned long long* gmax_bits) {
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (first) scale[i] = jacobi ? 1.0 / (1.0 + sqrt(cn[i])) : 1.0;
    const double s = scale[i];
    diag[i] = fmin(fmax(cn[i] * s * s, dmin), dmax);
    m = fmax(m, fabs(g[i]));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(gmax_bits, (unsigned long long)__double_as_longlong(m));
}

// S <- diag(D_c^2) (identity on the padding), rhs <- 0.
template <typename T>
__global__ void k_schur_init(T* S, T* rhs, int64_t n, int64_t n_pad, const double* diag_c, const double* radius) {
  const double rad = *radius;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad; i += (int64_t)gridDim.x * blockDim.x) {
    S[i * n_pad + i] = i < n ? (T)(diag_c[i] / rad) : T(1);
    rhs[i] = T(0);
  }
}

// Point-major Schur elimination: one warp per point.  Accumulates
//   V = D_p^2 + sum E'E, g_p = sum E'r, V^-1                      (per point)
//   rhs += F'r - (F'E) V^-1 g_p,  S += F'F - (F'E) V^-1 (E'F)    (lower triangle)
template <int M, typename T>
__global__ void __launch_bounds__(128) k_schur_point(Prob P, const double* __restrict__ scale_c,
                                                     const double* __restrict__ scale_p, const double* __restrict__ diag_p,
                                                     const double* __restrict__ radius, T* __restrict__ S, int64_t ld,
                                                     T* __restrict__ rhs, T* __restrict__ Vinv, T* __restrict__ gp,
                                                     T* __restrict__ Wbuf, T* __restrict__ What, int* __restrict__ flag) {
  constexpr int B = ObsJac<M, T>::B;
  const int lane = threadIdx.x & 31;
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (p >= P.np) return;
  const uint32_t ob = P.pt_off[p], oe = P.pt_off[p + 1];
  T v[6] = {}, g[3] = {};
  for (uint32_t o = ob + lane; o < oe; o += 32) {
    ObsJac<M, T> J;
    double cost;
    obs_jacobian<M, T, true>(P, o, scale_c, scale_p, J, &cost);
    const T r0 = (T)J.r[0], r1 = (T)J.r[1];
    v[0] += J.Jp[0][0] * J.Jp[0][0] + J.Jp[1][0] * J.Jp[1][0];
    v[1] += J.Jp[0][0] * J.Jp[0][1] + J.Jp[1][0] * J.Jp[1][1];
    v[2] += J.Jp[0][0] * J.Jp[0][2] + J.Jp[1][0] * J.Jp[1][2];
    v[3] += J.Jp[0][1] * J.Jp[0][1] + J.Jp[1][1] * J.Jp[1][1];
    v[4] += J.Jp[0][1] * J.Jp[0][2] + J.Jp[1][1] * J.Jp[1][2];
    v[5] += J.Jp[0][2] * J.Jp[0][2] + J.Jp[1][2] * J.Jp[1][2];
#pragma unroll
    for (int j = 0; j < 3; ++j) g[j] += J.Jp[0][j] * r0 + J.Jp[1][j] * r1;
    T* W = Wbuf + (int64_t)o * B * 3;
#pragma unroll
    for (int i = 0; i < B; ++i) {
#pragma unroll
      for (int j = 0; j < 3; ++j) W[i * 3 + j] = J.Jc[0][i] * J.Jp[0][j] + J.Jc[1][i] * J.Jp[1][j];
      const int ci = J.col[i];
      if (ci < 0) continue;
      atomicAdd(&rhs[ci], J.Jc[0][i] * r0 + J.Jc[1][i] * r1);
#pragma unroll
      for (int j = 0; j < B; ++j) {
        const int cj = J.col[j];
        if (cj < 0 || cj > ci) continue;
        atomicAdd(&S[(int64_t)ci * ld + cj], J.Jc[0][i] * J.Jc[0][j] + J.Jc[1][i] * J.Jc[1][j]);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) v[i] = warp_sum(v[i]);
#pragma unroll
  for (int i = 0; i < 3; ++i) g[i] = warp_sum(g[i]);
  // V + D_p^2 and its inverse through a 3x3 Cholesky (ceres: ete.llt().solve(I))
  const double rad = *radius;
  const T a00 = v[0] + (T)(diag_p[3 * p] / rad), a11 = v[3] + (T)(diag_p[3 * p + 1] / rad),
          a22 = v[5] + (T)(diag_p[3 * p + 2] / rad);
  const T l00 = sqrt(a00), l10 = v[1] / l00, l20 = v[2] / l00;
  const T d1 = a11 - l10 * l10;
  const T l11 = sqrt(d1), l21 = (v[4] - l20 * l10) / l11;
  const T d2 = a22 - l20 * l20 - l21 * l21;
  const T l22 = sqrt(d2);
  // inverse of L (lower), then V^-1 = L^-T L^-1
  const T i00 = T(1) / l00, i11 = T(1) / l11, i22 = T(1) / l22;
  const T i10 = -l10 * i00 * i11, i21 = -l21 * i11 * i22, i20 = -(l20 * i00 + l21 * i10) * i22;
  T vi[6];
  vi[0] = i00 * i00 + i10 * i10 + i20 * i20;
  vi[1] = i10 * i11 + i20 * i21;
  vi[2] = i20 * i22;
  vi[3] = i11 * i11 + i21 * i21;
  vi[4] = i21 * i22;
  vi[5] = i22 * i22;
  if (!(a00 > T(0)) || !(d1 > T(0)) || !(d2 > T(0)) || !isfinite((double)vi[0]) || !isfinite((double)vi[3]) ||
      !isfinite((double)vi[5])) {
    if (lane == 0) atomicExch(flag, 2);
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 6; ++i) Vinv[6 * p + i] = vi[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) gp[3 * p + i] = g[i];
  }
  const T Vf[3][3] = {{vi[0], vi[1], vi[2]}, {vi[1], vi[3], vi[4]}, {vi[2], vi[4], vi[5]}};
  for (uint32_t o = ob + lane; o < oe; o += 32) {
    const T* W = Wbuf + (int64_t)o * B * 3;
    T* Wh = What + (int64_t)o * B * 3;
    const uint32_t c = P.cam[o], gi = P.icam[o];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      T y[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) y[j] = W[i * 3] * Vf[0][j] + W[i * 3 + 1] * Vf[1][j] + W[i * 3 + 2] * Vf[2][j];
#pragma unroll
      for (int j = 0; j < 3; ++j) Wh[i * 3 + j] = y[j];
      const int ci = i < 6 ? P.ext_col[6 * (int64_t)c + i] : P.intr_col[(B - 6) * (int64_t)gi + (i - 6)];
      if (ci >= 0) atomicAdd(&rhs[ci], -(y[0] * g[0] + y[1] * g[1] + y[2] * g[2]));
    }
  }
  __syncwarp();
  // pair products: S[c_a(i)][c_b(j)] -= What_a[i] . W_b[j] on the lower triangle
  const uint32_t m = oe - ob;
  for (uint32_t a = 0; a < m; ++a) {
    const uint32_t oa = ob + a;
    const uint32_t ca = P.cam[oa], ga = P.icam[oa];
    for (uint32_t bb = 0; bb < m; ++bb) {
      const uint32_t obb = ob + bb;
      const uint32_t cb = P.cam[obb], gb = P.icam[obb];
      for (int e = lane; e < B * B; e += 32) {
        const int i = e / B, j = e % B;
        const int ci = i < 6 ? P.ext_col[6 * (int64_t)ca + i] : P.intr_col[(B - 6) * (int64_t)ga + (i - 6)];
        const int cj = j < 6 ? P.ext_col[6 * (int64_t)cb + j] : P.intr_col[(B - 6) * (int64_t)gb + (j - 6)];
        if (ci < 0 || cj < 0 || cj > ci) continue;
        const T* x = What + (int64_t)oa * B * 3 + i * 3;
        const T* y = Wbuf + (int64_t)obb * B * 3 + j * 3;
        atomicAdd(&S[(int64_t)ci * ld + cj], -(x[0] * y[0] + x[1] * y[1] + x[2] * y[2]));
      }
    }
  }
}

// Back substitution (one warp per point) + model cost change + candidate points.
//   y_p = V^-1 (g_p - sum E'F z), step = -(z, y), m = J step,
//   model_cost_change += -m.(r + m/2)
template <int M, typename T>
__global__ void __launch_bounds__(128) k_backsub(Prob P, const double* __restrict__ scale_c,
                                                 const double* __restrict__ scale_p, const T* __restrict__ z,
                                                 const T* __restrict__ Vinv, const T* __restrict__ gp,
                                                 double* __restrict__ pts_new, double* __restrict__ part_mcc,
                                                 double* __restrict__ part_step, int* __restrict__ flag) {
  constexpr int B = ObsJac<M, T>::B;
  __shared__ double smcc[4], sstep[4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  double mcc = 0.0, stp = 0.0;
  if (p < P.np) {
    const uint32_t ob = P.pt_off[p], oe = P.pt_off[p + 1];
    // pass 1: t = sum_o E_o' (F_o z)
    T t[3] = {};
    for (uint32_t o = ob + lane; o < oe; o += 32) {
      ObsJac<M, T> J;
      double cost;
      obs_jacobian<M, T, true>(P, o, scale_c, scale_p, J, &cost);
      T fz0 = T(0), fz1 = T(0);
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T zi = J.col[i] >= 0 ? z[J.col[i]] : T(0);
        fz0 += J.Jc[0][i] * zi;
        fz1 += J.Jc[1][i] * zi;
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) t[j] += J.Jp[0][j] * fz0 + J.Jp[1][j] * fz1;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) t[j] = warp_sum(t[j]);
    const T* vi = Vinv + 6 * p;
    const T q0 = gp[3 * p] - t[0], q1 = gp[3 * p + 1] - t[1], q2 = gp[3 * p + 2] - t[2];
    const T y[3] = {vi[0] * q0 + vi[1] * q1 + vi[2] * q2, vi[1] * q0 + vi[3] * q1 + vi[4] * q2,
                    vi[2] * q0 + vi[4] * q1 + vi[5] * q2};
    if (!isfinite((double)y[0]) || !isfinite((double)y[1]) || !isfinite((double)y[2])) {
      if (lane == 0) atomicExch(flag, 3);
    }
    // pass 2: model residuals
    for (uint32_t o = ob + lane; o < oe; o += 32) {
      ObsJac<M, T> J;
      double cost;
      obs_jacobian<M, T, true>(P, o, scale_c, scale_p, J, &cost);
      double m0 = 0.0, m1 = 0.0;
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const double zi = J.col[i] >= 0 ? (double)z[J.col[i]] : 0.0;
        m0 += (double)J.Jc[0][i] * zi;
        m1 += (double)J.Jc[1][i] * zi;
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        m0 += (double)J.Jp[0][j] * (double)y[j];
        m1 += (double)J.Jp[1][j] * (double)y[j];
      }
      m0 = -m0;
      m1 = -m1;
      mcc += -(m0 * (J.r[0] + m0 / 2.0) + m1 * (J.r[1] + m1 / 2.0));
    }
    if (lane < 3) {
      const double d = -(double)y[lane] * scale_p[3 * p + lane];
      pts_new[3 * p + lane] = P.pts[3 * p + lane] + d;
      stp = d * d;
    }
  }
  mcc = warp_sum(mcc);
  stp = warp_sum(stp);
  if (lane == 0) {
    smcc[warp] = mcc;
    sstep[warp] = stp;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    part_mcc[blockIdx.x] = smcc[0] + smcc[1] + smcc[2] + smcc[3];
    part_step[blockIdx.x] = sstep[0] + sstep[1] + sstep[2] + sstep[3];
  }
}

// Candidate camera-side parameters: x + (-z) * scale on the free coordinates.
template <typename T>
__global__ void k_cam_candidate(const double* ext, const double* intr, double* ext2, double* intr2, const int32_t* ext_col,
                                const int32_t* intr_col, int64_t n_ext, int64_t n_intr, const T* z, const double* scale_c,
                                double* part_step) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_ext + n_intr;
       i += (int64_t)gridDim.x * blockDim.x) {
    const bool is_e = i < n_ext;
    const int64_t j = is_e ? i : i - n_ext;
    const int32_t col = is_e ? ext_col[j] : intr_col[j];
    const double x = is_e ? ext[j] : intr[j];
    double d = 0.0;
    if (col >= 0) d = -(double)z[col] * scale_c[col];
    if (is_e) ext2[j] = x + d;
    else intr2[j] = x + d;
    acc += d * d;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    part_step[blockIdx.x] = s;
  }
}

// FP64 robustified cost 1/2 sum rho(|r|^2) at (ext, intr, pts); per-block partials.
template <int M>
__global__ void __launch_bounds__(256) k_cost(Prob P, const double* ext, const double* intr, const double* pts,
                                              double* part_cost, int* nonfinite) {
  constexpr int K = Model<M>::K;
  __shared__ double sh[8];
  double acc = 0.0;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.no; o += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = P.cam[o], g = P.icam[o], p = P.pt[o];
    double E[6], Kp[K], X[3], r[2];
#pragma unroll
    for (int i = 0; i < 6; ++i) E[i] = __ldg(&ext[6 * (int64_t)c + i]);
#pragma unroll
    for (int i = 0; i < K; ++i) Kp[i] = __ldg(&intr[K * (int64_t)g + i]);
#pragma unroll
    for (int i = 0; i < 3; ++i) X[i] = __ldg(&pts[3 * (int64_t)p + i]);
    const double2 ob = P.obs[o];
    double dJe[2][6], dJk[2][K], dJx[2][3];
    residual<M, double, false>(Kp, E, X, ob.x, ob.y, r, dJe, dJk, dJx, (double*)nullptr);
    double sr1;
    const double cst = robust<double>(P.loss_type, P.loss_a, r[0] * r[0] + r[1] * r[1], &sr1);
    if (!isfinite(cst)) atomicExch(nonfinite, 1);
    acc += cst;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    part_cost[blockIdx.x] = s;
  }
}

// Fixed-order reduction of per-block partials (deterministic).
__global__ void k_reduce3(const double* a, int na, const double* b, int nb, const double* c, int nc, const double* d,
                          int nd, double* out) {
  __shared__ double sh[4][256];
  const double* src[4] = {a, b, c, d};
  const int cnt[4] = {na, nb, nc, nd};
  for (int k = 0; k < 4; ++k) {
    double s = 0.0;
    for (int i = threadIdx.x; i < cnt[k]; i += 256) s += src[k][i];
    sh[k][threadIdx.x] = s;
  }
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

// Squared norm of the minimizer's parameter vector (see XNorm in the oracle).
__global__ void k_xnorm(const double* ext, const int32_t* ext_col, int64_t n_ext, const double* intr,
                        const uint8_t* intr_var, int k, int64_t n_intr, const double* pts, int64_t n_pts, double* part) {
  __shared__ double sh[8];
  double acc = 0.0;
  const int64_t total = n_ext + n_intr + n_pts;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    double v = 0.0;
    if (i < n_ext) {
      if (ext_col[i] >= 0) v = ext[i];
    } else if (i < n_ext + n_intr) {
      const int64_t j = i - n_ext;
      if (intr_var[j / k]) v = intr[j];
    } else {
      v = pts[i - n_ext - n_intr];
    }
    acc += v * v;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    part[blockIdx.x] = s;
  }
}

// ------------------------------------------------------------------ host driver
struct Solve {
  gbba_handle* h;
  cudaStream_t st;
  int model, k;
  int64_t nc, ni, np, no;
  int64_t n_red, n_pad;
  int precision;
  // device arrays
  double *ext, *intr, *pts, *ext2, *intr2, *pts2;
  double2* obs;
  uint32_t *cam, *icam, *pt, *pt_off;
  int32_t *ext_col, *intr_col;
  uint8_t* intr_var;
  double *cn_c, *cn_p, *g_c, *g_p, *scale_c, *scale_p, *diag_c, *diag_p;
  double* radius;
  unsigned long long* gmax_bits;
  int *flag, *nonfinite;
  void *S, *rhs, *zsol, *Linv, *Vinv, *gpv, *Wbuf, *What;
  double *part_mcc, *part_step_p, *part_step_c, *part_cost, *part_x, *scalars;
  int nb_obs, nb_pt, nb_cam, nb_x;
};

static Prob make_prob(const Solve& s, const double* ext, const double* intr, const double* pts, const gbba_options* o) {
  Prob P;
  P.ext = ext;
  P.intr = intr;
  P.pts = pts;
  P.obs = s.obs;
  P.cam = s.cam;
  P.icam = s.icam;
  P.pt = s.pt;
  P.pt_off = s.pt_off;
  P.ext_col = s.ext_col;
  P.intr_col = s.intr_col;
  P.nc = s.nc;
  P.ni = s.ni;
  P.np = s.np;
  P.no = s.no;
  P.loss_type = o ? o->loss_type : 0;
  P.loss_a = o ? o->loss_scale : 1.0;
  return P;
}

// Carve the workspace (run twice: once against a Planner for the size).
template <typename A>
static void carve(A& a, Solve& s, size_t tsize) {
  s.ext = a.template take<double>(6 * s.nc);
  s.intr = a.template take<double>(s.k * s.ni);
  s.pts = a.template take<double>(3 * s.np);
  s.ext2 = a.template take<double>(6 * s.nc);
  s.intr2 = a.template take<double>(s.k * s.ni);
  s.pts2 = a.template take<double>(3 * s.np);
  s.obs = a.template take<double2>(s.no);
  s.cam = a.template take<uint32_t>(s.no);
  s.icam = a.template take<uint32_t>(s.no);
  s.pt = a.template take<uint32_t>(s.no);
  s.pt_off = a.template take<uint32_t>(s.np + 1);
  s.ext_col = a.template take<int32_t>(6 * s.nc);
  s.intr_col = a.template take<int32_t>(s.k * s.ni);
  s.intr_var = a.template take<uint8_t>(s.ni);
  s.cn_c = a.template take<double>(s.n_red + 1);
  s.g_c = a.template take<double>(s.n_red + 1);
  s.scale_c = a.template take<double>(s.n_red + 1);
  s.diag_c = a.template take<double>(s.n_red + 1);
  s.cn_p = a.template take<double>(3 * s.np);
  s.g_p = a.template take<double>(3 * s.np);
  s.scale_p = a.template take<double>(3 * s.np);
  s.diag_p = a.template take<double>(3 * s.np);
  s.radius = a.template take<double>(1);
  s.gmax_bits = a.template take<unsigned long long>(1);
  s.flag = a.template take<int>(1);
  s.nonfinite = a.template take<int>(1);
  s.S = a.template take<char>((size_t)s.n_pad * s.n_pad * tsize);
  s.rhs = a.template take<char>((size_t)s.n_pad * tsize);
  s.zsol = a.template take<char>((size_t)s.n_pad * tsize);
  s.Linv = a.template take<char>((size_t)s.n_pad * 64 * tsize);
  s.Vinv = a.template take<char>((size_t)s.np * 6 * tsize);
  s.gpv = a.template take<char>((size_t)s.np * 3 * tsize);
  s.Wbuf = a.template take<char>((size_t)s.no * (6 + s.k) * 3 * tsize);
  s.What = a.template take<char>((size_t)s.no * (6 + s.k) * 3 * tsize);
  s.part_mcc = a.template take<double>(s.nb_pt);
  s.part_step_p = a.template take<double>(s.nb_pt);
  s.part_step_c = a.template take<double>(s.nb_cam);
  s.part_cost = a.template take<double>(s.nb_obs);
  s.part_x = a.template take<double>(s.nb_x);
  s.scalars = a.template take<double>(8);
}

static void scan_offsets(gbba_handle* h, const uint32_t* counts, uint32_t* off, int64_t n, uint32_t* tmp_chunks,
                         cudaStream_t st) {
  const int64_t nchunks = ceil_div(n, 1024);
  k_scan_chunks<<<(unsigned)nchunks, 1024, 0, st>>>(counts, off, tmp_chunks, n);
  check_launch(h);
  k_scan_carry<<<1, 32, 0, st>>>(tmp_chunks, nchunks, off + n);
  check_launch(h);
  k_scan_add<<<(unsigned)nchunks, 1024, 0, st>>>(off, tmp_chunks, n);
  check_launch(h);
}


static void copy_in(void* dst, const void* src, size_t bytes, int memory, cudaStream_t st) {
  if (bytes == 0) return;
  GBBA_CUDA(cudaMemcpyAsync(dst, src, bytes, memory == GBBA_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
}

static void copy_to_host(void* dst, const void* src, size_t bytes, int memory) {
  if (bytes == 0) return;
  if (memory == GBBA_MEMORY_HOST) std::memcpy(dst, src, bytes);
  else GBBA_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
}

static int popcount_low(uint32_t mask, int bits) {
  int n = 0;
  for (int j = 0; j < bits; ++j) n += (mask >> j) & 1u;
  return n;
}

// Upload / sort / validate a problem into the handle's workspace.  The
// caller's arrays are never modified until the final write-back.
static void setup(gbba_handle* h, const gbba_problem* P, const gbba_options* o, Solve& s) {
  s.h = h;
  s.st = h->active;
  s.model = P->camera_model;
  s.k = model_k(s.model);
  s.nc = P->num_cameras;
  s.ni = P->num_intrinsics;
  s.np = P->num_points;
  s.no = P->num_observations;
  s.precision = o->precision;
  const int64_t no = s.no, np = s.np, nc = s.nc, ni = s.ni;
  cudaStream_t st = s.st;
  std::vector<uint8_t> cc(nc, 0), ic(ni, 0);
  if (P->camera_constant) copy_to_host(cc.data(), P->camera_constant, nc, P->memory);
  if (P->intrinsic_constant) copy_to_host(ic.data(), P->intrinsic_constant, ni, P->memory);
  // Upper bound of the reduced system (blocks without observations are only
  // known after the device pass below); S is allocated for it.
  const int free_e = 6 - popcount_low(P->extrinsic_fixed_mask, 6);
  const int free_i = s.k - popcount_low(P->intrinsic_fixed_mask, s.k);
  int64_t n_max = 0;
  for (int64_t c = 0; c < nc; ++c) n_max += cc[c] ? 0 : free_e;
  for (int64_t g = 0; g < ni; ++g) n_max += ic[g] ? 0 : free_i;
  s.n_red = n_max;
  s.n_pad = ceil_div(std::max<int64_t>(n_max, 1), 64) * 64;
  const bool dense = o->linear_solver == GBBA_SOLVER_DENSE_SCHUR ||
                     (o->linear_solver == GBBA_SOLVER_AUTO && s.n_pad <= (int64_t)o->dense_schur_max_size + 64);
  GBBA_REQUIRE(dense, GBBA_ERROR_NOT_SUPPORTED, "iterative Schur solver selected but not built for this call");
  s.nb_obs = std::max(1, std::min<int>((int)ceil_div(std::max<int64_t>(no, 1), 256), h->sm_count * 8));
  s.nb_pt = (int)std::max<int64_t>(1, ceil_div(np * 32, 128));
  s.nb_cam = 64;
  s.nb_x = 64;
  const size_t tsize = s.precision == GBBA_PRECISION_FP64 ? sizeof(double) : sizeof(float);

  // one reservation for staging + solve workspace
  Planner pl;
  pl.take<double>(2 * no);
  pl.take<uint32_t>(3 * no);
  pl.take<uint32_t>(np + 1);
  pl.take<uint32_t>(np + 1);
  pl.take<uint32_t>(ceil_div(np + 1, 1024) + 1);
  pl.take<uint32_t>(no);
  pl.take<uint8_t>(nc + ni);
  pl.take<int>(4);
  Solve tmp = s;
  carve(pl, tmp, tsize);
  h->arena.reset();
  h->arena.reserve(pl.used + 4096);
  double* obs_in = h->arena.take<double>(2 * no);
  uint32_t* idx_in = h->arena.take<uint32_t>(3 * no);
  uint32_t* counts = h->arena.take<uint32_t>(np + 1);
  uint32_t* fill = h->arena.take<uint32_t>(np + 1);
  uint32_t* chunks = h->arena.take<uint32_t>(ceil_div(np + 1, 1024) + 1);
  uint32_t* perm = h->arena.take<uint32_t>(no);
  uint8_t* used = h->arena.take<uint8_t>(nc + ni);
  int* err = h->arena.take<int>(4);
  carve(h->arena, s, tsize);

  copy_in(obs_in, P->observations, sizeof(double) * 2 * no, P->memory, st);
  copy_in(idx_in, P->camera_index, sizeof(uint32_t) * no, P->memory, st);
  copy_in(idx_in + no, P->intrinsic_index, sizeof(uint32_t) * no, P->memory, st);
  copy_in(idx_in + 2 * no, P->point_index, sizeof(uint32_t) * no, P->memory, st);
  GBBA_CUDA(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (np + 1), st));
  GBBA_CUDA(cudaMemsetAsync(fill, 0, sizeof(uint32_t) * (np + 1), st));
  GBBA_CUDA(cudaMemsetAsync(used, 0, nc + ni, st));
  GBBA_CUDA(cudaMemsetAsync(err, 0, sizeof(int) * 4, st));
  const int grid = s.nb_obs;
  k_validate<<<grid, 256, 0, st>>>(idx_in, idx_in + no, idx_in + 2 * no, no, nc, ni, np, err, counts, used, used + nc);
  check_launch(h);
  int herr = 0;
  std::vector<uint8_t> hused(nc + ni);
  GBBA_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaMemcpyAsync(hused.data(), used, nc + ni, cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaStreamSynchronize(st));
  GBBA_REQUIRE(herr == 0, GBBA_ERROR_INVALID_ARGUMENT, "observation index out of range");

  // reduced column maps (ceres: constant blocks and held coordinates are not
  // columns of the Jacobian; blocks without residuals are not in the program)
  std::vector<int32_t> ecol(6 * nc, -1), icol(s.k * ni, -1);
  std::vector<uint8_t> ivar(ni, 0);
  int64_t col = 0;
  for (int64_t c = 0; c < nc; ++c) {
    if (!hused[c] || cc[c]) continue;
    for (int j = 0; j < 6; ++j)
      if (!(P->extrinsic_fixed_mask & (1u << j))) ecol[6 * c + j] = (int32_t)col++;
  }
  for (int64_t g = 0; g < ni; ++g) {
    if (!hused[nc + g] || ic[g]) continue;
    for (int j = 0; j < s.k; ++j)
      if (!(P->intrinsic_fixed_mask & (1u << j))) {
        icol[s.k * g + j] = (int32_t)col++;
        ivar[g] = 1;
      }
  }
  s.n_red = col;
  s.n_pad = ceil_div(std::max<int64_t>(col, 1), 64) * 64;

  // counting sort of observations by point (input order kept within a point)
  scan_offsets(h, counts, s.pt_off, np, chunks, st);
  k_scatter<<<grid, 256, 0, st>>>(idx_in + 2 * no, no, s.pt_off, fill, perm);
  check_launch(h);
  k_segment_sort<<<std::max(1, (int)std::min<int64_t>(ceil_div(np, 256), h->sm_count * 8)), 256, 0, st>>>(perm, s.pt_off, np);
  check_launch(h);
  k_gather<<<grid, 256, 0, st>>>(perm, no, obs_in, idx_in, idx_in + no, idx_in + 2 * no, s.obs, s.cam, s.icam, s.pt);
  check_launch(h);
  copy_in(s.ext, P->extrinsics, sizeof(double) * 6 * nc, P->memory, st);
  copy_in(s.intr, P->intrinsics, sizeof(double) * s.k * ni, P->memory, st);
  copy_in(s.pts, P->points, sizeof(double) * 3 * np, P->memory, st);
  GBBA_CUDA(cudaMemcpyAsync(s.ext_col, ecol.data(), sizeof(int32_t) * ecol.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(s.intr_col, icol.data(), sizeof(int32_t) * icol.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(s.intr_var, ivar.data(), ni, cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaStreamSynchronize(st));  // the host vectors above go out of scope
}


// ------------------------------------------------------------------ LM driver
struct Scalars {
  double mcc, step2_p, step2_c, cost;
  int flag, nonfinite;
};

template <int M, typename T>
static gbba_status run_lm(Solve& s, const gbba_options* o, gbba_summary* sum) {
  gbba_handle* h = s.h;
  cudaStream_t st = s.st;
  const double t0 = now_s();
  const int64_t n_e = 6 * s.nc, n_i = (int64_t)s.k * s.ni;
  T* S = (T*)s.S;
  T* rhs = (T*)s.rhs;
  T* z = (T*)s.zsol;
  double* pin = h->pinned;
  const int gx = s.nb_x;

  auto launch_cost = [&](const double* e, const double* i, const double* p) {
    Prob Pc = make_prob(s, e, i, p, o);
    k_cost<M><<<s.nb_obs, 256, 0, st>>>(Pc, e, i, p, s.part_cost, s.nonfinite);
    check_launch(h);
  };
  // gradient max norm and x norm at the current point; scale on first use
  auto linearize = [&](bool first, double* gmax, double* xnorm) {
    Prob P = make_prob(s, s.ext, s.intr, s.pts, o);
    GBBA_CUDA(cudaMemsetAsync(s.cn_c, 0, sizeof(double) * (s.n_red + 1), st));
    GBBA_CUDA(cudaMemsetAsync(s.g_c, 0, sizeof(double) * (s.n_red + 1), st));
    GBBA_CUDA(cudaMemsetAsync(s.cn_p, 0, sizeof(double) * 3 * s.np, st));
    GBBA_CUDA(cudaMemsetAsync(s.g_p, 0, sizeof(double) * 3 * s.np, st));
    GBBA_CUDA(cudaMemsetAsync(s.gmax_bits, 0, sizeof(unsigned long long), st));
    k_linearize<M, T><<<s.nb_obs, 256, 0, st>>>(P, s.cn_c, s.cn_p, s.g_c, s.g_p);
    check_launch(h);
    if (s.n_red > 0) {
      k_scale_diag<<<(unsigned)std::min<int64_t>(ceil_div(s.n_red, 256), 1024), 256, 0, st>>>(
          s.n_red, s.cn_c, s.g_c, s.scale_c, s.diag_c, first ? 1 : 0, o->jacobi_scaling, o->min_lm_diagonal,
          o->max_lm_diagonal, s.gmax_bits);
      check_launch(h);
    }
    k_scale_diag<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(3 * s.np, 256), 4096)), 256, 0, st>>>(
        3 * s.np, s.cn_p, s.g_p, s.scale_p, s.diag_p, first ? 1 : 0, o->jacobi_scaling, o->min_lm_diagonal,
        o->max_lm_diagonal, s.gmax_bits);
    check_launch(h);
    k_xnorm<<<gx, 256, 0, st>>>(s.ext, s.ext_col, n_e, s.intr, s.intr_var, s.k, n_i, s.pts, 3 * s.np, s.part_x);
    check_launch(h);
    k_reduce3<<<1, 256, 0, st>>>(s.part_x, gx, s.part_x, 0, s.part_x, 0, s.part_x, 0, s.scalars + 4);
    check_launch(h);
    GBBA_CUDA(cudaMemcpyAsync(pin, s.gmax_bits, sizeof(double), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaMemcpyAsync(pin + 1, s.scalars + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    unsigned long long bits;
    std::memcpy(&bits, pin, sizeof(bits));
    *gmax = __builtin_bit_cast(double, (long long)bits);
    *xnorm = std::sqrt(pin[1]);
  };

  // initial cost
  GBBA_CUDA(cudaMemsetAsync(s.nonfinite, 0, sizeof(int), st));
  launch_cost(s.ext, s.intr, s.pts);
  k_reduce3<<<1, 256, 0, st>>>(s.part_cost, s.nb_obs, s.part_cost, 0, s.part_cost, 0, s.part_cost, 0, s.scalars);
  check_launch(h);
  int nonfinite = 0;
  GBBA_CUDA(cudaMemcpyAsync(pin, s.scalars, sizeof(double), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaMemcpyAsync(&nonfinite, s.nonfinite, sizeof(int), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaStreamSynchronize(st));
  double cost = pin[0];
  sum->initial_cost = cost;
  sum->reduced_system_size = s.n_red;
  if (nonfinite || !std::isfinite(cost)) {
    sum->termination_type = GBBA_FAILURE;
    sum->usable = 0;
    sum->final_cost = cost;
    return GBBA_ERROR_NUMERICAL;
  }
  double gmax = 0, x_norm = 0;
  const double tj0 = now_s();
  linearize(true, &gmax, &x_norm);
  sum->jacobian_time_s += now_s() - tj0;

  int term = -1;
  if (gmax <= o->gradient_tolerance) term = GBBA_CONVERGENCE;
  double radius = o->initial_trust_region_radius, decrease_factor = 2.0;
  int invalid_steps = 0, iteration = 0;
  cudaEvent_t ev[6];
  for (int i = 0; i < 6; ++i) GBBA_CUDA(cudaEventCreate(&ev[i]));
  while (term < 0) {
    if (iteration >= o->max_num_iterations) {
      term = GBBA_NO_CONVERGENCE;
      break;
    }
    Prob P = make_prob(s, s.ext, s.intr, s.pts, o);
    pin[2] = radius;
    GBBA_CUDA(cudaMemcpyAsync(s.radius, pin + 2, sizeof(double), cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaMemsetAsync(s.flag, 0, sizeof(int), st));
    GBBA_CUDA(cudaMemsetAsync(s.nonfinite, 0, sizeof(int), st));
    GBBA_CUDA(cudaEventRecord(ev[0], st));
    GBBA_CUDA(cudaMemsetAsync(S, 0, sizeof(T) * s.n_pad * s.n_pad, st));
    k_schur_init<T><<<(unsigned)std::min<int64_t>(ceil_div(s.n_pad, 256), 1024), 256, 0, st>>>(S, rhs, s.n_red, s.n_pad,
                                                                                            s.diag_c, s.radius);
    check_launch(h);
    GBBA_CUDA(cudaEventRecord(ev[4], st));
    if (s.np > 0) {
      k_schur_point<M, T><<<s.nb_pt, 128, 0, st>>>(P, s.scale_c, s.scale_p, s.diag_p, s.radius, S, s.n_pad, rhs,
                                                    (T*)s.Vinv, (T*)s.gpv, (T*)s.Wbuf, (T*)s.What, s.flag);
      check_launch(h);
      ++sum->schur_kernel_launches;
    }
    GBBA_CUDA(cudaEventRecord(ev[1], st));
    const int64_t launches0 = h->launches;
    dense_cholesky_solve<T>(h, S, s.n_pad, rhs, z, (T*)s.Linv, s.flag, st);
    sum->factor_launches += (int32_t)(h->launches - launches0);
    GBBA_CUDA(cudaEventRecord(ev[5], st));
    if (s.np > 0) {
      k_backsub<M, T><<<s.nb_pt, 128, 0, st>>>(P, s.scale_c, s.scale_p, z, (T*)s.Vinv, (T*)s.gpv, s.pts2, s.part_mcc,
                                                s.part_step_p, s.flag);
      check_launch(h);
    }
    k_cam_candidate<T><<<s.nb_cam, 256, 0, st>>>(s.ext, s.intr, s.ext2, s.intr2, s.ext_col, s.intr_col, n_e, n_i, z,
                                                 s.scale_c, s.part_step_c);
    check_launch(h);
    GBBA_CUDA(cudaEventRecord(ev[2], st));
    launch_cost(s.ext2, s.intr2, s.pts2);
    k_reduce3<<<1, 256, 0, st>>>(s.part_mcc, s.np > 0 ? s.nb_pt : 0, s.part_step_p, s.np > 0 ? s.nb_pt : 0,
                                 s.part_step_c, s.nb_cam, s.part_cost, s.nb_obs, s.scalars);
    check_launch(h);
    GBBA_CUDA(cudaEventRecord(ev[3], st));
    Scalars* hs = reinterpret_cast<Scalars*>(pin + 8);
    GBBA_CUDA(cudaMemcpyAsync(hs, s.scalars, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaMemcpyAsync(&hs->flag, s.flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaMemcpyAsync(&hs->nonfinite, s.nonfinite, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    float ms_a = 0, ms_b = 0, ms_c = 0, ms_k = 0, ms_f = 0;
    cudaEventElapsedTime(&ms_a, ev[0], ev[1]);
    cudaEventElapsedTime(&ms_b, ev[1], ev[2]);
    cudaEventElapsedTime(&ms_c, ev[2], ev[3]);
    cudaEventElapsedTime(&ms_k, ev[4], ev[1]);
    cudaEventElapsedTime(&ms_f, ev[1], ev[5]);
    sum->schur_kernel_time_s += ms_k * 1e-3;
    sum->factor_time_s += ms_f * 1e-3;
    sum->jacobian_time_s += ms_a * 1e-3;
    sum->linear_solver_time_s += ms_b * 1e-3;
    sum->residual_time_s += ms_c * 1e-3;
    ++iteration;

    // TrustRegionMinimizer::Minimize step evaluation (trust_region_minimizer.cc:327-580)
    const bool solved = hs->flag == 0;
    const double mcc = hs->mcc;
    const bool valid = solved && std::isfinite(mcc) && mcc >= 0.0;
    bool success = false;
    double relative_decrease = 0.0;
    if (!valid) {
      if (++invalid_steps >= o->max_num_consecutive_invalid_steps) {
        term = GBBA_FAILURE;
        break;
      }
    } else {
      invalid_steps = 0;
      const double new_cost = (hs->nonfinite || !std::isfinite(hs->cost)) ? std::numeric_limits<double>::max() : hs->cost;
      const double step_norm = std::sqrt(hs->step2_p + hs->step2_c);
      if (step_norm <= o->parameter_tolerance * (x_norm + o->parameter_tolerance)) {
        term = GBBA_CONVERGENCE;
        break;
      }
      const double cost_change = cost - new_cost;
      if (std::fabs(cost_change) <= o->function_tolerance * cost) {
        term = GBBA_CONVERGENCE;
        break;
      }
      relative_decrease = cost_change / mcc;
      success = relative_decrease > o->min_relative_decrease;
      if (success) cost = new_cost;
    }
    if (success) {
      ++sum->num_successful_steps;
      radius = radius / std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * relative_decrease - 1.0, 3));
      radius = std::min(o->max_trust_region_radius, radius);
      decrease_factor = 2.0;
      std::swap(s.ext, s.ext2);
      std::swap(s.intr, s.intr2);
      std::swap(s.pts, s.pts2);
      const double tj = now_s();
      linearize(false, &gmax, &x_norm);
      sum->jacobian_time_s += now_s() - tj;
      if (gmax <= o->gradient_tolerance) term = GBBA_CONVERGENCE;
    } else {
      ++sum->num_unsuccessful_steps;
      radius = radius / decrease_factor;  // StepRejected and StepIsInvalid
      decrease_factor *= 2.0;
      if (radius < o->min_trust_region_radius) term = GBBA_CONVERGENCE;
    }
  }
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  sum->termination_type = term;
  sum->usable = term != GBBA_FAILURE ? 1 : 0;
  sum->final_cost = cost;
  sum->num_iterations = sum->num_successful_steps + sum->num_unsuccessful_steps;
  sum->total_time_s = now_s() - t0;
  return GBBA_SUCCESS;
}

static void copy_out(void* dst, const void* src, size_t bytes, int memory, cudaStream_t st) {
  if (bytes == 0) return;
  GBBA_CUDA(cudaMemcpyAsync(dst, src, bytes, memory == GBBA_MEMORY_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
}

// Entry used by gbba_solve: setup + LM + write-back.
gbba_status solve_impl(gbba_handle* h, const gbba_problem* P, const gbba_options* o, gbba_summary* sum) {
  const double t0 = now_s();
  if (P->num_observations == 0) {  // nothing to refine
    sum->termination_type = GBBA_CONVERGENCE;
    sum->usable = 1;
    return GBBA_SUCCESS;
  }
  Solve s{};
  setup(h, P, o, s);
  gbba_status st = GBBA_SUCCESS;
  const bool fp64 = o->precision == GBBA_PRECISION_FP64;
  switch (s.model) {
    case kPinholeF: st = fp64 ? run_lm<kPinholeF, double>(s, o, sum) : run_lm<kPinholeF, float>(s, o, sum); break;
    case kRadialK3: st = fp64 ? run_lm<kRadialK3, double>(s, o, sum) : run_lm<kRadialK3, float>(s, o, sum); break;
    default: st = fp64 ? run_lm<kBrownT2, double>(s, o, sum) : run_lm<kBrownT2, float>(s, o, sum); break;
  }
  if (st == GBBA_SUCCESS && sum->usable) {
    copy_out(P->extrinsics, s.ext, sizeof(double) * 6 * s.nc, P->memory, s.st);
    copy_out(P->intrinsics, s.intr, sizeof(double) * s.k * s.ni, P->memory, s.st);
    copy_out(P->points, s.pts, sizeof(double) * 3 * s.np, P->memory, s.st);
    GBBA_CUDA(cudaStreamSynchronize(s.st));
  }
  sum->total_time_s = now_s() - t0;
  return st;
}

}  // namespace gbba
