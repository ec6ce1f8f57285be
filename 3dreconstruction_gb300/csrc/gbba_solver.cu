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
#include <type_traits>

#include <cub/device/device_radix_sort.cuh>
#include <math_constants.h>

#include "gbba_device.cuh"
#include "gbba_internal.h"

namespace gbba {

template <typename T>
void dense_cholesky_solve(gbba_handle* h, T* S, int64_t n_pad, T* b, T* x, T* Linv_all, int* flag, cudaStream_t st);
template <typename T>
void dense_cholesky_prepare();

// Tile width of the dense factorisation, which S's size is padded to.
constexpr int64_t kDenseTile = 64;

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
  // FP64 camera poses (pose_matrix, 12 per camera) of ext, or null: the
  // mixed path evaluates its FP64 residuals from them.
  const double* pose;
  // FP32 copies of the parameters and of the Jacobi scales, or null: the
  // mixed path's FP32 Jacobian reads them instead of converting per
  // observation (conversions and FP64 products run on GB300's FP64 pipe).
  const float *ext_f, *intr_f, *pts_f, *scale_cf, *scale_pf;
  // Residual cache of the mixed path, or null: per observation r sqrt(rho')
  // and sqrt(rho') from the FP64 cost pass at these parameters (read by the
  // Schur build instead of a second FP64 residual), and where the cost pass
  // writes them.
  const float4* rc;
  float4* rc_out;
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
  double Kd[K], Xd[3];
#pragma unroll
  for (int i = 0; i < K; ++i) Kd[i] = __ldg(&P.intr[K * (int64_t)g + i]);
#pragma unroll
  for (int i = 0; i < 3; ++i) Xd[i] = __ldg(&P.pts[3 * (int64_t)p + i]);
  T Je[2][6], Jk[2][K], Jx[2][3];
  double r[2];
  double r_sr1 = -1.0;  // >= 0: r is already corrected and this is sqrt(rho') (residual cache)
  if constexpr (sizeof(T) == 8) {
    double Ed[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) Ed[i] = __ldg(&P.ext[6 * (int64_t)c + i]);
    residual<M, T, true>(Kd, Ed, Xd, ob.x, ob.y, r, Je, Jk, Jx, (T*)nullptr);
  } else {
    T Ef[6], Kf[K], Xf[3], rf[2];
    if (P.rc) {
      const float4 q = __ldg(&P.rc[o]);
      r[0] = q.x;
      r[1] = q.y;
      r_sr1 = q.z;
    } else if (P.pose) {
      residual_pose<M, double>(Kd, P.pose + 12 * (int64_t)c, Xd, ob.x, ob.y, r);
    } else {
      double Ed[6], dJe[2][6], dJk[2][K], dJx[2][3];
#pragma unroll
      for (int i = 0; i < 6; ++i) Ed[i] = __ldg(&P.ext[6 * (int64_t)c + i]);
      residual<M, double, false>(Kd, Ed, Xd, ob.x, ob.y, r, dJe, dJk, dJx, (double*)nullptr);
    }
    if (P.ext_f) {
#pragma unroll
      for (int i = 0; i < 6; ++i) Ef[i] = __ldg(&P.ext_f[6 * (int64_t)c + i]);
#pragma unroll
      for (int i = 0; i < K; ++i) Kf[i] = __ldg(&P.intr_f[K * (int64_t)g + i]);
#pragma unroll
      for (int i = 0; i < 3; ++i) Xf[i] = __ldg(&P.pts_f[3 * (int64_t)p + i]);
    } else {
#pragma unroll
      for (int i = 0; i < 6; ++i) Ef[i] = (T)__ldg(&P.ext[6 * (int64_t)c + i]);
#pragma unroll
      for (int i = 0; i < K; ++i) Kf[i] = (T)Kd[i];
#pragma unroll
      for (int i = 0; i < 3; ++i) Xf[i] = (T)Xd[i];
    }
    residual<M, T, true>(Kf, Ef, Xf, (T)ob.x, (T)ob.y, rf, Je, Jk, Jx, (T*)nullptr);
  }
  double sr1;
  if (r_sr1 >= 0.0) {
    sr1 = r_sr1;
    *cost = 0.0;  // not evaluated: the cost pass has it
    J.r[0] = r[0];
    J.r[1] = r[1];
  } else {
    *cost = robust<double>(P.loss_type, P.loss_a, r[0] * r[0] + r[1] * r[1], &sr1);
    J.r[0] = r[0] * sr1;
    J.r[1] = r[1] * sr1;
  }
  const T s = (T)sr1;
#pragma unroll
  for (int j = 0; j < 6; ++j) J.col[j] = __ldg(&P.ext_col[6 * (int64_t)c + j]);
#pragma unroll
  for (int j = 0; j < K; ++j) J.col[6 + j] = __ldg(&P.intr_col[K * (int64_t)g + j]);
#pragma unroll
  for (int j = 0; j < ObsJac<M, T>::B; ++j) {
    T sc = s;
    if (kScale) {
      if (sizeof(T) == 4 && P.scale_cf) sc = J.col[j] >= 0 ? (T)P.scale_cf[J.col[j]] * s : T(0);
      else sc = J.col[j] >= 0 ? (T)(scale_c[J.col[j]] * sr1) : T(0);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) J.Jc[i][j] = (j < 6 ? Je[i][j] : Jk[i][j - 6]) * sc;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const T sc = !kScale ? s
                 : (sizeof(T) == 4 && P.scale_pf) ? (T)P.scale_pf[3 * (int64_t)p + j] * s
                                                 : (T)(scale_p[3 * (int64_t)p + j] * sr1);
#pragma unroll
    for (int i = 0; i < 2; ++i) J.Jp[i][j] = Jx[i][j] * sc;
  }
}

// Squared column norms and gradient (unscaled, corrected) at the current x.
// Column norms and gradient of the first linearisation, summed
// deterministically in fixed point: k_linearize_max records each column's
// largest term (ordered bits of a non-negative double under atomicMax),
// k_linearize_exp turns it into a power-of-two scale per column for which a
// sum over all observations stays below 2^62, and k_linearize adds the
// scaled terms as integers (an integer sum does not depend on the order of
// the adds).  k_linearize_conv converts back.  Each sum keeps about 2^-62 n_o
// of its largest term (finer than FP64 atomics over the same terms).
template <int M, typename T>
__global__ void __launch_bounds__(256) k_linearize_max(Prob P, unsigned long long* __restrict__ mn_c,
                                                       unsigned long long* __restrict__ mn_p,
                                                       unsigned long long* __restrict__ mg_c,
                                                       unsigned long long* __restrict__ mg_p) {
  constexpr int B = ObsJac<M, T>::B;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.no; o += (int64_t)gridDim.x * blockDim.x) {
    ObsJac<M, T> J;
    double cost;
    obs_jacobian<M, T, false>(P, o, nullptr, nullptr, J, &cost);
    auto mx = [](unsigned long long* p, double v) {
      // |v| as ordered bits; a non-finite term keeps the all-ones word (the
      // sums of its column become NaN)
      const double a = fabs(v);
      atomicMax(p, isfinite(a) ? (unsigned long long)__double_as_longlong(a) : ~0ull);
    };
#pragma unroll
    for (int j = 0; j < B; ++j) {
      if (J.col[j] < 0) continue;
      const double a = J.Jc[0][j], b = J.Jc[1][j];
      mx(&mn_c[J.col[j]], a * a + b * b);
      mx(&mg_c[J.col[j]], a * J.r[0] + b * J.r[1]);
    }
    const int64_t p = P.pt[o];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double a = J.Jp[0][j], b = J.Jp[1][j];
      mx(&mn_p[3 * p + j], a * a + b * b);
      mx(&mg_p[3 * p + j], a * J.r[0] + b * J.r[1]);
    }
  }
}

// Per column: the two exponents (norm, gradient) packed into one double of
// the LM-diagonal array (free until k_scale_diag rewrites it), and the
// accumulators cleared.
__global__ void k_linearize_exp(int64_t n, double nobs, unsigned long long* __restrict__ mn,
                                unsigned long long* __restrict__ mg, double* __restrict__ exps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int en = lin_exp(mn[i], nobs), eg = lin_exp(mg[i], nobs);
    exps[i] = (double)(en + 8192) * 16384.0 + (double)(eg + 8192);
    mn[i] = 0ull;
    mg[i] = 0ull;
  }
}
__device__ __forceinline__ void lin_unpack(double packed, int& en, int& eg) {
  const int hi = (int)(packed / 16384.0);
  en = hi - 8192;
  eg = (int)(packed - (double)hi * 16384.0) - 8192;
}
template <int M, typename T>
__global__ void __launch_bounds__(256) k_linearize(Prob P, double* __restrict__ cn_c, double* __restrict__ cn_p,
                                                   double* __restrict__ g_c, double* __restrict__ g_p,
                                                   const double* __restrict__ exp_c, const double* __restrict__ exp_p) {
  constexpr int B = ObsJac<M, T>::B;
  auto add = [](double* p, double v, int k) {
    atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)lin_fx(v, k));
  };
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.no; o += (int64_t)gridDim.x * blockDim.x) {
    ObsJac<M, T> J;
    double cost;
    obs_jacobian<M, T, false>(P, o, nullptr, nullptr, J, &cost);
#pragma unroll
    for (int j = 0; j < B; ++j) {
      if (J.col[j] < 0) continue;
      const double a = J.Jc[0][j], b = J.Jc[1][j];
      int en, eg;
      lin_unpack(exp_c[J.col[j]], en, eg);
      add(&cn_c[J.col[j]], a * a + b * b, en);
      add(&g_c[J.col[j]], a * J.r[0] + b * J.r[1], eg);
    }
    const int64_t p = P.pt[o];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double a = J.Jp[0][j], b = J.Jp[1][j];
      int en, eg;
      lin_unpack(exp_p[3 * p + j], en, eg);
      add(&cn_p[3 * p + j], a * a + b * b, en);
      add(&g_p[3 * p + j], a * J.r[0] + b * J.r[1], eg);
    }
  }
}
// The fixed-point sums back to floating point (NaN for a column with a
// non-finite term).
__global__ void k_linearize_conv(int64_t n, double* __restrict__ cn, double* __restrict__ g,
                                 const double* __restrict__ exps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int en, eg;
    lin_unpack(exps[i], en, eg);
    const long long vn = __double_as_longlong(cn[i]), vg = __double_as_longlong(g[i]);
    cn[i] = en >= kFxNonFinite ? CUDART_NAN : ldexp((double)vn, -en);
    g[i] = eg >= kFxNonFinite ? CUDART_NAN : ldexp((double)vg, -eg);
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
// With fused, the camera diagonal D_c^2 / radius is added later in the same
// iteration (k_rhs_camera forms it from the current Jacobian).
template <typename T>
__global__ void k_schur_init(T* S, T* rhs, int64_t n, int64_t n_pad, const double* diag_c, const double* radius,
                             int fused) {
  const double rad = *radius;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad; i += (int64_t)gridDim.x * blockDim.x) {
    S[i * n_pad + i] = i < n ? (fused ? T(0) : (T)(diag_c[i] / rad)) : T(1);
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

// ---------------------------------------------------------------- atomic-free Schur build
// Used when every free intrinsic block belongs to a single camera (per-camera
// intrinsics, or intrinsics held): the camera-side columns of an observation
// are then owned by its camera, so S splits into camera-pair blocks.
//
// Per-observation record of 9B + 8 values (B = 6 + K):
//   [ Jc (2 x B) | W = Jc^T Jp (B x 3) | W V^-1 (B x 3) | q = Jc^T r - W V^-1 g_p (B) | Jp (2 x 3) | r (2) ]
// (scaled, corrected Jacobian blocks and residual of the current linearisation)
template <int B>
struct Rec {
  static constexpr int kJc = 0, kW = 2 * B, kWh = 5 * B, kQ = 8 * B, kJp = 9 * B, kR = 9 * B + 6, kSize = 9 * B + 8;
};
// Compact record of the iterative path (2B + 16 values), which forms no
// camera-pair products and recomputes the W products where it reads them:
//   [ Jc (2 x B) | Jp (2 x 3) | Jp V^-1 (2 x 3) | r (2) | u = r - Jp V^-1 g_p (2) ]
// (W = Jc^T Jp, W V^-1 W^T = Jc^T (Jp V^-1 Jp^T) Jc, q = Jc^T u).
template <int B>
struct RecC {
  static constexpr int kJc = 0, kJp = 2 * B, kJpV = 2 * B + 6, kR = 2 * B + 12, kU = 2 * B + 14, kSize = 2 * B + 16;
};
static_assert(Rec<12>::kSize == 9 * 12 + 8 && RecC<12>::kSize == 2 * 12 + 16, "record sizes used by the workspace planner");
// The record layout of a path: compact for the iterative solver.
template <int B, bool kCompact>
using RecOf = typename std::conditional<kCompact, RecC<B>, Rec<B>>::type;

// n (a multiple of 4) consecutive FP32 values from a 16-byte aligned address,
// in 16-byte loads issued together.
template <int N>
__device__ __forceinline__ void ld_vec4(const float* __restrict__ p, float v[N]) {
  static_assert(N % 4 == 0, "whole 16-byte pieces");
#pragma unroll
  for (int i = 0; i < N; i += 4) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p + i));
    v[i] = q.x;
    v[i + 1] = q.y;
    v[i + 2] = q.z;
    v[i + 3] = q.w;
  }
}

// (V + D_p^2 / radius)^-1 of one point by a 3x3 Cholesky; v = upper
// triangle of V (00 01 02 11 12 22).  Returns false on a non-positive pivot
// or a non-finite inverse.
template <typename T>
__device__ __forceinline__ bool point_vinv(const T v[6], const double* __restrict__ dp, double rad, T vi[6],
                                           T* pivot_ratio = nullptr) {
  const T a00 = v[0] + (T)(dp[0] / rad), a11 = v[3] + (T)(dp[1] / rad), a22 = v[5] + (T)(dp[2] / rad);
  const T l00 = sqrt(a00), l10 = v[1] / l00, l20 = v[2] / l00;
  const T d1 = a11 - l10 * l10;
  const T l11 = sqrt(d1), l21 = (v[4] - l20 * l10) / l11;
  const T d2 = a22 - l20 * l20 - l21 * l21;
  // smallest over largest squared pivot: a lower bound of 1 / cond(V)
  if (pivot_ratio) *pivot_ratio = fmin(a00, fmin(d1, d2)) / fmax(a00, fmax(d1, d2));
  const T l22 = sqrt(d2);
  const T i00 = T(1) / l00, i11 = T(1) / l11, i22 = T(1) / l22;
  const T i10 = -l10 * i00 * i11, i21 = -l21 * i11 * i22, i20 = -(l20 * i00 + l21 * i10) * i22;
  vi[0] = i00 * i00 + i10 * i10 + i20 * i20;
  vi[1] = i10 * i11 + i20 * i21;
  vi[2] = i20 * i22;
  vi[3] = i11 * i11 + i21 * i21;
  vi[4] = i21 * i22;
  vi[5] = i22 * i22;
  return a00 > T(0) && d1 > T(0) && d2 > T(0) && isfinite(vi[0]) && isfinite(vi[3]) && isfinite(vi[5]);
}

// V and g_p contributions of one observation (upper triangle of Jp^T Jp, Jp^T r).
template <int M, typename T>
__device__ __forceinline__ void point_terms(const ObsJac<M, T>& J, T v[6], T g[3]) {
  const T r0 = (T)J.r[0], r1 = (T)J.r[1];
  v[0] = J.Jp[0][0] * J.Jp[0][0] + J.Jp[1][0] * J.Jp[1][0];
  v[1] = J.Jp[0][0] * J.Jp[0][1] + J.Jp[1][0] * J.Jp[1][1];
  v[2] = J.Jp[0][0] * J.Jp[0][2] + J.Jp[1][0] * J.Jp[1][2];
  v[3] = J.Jp[0][1] * J.Jp[0][1] + J.Jp[1][1] * J.Jp[1][1];
  v[4] = J.Jp[0][1] * J.Jp[0][2] + J.Jp[1][1] * J.Jp[1][2];
  v[5] = J.Jp[0][2] * J.Jp[0][2] + J.Jp[1][2] * J.Jp[1][2];
#pragma unroll
  for (int j = 0; j < 3; ++j) g[j] = J.Jp[0][j] * r0 + J.Jp[1][j] * r1;
}

// Points are processed in groups: consecutive points whose observations fit
// one warp (at most 32 in total) share a warp, one observation per lane; a
// point with no observation or with more than 32 has a warp of its own.
// pt_grp[i] is the first point of group i (pt_grp[n_groups] = np).
constexpr int kGroupChunk = 256;  // points per thread of the greedy packing

// Greedy packing over chunks of kGroupChunk points (a chunk always starts a
// new group): with write = 0 counts the groups of each chunk into out[chunk],
// with write = 1 writes their first points at out[goff[chunk]...].
__global__ void k_pt_groups(const uint32_t* __restrict__ pt_off, int64_t np, const uint32_t* __restrict__ goff,
                            uint32_t* __restrict__ out, int write) {
  const int64_t ch = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nch = (np + kGroupChunk - 1) / kGroupChunk;
  if (ch >= nch) return;
  const int64_t p_end = min(np, (ch + 1) * kGroupChunk);
  uint32_t ng = 0, cur = 0;
  uint32_t* dst = write ? out + goff[ch] : nullptr;
  for (int64_t p = ch * kGroupChunk; p < p_end; ++p) {
    const uint32_t n = pt_off[p + 1] - pt_off[p];
    const bool alone = n == 0 || n > 32;
    if (alone || cur == 0 || cur + n > 32) {
      if (write) dst[ng] = (uint32_t)p;
      ++ng;
      cur = alone ? 33u : n;  // 33 closes the group
    } else {
      cur += n;
    }
  }
  if (!write) out[ch] = ng;
  else if (ch == nch - 1) out[goff[nch]] = (uint32_t)np;
}

// Stage 1, one warp per point group: V, V^-1, g_p and the observation records.
// The LM diagonal of a point's columns is formed here from the current
// Jacobian (D_p^2 = clamp(diag(Jp'Jp))), stored in diag_p; the point's
// gradient max norm (unscaled) goes into one of kGmaxShards slots.
constexpr int kGmaxShards = 64;
__device__ __forceinline__ void gmax_update(unsigned long long* shards, double m) {
  if (!shards) return;  // no gradient tolerance: the norm is not needed
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0)
    atomicMax(shards + (((blockIdx.x * blockDim.x + threadIdx.x) >> 5) & (kGmaxShards - 1)),
              (unsigned long long)__double_as_longlong(m));
}

template <int M, typename T, bool kFp64Inverse = false, bool kCompact = false>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 7 : 1) k_schur_point_rec(Prob P, const uint32_t* __restrict__ pt_grp, int64_t n_groups,
                                                         const double* __restrict__ scale_c,
                                                         const double* __restrict__ scale_p,
                                                         double* __restrict__ diag_p, double dmin, double dmax,
                                                         unsigned long long* __restrict__ gmax_shards,
                                                         const double* __restrict__ radius, T* __restrict__ Vinv,
                                                         T* __restrict__ gp, T* __restrict__ rec,
                                                         int* __restrict__ flag) {
  constexpr int B = ObsJac<M, T>::B;
  using R = Rec<B>;
  using RC = RecC<B>;
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= n_groups) return;
  const uint32_t p0 = pt_grp[w], p1 = pt_grp[w + 1];
  const uint32_t o0 = P.pt_off[p0], o1 = P.pt_off[p1];
  const double rad = *radius;
  if (p1 - p0 > 1 || (o1 - o0 >= 1 && o1 - o0 <= 32)) {
    // ---- packed: lane i holds observation o0 + i
    const uint32_t o = o0 + lane;
    const bool valid = o < o1;
    ObsJac<M, T> J{};
    T v[6] = {}, g[3] = {};
    uint32_t p = 0;
    int head = lane, tail = lane;
    if (valid) {
      double cost;
      obs_jacobian<M, T, true>(P, o, scale_c, scale_p, J, &cost);
      point_terms<M, T>(J, v, g);
      p = P.pt[o];
      head = (int)(P.pt_off[p] - o0);
      tail = (int)(P.pt_off[p + 1] - o0) - 1;
    }
    // segmented inclusive scan over the point's lanes, then the total from its last lane
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const bool take = lane - d >= head;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const T y = __shfl_up_sync(0xffffffffu, v[i], d);
        if (take) v[i] += y;
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const T y = __shfl_up_sync(0xffffffffu, g[i], d);
        if (take) g[i] += y;
      }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) v[i] = __shfl_sync(0xffffffffu, v[i], tail);
#pragma unroll
    for (int i = 0; i < 3; ++i) g[i] = __shfl_sync(0xffffffffu, g[i], tail);
    double gm = 0.0;
    if (gmax_shards && valid && lane == head) {
#pragma unroll
      for (int j = 0; j < 3; ++j) gm = fmax(gm, fabs((double)g[j] / scale_p[3 * (int64_t)p + j]));
    }
    gmax_update(gmax_shards, gm);
    // lanes past the group's observations stay (the record copy below is
    // the warp's); their side effects are masked
    const double dp[3] = {fmin(fmax((double)v[0], dmin), dmax), fmin(fmax((double)v[3], dmin), dmax),
                          fmin(fmax((double)v[5], dmin), dmax)};
    T vi[6], pr = T(1);
    bool ok = point_vinv<T>(v, dp, rad, vi, &pr);
    if constexpr (sizeof(T) == 4 && kFp64Inverse) {
      // FP32 pivots spanning more than 1e4: V again from an FP64 Jacobian,
      // summed and inverted in FP64 (the point's lanes; the warp's scan)
      const bool bad = valid && ok && !(pr >= T(1e-4));
      if (__any_sync(0xffffffffu, bad)) {
        double v64[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (bad) {
          ObsJac<M, double> J64;
          double c64, g64[3];
          obs_jacobian<M, double, true>(P, o, scale_c, scale_p, J64, &c64);
          point_terms<M, double>(J64, v64, g64);
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const bool take = lane - d >= head;
#pragma unroll
          for (int i = 0; i < 6; ++i) {
            const double y = __shfl_up_sync(0xffffffffu, v64[i], d);
            if (take) v64[i] += y;
          }
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) v64[i] = __shfl_sync(0xffffffffu, v64[i], tail);
        if (bad) {
          double vi64[6];
          ok = point_vinv<double>(v64, dp, rad, vi64);
#pragma unroll
          for (int i = 0; i < 6; ++i) vi[i] = (T)vi64[i];
        }
      }
    }
    if (valid && lane == head) {
      if (!ok) atomicExch(flag, 2);
#pragma unroll
      for (int i = 0; i < 6; ++i) Vinv[6 * (int64_t)p + i] = vi[i];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        gp[3 * (int64_t)p + i] = g[i];
        diag_p[3 * (int64_t)p + i] = dp[i];
      }
    }
    const T Vf[3][3] = {{vi[0], vi[1], vi[2]}, {vi[1], vi[3], vi[4]}, {vi[2], vi[4], vi[5]}};
    const T r0 = (T)J.r[0], r1 = (T)J.r[1];
    if constexpr (kCompact) {
      // [Jc Jp JpV r u] (RecC); FP32: through shared memory, one coalesced copy
      T jv[6], u[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
#pragma unroll
        for (int j = 0; j < 3; ++j) jv[3 * q + j] = J.Jp[q][0] * Vf[0][j] + J.Jp[q][1] * Vf[1][j] + J.Jp[q][2] * Vf[2][j];
      }
      u[0] = r0 - (jv[0] * g[0] + jv[1] * g[1] + jv[2] * g[2]);
      u[1] = r1 - (jv[3] * g[0] + jv[4] * g[1] + jv[5] * g[2]);
      auto put = [&](T* d) {
#pragma unroll
        for (int i = 0; i < B; ++i) {
          d[RC::kJc + i] = J.Jc[0][i];
          d[RC::kJc + B + i] = J.Jc[1][i];
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          d[RC::kJp + j] = J.Jp[0][j];
          d[RC::kJp + 3 + j] = J.Jp[1][j];
        }
#pragma unroll
        for (int j = 0; j < 6; ++j) d[RC::kJpV + j] = jv[j];
        d[RC::kR] = r0;
        d[RC::kR + 1] = r1;
        d[RC::kU] = u[0];
        d[RC::kU + 1] = u[1];
      };
      if constexpr (sizeof(T) == 4) {
        constexpr int H = RC::kSize;
        constexpr int kPitch = H % 2 == 1 ? H : H + 1;  // odd: no bank conflicts
        __shared__ float cst[4][32 * kPitch];
        float* sw0 = cst[(threadIdx.x >> 5) & 3];
        if (valid) put(sw0 + lane * kPitch);
        __syncwarp();
        const int n = (int)(o1 - o0);
        float* dst = rec + (int64_t)o0 * RC::kSize;  // the group's records are consecutive
        for (int e = lane; e < n * H; e += 32) {
          const int k = e / H;
          dst[e] = sw0[k * kPitch + (e - k * H)];
        }
        __syncwarp();
      } else {
        if (valid) put(rec + (int64_t)o * RC::kSize);
      }
      return;
    }
    T* rc = rec + (int64_t)o * R::kSize;
    if constexpr (B % 4 == 0 && sizeof(T) == 4) {
      // The group's records are consecutive: each lane writes its record
      // into shared memory in two halves, [Jc W] and [W V^-1 q Jp r], and
      // after each half the warp copies the 32 records' half out with
      // coalesced 16-byte stores.
      constexpr int H1 = 5 * B, H2 = 4 * B + 8;
      constexpr int HM = H1 > H2 ? H1 : H2;
      constexpr int kPitch = (HM / 4) % 2 == 1 ? HM : HM + 4;  // 16-byte rows, odd: no bank conflicts
      __shared__ __align__(16) float rst[4][32 * kPitch];
      float* sw0 = rst[(threadIdx.x >> 5) & 3];
      float* sw = sw0 + lane * kPitch;
      const int n = (int)(o1 - o0);
      auto copy_out = [&](int H, int off) {
        __syncwarp();
        const int per = H / 4;
        for (int u = lane; u < n * per; u += 32) {
          const int k = u / per, e = u - k * per;
          const float4 val = *reinterpret_cast<const float4*>(sw0 + k * kPitch + 4 * e);
          *reinterpret_cast<float4*>(rec + (int64_t)(o0 + k) * R::kSize + off + 4 * e) = val;
        }
        __syncwarp();
      };
      static_assert(R::kW == 2 * B && R::kWh == 5 * B && R::kQ == 8 * B && R::kJp == 9 * B, "record layout");
      if (valid) {
#pragma unroll
        for (int c4 = 0; c4 < 2 * B; c4 += 4) {
          T t4[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) t4[e] = c4 + e < B ? J.Jc[0][c4 + e] : J.Jc[1][c4 + e - B];
          st4<T>(sw + c4, t4);
        }
#pragma unroll
        for (int i0 = 0; i0 < B; i0 += 4) {
          T wc[12];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int j = 0; j < 3; ++j) wc[3 * ii + j] = J.Jc[0][i0 + ii] * J.Jp[0][j] + J.Jc[1][i0 + ii] * J.Jp[1][j];
#pragma unroll
          for (int e = 0; e < 3; ++e) st4<T>(sw + 2 * B + 3 * i0 + 4 * e, wc + 4 * e);
        }
      }
      copy_out(H1, R::kJc);
      if (valid) {
#pragma unroll
        for (int i0 = 0; i0 < B; i0 += 4) {
          T yc[12], qc[4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) {
            const int i = i0 + ii;
            T wr[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) wr[j] = J.Jc[0][i] * J.Jp[0][j] + J.Jc[1][i] * J.Jp[1][j];
#pragma unroll
            for (int j = 0; j < 3; ++j) yc[3 * ii + j] = wr[0] * Vf[0][j] + wr[1] * Vf[1][j] + wr[2] * Vf[2][j];
            qc[ii] = (J.Jc[0][i] * r0 + J.Jc[1][i] * r1) -
                     (yc[3 * ii] * g[0] + yc[3 * ii + 1] * g[1] + yc[3 * ii + 2] * g[2]);
          }
#pragma unroll
          for (int e = 0; e < 3; ++e) st4<T>(sw + 3 * i0 + 4 * e, yc + 4 * e);
          st4<T>(sw + 3 * B + i0, qc);
        }
        const T t8[8] = {J.Jp[0][0], J.Jp[0][1], J.Jp[0][2], J.Jp[1][0], J.Jp[1][1], J.Jp[1][2], r0, r1};
        st4<T>(sw + 4 * B, t8);
        st4<T>(sw + 4 * B + 4, t8 + 4);
      }
      copy_out(H2, R::kWh);
      return;
    }
    if (!valid) return;
    if constexpr (B % 4 == 0) {
      // every field starts on a 16-byte boundary: write the record in 16-byte pieces
#pragma unroll
      for (int c4 = 0; c4 < 2 * B; c4 += 4) {
        T t4[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) t4[e] = c4 + e < B ? J.Jc[0][c4 + e] : J.Jc[1][c4 + e - B];
        st4<T>(rc + R::kJc + c4, t4);
      }
#pragma unroll
      for (int i0 = 0; i0 < B; i0 += 4) {
        T wc[12], yc[12], qc[4];
#pragma unroll
        for (int ii = 0; ii < 4; ++ii) {
          const int i = i0 + ii;
#pragma unroll
          for (int j = 0; j < 3; ++j) wc[3 * ii + j] = J.Jc[0][i] * J.Jp[0][j] + J.Jc[1][i] * J.Jp[1][j];
#pragma unroll
          for (int j = 0; j < 3; ++j)
            yc[3 * ii + j] = wc[3 * ii] * Vf[0][j] + wc[3 * ii + 1] * Vf[1][j] + wc[3 * ii + 2] * Vf[2][j];
          qc[ii] = (J.Jc[0][i] * r0 + J.Jc[1][i] * r1) -
                   (yc[3 * ii] * g[0] + yc[3 * ii + 1] * g[1] + yc[3 * ii + 2] * g[2]);
        }
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          st4<T>(rc + R::kW + 3 * i0 + 4 * e, wc + 4 * e);
          st4<T>(rc + R::kWh + 3 * i0 + 4 * e, yc + 4 * e);
        }
        st4<T>(rc + R::kQ + i0, qc);
      }
      const T t8[8] = {J.Jp[0][0], J.Jp[0][1], J.Jp[0][2], J.Jp[1][0], J.Jp[1][1], J.Jp[1][2], r0, r1};
      st4<T>(rc + R::kJp, t8);
      st4<T>(rc + R::kJp + 4, t8 + 4);
      return;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      rc[R::kJp + j] = J.Jp[0][j];
      rc[R::kJp + 3 + j] = J.Jp[1][j];
    }
    rc[R::kR] = r0;
    rc[R::kR + 1] = r1;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      rc[R::kJc + i] = J.Jc[0][i];
      rc[R::kJc + B + i] = J.Jc[1][i];
      T wr[3], y[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) wr[j] = J.Jc[0][i] * J.Jp[0][j] + J.Jc[1][i] * J.Jp[1][j];
#pragma unroll
      for (int j = 0; j < 3; ++j) y[j] = wr[0] * Vf[0][j] + wr[1] * Vf[1][j] + wr[2] * Vf[2][j];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        rc[R::kW + i * 3 + j] = wr[j];
        rc[R::kWh + i * 3 + j] = y[j];
      }
      rc[R::kQ + i] = (J.Jc[0][i] * r0 + J.Jc[1][i] * r1) - (y[0] * g[0] + y[1] * g[1] + y[2] * g[2]);
    }
    return;
  }
  // ---- one point (no observation, or more than 32): lanes stride its observations
  const uint32_t p = p0;
  T v[6] = {}, g[3] = {};
  for (uint32_t o = o0 + lane; o < o1; o += 32) {
    ObsJac<M, T> J;
    double cost;
    obs_jacobian<M, T, true>(P, o, scale_c, scale_p, J, &cost);
    T dv[6], dg[3];
    point_terms<M, T>(J, dv, dg);
#pragma unroll
    for (int i = 0; i < 6; ++i) v[i] += dv[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) g[i] += dg[i];
    const T r0 = (T)J.r[0], r1 = (T)J.r[1];
    if constexpr (kCompact) {
      // Jc, Jp and r now; Jp V^-1 and u once V^-1 is known
      T* rc = rec + (int64_t)o * RC::kSize;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        rc[RC::kJp + j] = J.Jp[0][j];
        rc[RC::kJp + 3 + j] = J.Jp[1][j];
      }
      rc[RC::kR] = r0;
      rc[RC::kR + 1] = r1;
#pragma unroll
      for (int i = 0; i < B; ++i) {
        rc[RC::kJc + i] = J.Jc[0][i];
        rc[RC::kJc + B + i] = J.Jc[1][i];
      }
      continue;
    }
    T* rc = rec + (int64_t)o * R::kSize;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      rc[R::kJp + j] = J.Jp[0][j];
      rc[R::kJp + 3 + j] = J.Jp[1][j];
    }
    rc[R::kR] = r0;
    rc[R::kR + 1] = r1;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      rc[R::kJc + i] = J.Jc[0][i];
      rc[R::kJc + B + i] = J.Jc[1][i];
#pragma unroll
      for (int j = 0; j < 3; ++j) rc[R::kW + i * 3 + j] = J.Jc[0][i] * J.Jp[0][j] + J.Jc[1][i] * J.Jp[1][j];
      rc[R::kQ + i] = J.Jc[0][i] * r0 + J.Jc[1][i] * r1;
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) v[i] = warp_sum(v[i]);
#pragma unroll
  for (int i = 0; i < 3; ++i) g[i] = warp_sum(g[i]);
  double gm = 0.0;
  if (gmax_shards && lane == 0) {
#pragma unroll
    for (int j = 0; j < 3; ++j) gm = fmax(gm, fabs((double)g[j] / scale_p[3 * (int64_t)p + j]));
  }
  gmax_update(gmax_shards, gm);
  const double dp[3] = {fmin(fmax((double)v[0], dmin), dmax), fmin(fmax((double)v[3], dmin), dmax),
                        fmin(fmax((double)v[5], dmin), dmax)};
  T vi[6];
  const bool ok = point_vinv<T>(v, dp, rad, vi);
  if (lane == 0) {
    if (!ok) atomicExch(flag, 2);
#pragma unroll
    for (int i = 0; i < 6; ++i) Vinv[6 * (int64_t)p + i] = vi[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      gp[3 * (int64_t)p + i] = g[i];
      diag_p[3 * (int64_t)p + i] = dp[i];
    }
  }
  const T Vf[3][3] = {{vi[0], vi[1], vi[2]}, {vi[1], vi[3], vi[4]}, {vi[2], vi[4], vi[5]}};
  if constexpr (kCompact) {
    for (uint32_t o = o0 + lane; o < o1; o += 32) {
      T* rc = rec + (int64_t)o * RC::kSize;
      T jv[6];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
#pragma unroll
        for (int j = 0; j < 3; ++j)
          jv[3 * q + j] = rc[RC::kJp + 3 * q] * Vf[0][j] + rc[RC::kJp + 3 * q + 1] * Vf[1][j] +
                          rc[RC::kJp + 3 * q + 2] * Vf[2][j];
      }
#pragma unroll
      for (int j = 0; j < 6; ++j) rc[RC::kJpV + j] = jv[j];
      rc[RC::kU] = rc[RC::kR] - (jv[0] * g[0] + jv[1] * g[1] + jv[2] * g[2]);
      rc[RC::kU + 1] = rc[RC::kR + 1] - (jv[3] * g[0] + jv[4] * g[1] + jv[5] * g[2]);
    }
    return;
  }
  for (uint32_t o = o0 + lane; o < o1; o += 32) {
    T* rc = rec + (int64_t)o * R::kSize;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      const T w0 = rc[R::kW + i * 3], w1 = rc[R::kW + i * 3 + 1], w2 = rc[R::kW + i * 3 + 2];
      T y[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) y[j] = w0 * Vf[0][j] + w1 * Vf[1][j] + w2 * Vf[2][j];
#pragma unroll
      for (int j = 0; j < 3; ++j) rc[R::kWh + i * 3 + j] = y[j];
      rc[R::kQ + i] -= y[0] * g[0] + y[1] * g[1] + y[2] * g[2];
    }
  }
}

// Column of camera c's i-th camera-side coordinate (-1 = held).
__device__ __forceinline__ int cam_col(const int32_t* ext_col, const int32_t* intr_col, const int32_t* cam_group, int K,
                                       uint32_t c, int i) {
  if (i < 6) return ext_col[6 * (int64_t)c + i];
  const int32_t g = cam_group[c];
  return g < 0 ? -1 : intr_col[K * (int64_t)g + (i - 6)];
}

// Stage 2, one warp per work item: a chunk of at most kPairChunk observation
// pairs (a, b) of one camera-pair block (ca >= cb), reduced in order:
//   U_a [a == b]  -  (W V^-1)_a  W_b^T
// A block held by a single chunk is written once into S (lower triangle;
// entries that fall above the diagonal are written transposed); the chunks of
// a longer block (the diagonal blocks hold one pair per observation of the
// camera) write partial sums that k_pair_merge adds in chunk order.  No
// atomics: each S entry has a single writer.
constexpr int kPairChunk = 128;
struct PairItem {
  uint32_t key, begin, end;
  int32_t slot;  // -1: write S directly; else the partial-sum slot
};
struct PairMerge {
  uint32_t key, first, count;
};

template <int B, typename T>
__device__ __forceinline__ void write_block(uint32_t ca, uint32_t cb, const T* acc, int lane,
                                            const int32_t* __restrict__ ext_col, const int32_t* __restrict__ intr_col,
                                            const int32_t* __restrict__ cam_group, int K, T* __restrict__ S,
                                            int64_t ld) {
  constexpr int E = (B * B + 31) / 32;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int idx = lane + 32 * e;
    if (idx >= B * B) continue;
    const int i = idx / B, j = idx % B;
    const int ci = cam_col(ext_col, intr_col, cam_group, K, ca, i);
    const int cj = cam_col(ext_col, intr_col, cam_group, K, cb, j);
    if (ci < 0 || cj < 0) continue;
    if (ca == cb && ci < cj) continue;
    if (ci >= cj) S[(int64_t)ci * ld + cj] += acc[e];
    else S[(int64_t)cj * ld + ci] += acc[e];
  }
}

// Register tiling of one B x B camera-pair block over a warp: lane t of a
// group owns the 3x3 output tile (ti, tj) = (t / TPD, t % TPD).  When the
// block needs at most 16 tiles the warp splits into two groups of 16 lanes
// that take alternate pairs (their sums are added in group order at the end).
// Staged operands are padded so that a tile's three rows are 16-byte loads:
// W V^-1 and W as TPD groups of 12 values (3 rows x 3 + 3 padding), Jc as
// 2 rows x TPD groups of 4 values (3 + 1 padding).
template <int B>
struct PairTile {
  static constexpr int TPD = (B + 2) / 3;
  static constexpr int NT = TPD * TPD;
  static constexpr int G = NT <= 16 ? 2 : 1;
  static constexpr int LPG = NT <= 16 ? 16 : 32;
  static constexpr int WSZ = TPD * 12;
  static constexpr int JSZ = 2 * TPD * 4;
  static constexpr int PSZ = 2 * WSZ + JSZ;
  static constexpr int VALS = 8 * B;                  // staged values per pair
  static constexpr int SLOTS = (VALS + 31) / 32;       // per lane
};

template <typename T>
__device__ __forceinline__ void lds12(const T* p, T v[12]) {
#pragma unroll
  for (int q = 0; q < 3; ++q) ld4<T>(p + 4 * q, v + 4 * q);
}

template <int B, typename T, bool kKahan = false>
__global__ void __launch_bounds__(128) k_schur_pairs(const PairItem* __restrict__ items, int64_t nitems,
                                                     const unsigned long long* __restrict__ pairs,
                                                     const T* __restrict__ rec, const int32_t* __restrict__ ext_col,
                                                     const int32_t* __restrict__ intr_col,
                                                     const int32_t* __restrict__ cam_group, int K, int64_t nc,
                                                     T* __restrict__ S, int64_t ld, T* __restrict__ partial) {
  using R = Rec<B>;
  using PT = PairTile<B>;
  // Pairs per stage: small stages keep registers and shared memory low, so
  // that many warps have loads in flight (measured on the medium workload,
  // 2 pairs per stage beat 4, 8 and 16).
  constexpr int ST = 2;
  __shared__ __align__(16) T sh[4][ST * PT::PSZ];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= nitems) return;
  const PairItem it = items[w];
  T* sw = sh[warp];
  // this lane's staging slots: source offset in the a- or b-record, destination
  int src[PT::SLOTS], dst[PT::SLOTS], kind[PT::SLOTS];  // kind: 0 = a (W V^-1), 1 = b (W), 2 = a (Jc), 3 = none
#pragma unroll
  for (int u = 0; u < PT::SLOTS; ++u) {
    const int f = lane + 32 * u;
    if (f < 3 * B) {
      const int i = f / 3, k = f % 3;
      kind[u] = 0;
      src[u] = R::kWh + f;
      dst[u] = (i / 3) * 12 + (i % 3) * 3 + k;
    } else if (f < 6 * B) {
      const int g = f - 3 * B, i = g / 3, k = g % 3;
      kind[u] = 1;
      src[u] = R::kW + g;
      dst[u] = PT::WSZ + (i / 3) * 12 + (i % 3) * 3 + k;
    } else if (f < 8 * B) {
      const int g = f - 6 * B, r = g / B, i = g % B;
      kind[u] = 2;
      src[u] = R::kJc + g;
      dst[u] = 2 * PT::WSZ + r * PT::TPD * 4 + (i / 3) * 4 + i % 3;
    } else {
      kind[u] = 3;
      src[u] = 0;
      dst[u] = 0;
    }
  }
  const int grp = lane / PT::LPG, t = lane % PT::LPG;
  const bool active = grp < PT::G && t < PT::NT;
  const int ti = active ? t / PT::TPD : 0, tj = active ? t % PT::TPD : 0;
  T acc[3][3], cmp[3][3];  // cmp: Kahan compensation (kKahan)
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[r][c] = cmp[r][c] = T(0);
  auto add = [&](int r, int c, T v) {
    if constexpr (kKahan) {
      const T y = v - cmp[r][c];
      const T t = acc[r][c] + y;
      cmp[r][c] = (t - acc[r][c]) - y;
      acc[r][c] = t;
    } else {
      acc[r][c] += v;
    }
  };
  // The item's pair list (at most kPairChunk = 128 entries) is loaded once,
  // four per lane; pair q of the item is then a shuffle away.
  static_assert(kPairChunk <= 128, "pair list held in four registers per lane");
  unsigned long long pidx[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t qi = it.begin + lane + 32 * j;
    pidx[j] = qi < it.end ? pairs[qi] : 0ull;
  }
  auto pair_at = [&](uint32_t q) {  // q relative to it.begin; uniform over the warp's 16-pair stage
    const uint32_t j = q >> 5;
    const unsigned long long v = j == 0 ? pidx[0] : j == 1 ? pidx[1] : j == 2 ? pidx[2] : pidx[3];
    return __shfl_sync(0xffffffffu, v, (int)(q & 31));
  };
  // Software pipeline: the loads of stage s+1 are issued before stage s is
  // multiplied out of shared memory.
  T v[ST][PT::SLOTS];
  auto stage_load = [&](uint32_t q0) {
    const int n = (int)min((uint32_t)ST, it.end - q0);
#pragma unroll
    for (int q = 0; q < ST; ++q) {
      if (q < n) {
        const unsigned long long pr = pair_at(q0 - it.begin + q);
        const uint32_t a = (uint32_t)(pr >> 32), b = (uint32_t)(pr & 0xffffffffu);
        const T* ra = rec + (int64_t)a * R::kSize;
        const T* rb = rec + (int64_t)b * R::kSize;
#pragma unroll
        for (int u = 0; u < PT::SLOTS; ++u) {
          if (kind[u] == 0 || (kind[u] == 2 && a == b)) v[q][u] = ra[src[u]];
          else if (kind[u] == 1) v[q][u] = rb[src[u]];
        }
      }
    }
  };
  auto stage_store = [&](uint32_t q0) {
    const int n = (int)min((uint32_t)ST, it.end - q0);
#pragma unroll
    for (int q = 0; q < ST; ++q)
      if (q < n) {
#pragma unroll
        for (int u = 0; u < PT::SLOTS; ++u)
          if (kind[u] != 3) sw[q * PT::PSZ + dst[u]] = v[q][u];
      }
  };
  if (it.begin < it.end) stage_load(it.begin);
  for (uint32_t q0 = it.begin; q0 < it.end; q0 += ST) {
    const int n = (int)min((uint32_t)ST, it.end - q0);
    __syncwarp();
    stage_store(q0);
    __syncwarp();
    if (q0 + ST < it.end) stage_load(q0 + ST);
    // pair q of this stage is a diagonal pair (same observation) when bit q is set
    uint32_t same_bits = 0;
#pragma unroll
    for (int q = 0; q < ST; ++q) {
      if (q < n) {
        const unsigned long long pr = pair_at(q0 - it.begin + q);
        if ((uint32_t)(pr >> 32) == (uint32_t)(pr & 0xffffffffu)) same_bits |= 1u << q;
      }
    }
    if (active) {
      for (int q = grp; q < n; q += PT::G) {
        const T* sp = sw + q * PT::PSZ;
        T A[12], Bv[12];
        lds12<T>(sp + ti * 12, A);
        lds12<T>(sp + PT::WSZ + tj * 12, Bv);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            add(r, c, -(A[3 * r] * Bv[3 * c] + A[3 * r + 1] * Bv[3 * c + 1] + A[3 * r + 2] * Bv[3 * c + 2]));
        if (same_bits & (1u << q)) {
          T ja0[4], ja1[4], jb0[4], jb1[4];
          ld4<T>(sp + 2 * PT::WSZ + ti * 4, ja0);
          ld4<T>(sp + 2 * PT::WSZ + PT::TPD * 4 + ti * 4, ja1);
          ld4<T>(sp + 2 * PT::WSZ + tj * 4, jb0);
          ld4<T>(sp + 2 * PT::WSZ + PT::TPD * 4 + tj * 4, jb1);
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) add(r, c, ja0[r] * jb0[c] + ja1[r] * jb1[c]);
        }
      }
    }
  }
  if constexpr (kKahan) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[r][c] -= cmp[r][c];
  }
  if (PT::G == 2) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[r][c] += __shfl_down_sync(0xffffffffu, acc[r][c], 16);
  }
  if (!active || grp != 0) return;
  const uint32_t ca = (uint32_t)(it.key / nc), cb = (uint32_t)(it.key % nc);
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int i = 3 * ti + r;
    if (i >= B) continue;
    const int ci = it.slot >= 0 ? 0 : cam_col(ext_col, intr_col, cam_group, K, ca, i);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int j = 3 * tj + c;
      if (j >= B) continue;
      if (it.slot >= 0) {
        partial[(int64_t)it.slot * B * B + i * B + j] = acc[r][c];
        continue;
      }
      const int cj = cam_col(ext_col, intr_col, cam_group, K, cb, j);
      if (ci < 0 || cj < 0) continue;
      if (ca == cb && ci < cj) continue;
      if (ci >= cj) S[(int64_t)ci * ld + cj] += acc[r][c];
      else S[(int64_t)cj * ld + ci] += acc[r][c];
    }
  }
}

// Sum of a chunked block's partials in chunk order, written into S.
template <int B, typename T>
__global__ void __launch_bounds__(128) k_pair_merge(const PairMerge* __restrict__ merges, int64_t nmerges,
                                                    const T* __restrict__ partial, const int32_t* __restrict__ ext_col,
                                                    const int32_t* __restrict__ intr_col,
                                                    const int32_t* __restrict__ cam_group, int K, int64_t nc,
                                                    T* __restrict__ S, int64_t ld) {
  constexpr int E = (B * B + 31) / 32;
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= nmerges) return;
  const PairMerge m = merges[w];
  T acc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) acc[e] = T(0);
  for (uint32_t c = 0; c < m.count; ++c) {
    const T* in = partial + (int64_t)(m.first + c) * B * B;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int idx = lane + 32 * e;
      if (idx < B * B) acc[e] += in[idx];
    }
  }
  write_block<B, T>((uint32_t)(m.key / nc), (uint32_t)(m.key % nc), acc, lane, ext_col, intr_col, cam_group, K, S, ld);
}

// Stage 3, one block of 256 threads per camera, from the observation records
// of the camera (camera CSR):
//   rhs of the camera's columns = sum of q (compact records: q = Jc^T u),
//   column norms of the scaled, corrected Jacobian -> LM diagonal
//   D_c^2 = clamp(sum Jc^2), stored in diag_c and (dense) added to S's
//   diagonal as D_c^2 / radius, and the camera gradient's max norm
//   (unscaled, sum Jc r / scale) into the gradient shards.
// Thread t sums observations t, t+256, ...; the per-thread sums are reduced
// by a warp butterfly and then over the eight warps in order (a fixed order).
constexpr int kRhsThreads = 256;
template <int B, typename T, bool kCompact = false>
__global__ void __launch_bounds__(kRhsThreads) k_rhs_camera(const uint32_t* __restrict__ cam_off,
                                                            const uint32_t* __restrict__ cam_obs,
                                                            const T* __restrict__ rec,
                                                            const int32_t* __restrict__ ext_col,
                                                            const int32_t* __restrict__ intr_col,
                                                            const int32_t* __restrict__ cam_group, int K, int64_t nc,
                                                            T* __restrict__ rhs, const double* __restrict__ scale_c,
                                                            double* __restrict__ diag_c, double dmin, double dmax,
                                                            const double* __restrict__ radius, T* __restrict__ S,
                                                            int64_t ld, unsigned long long* __restrict__ gmax_shards) {
  using R = RecOf<B, kCompact>;
  __shared__ T part[3][kRhsThreads / 32][B];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t c = blockIdx.x;
  T acc[B], nrm[B], grd[B];
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = nrm[i] = grd[i] = T(0);
  if constexpr (sizeof(T) == 4 && kCompact && RecC<B>::kSize % 4 == 0) {
    // compact records, 16-byte aligned: thread t reads its observations'
    // Jc and (r, u) in 16-byte loads (q = Jc^T u)
    using RC = RecC<B>;
    static_assert((2 * B) % 4 == 0 && RC::kU == RC::kR + 2 && RC::kR % 4 == 0, "16-byte pieces");
    for (uint32_t q = cam_off[c] + threadIdx.x; q < cam_off[c + 1]; q += kRhsThreads) {
      const float* r = rec + (int64_t)cam_obs[q] * RC::kSize;
      float jc[2 * B], ru[4];
      ld_vec4<2 * B>(r + RC::kJc, jc);
      ld_vec4<4>(r + RC::kR, ru);
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T j0 = jc[i], j1 = jc[B + i];
        acc[i] += j0 * ru[2] + j1 * ru[3];
        nrm[i] += j0 * j0 + j1 * j1;
        grd[i] += j0 * ru[0] + j1 * ru[1];
      }
    }
  } else if constexpr (sizeof(T) == 4 && !kCompact && B % 4 == 0) {
    // full records, 16-byte aligned fields: thread t reads its
    // observations' Jc, q and r in 16-byte loads
    using RF = Rec<B>;
    static_assert(RF::kQ % 4 == 0 && RF::kR % 4 == 2 && RF::kSize % 4 == 0, "16-byte pieces");
    for (uint32_t q = cam_off[c] + threadIdx.x; q < cam_off[c + 1]; q += kRhsThreads) {
      const float* r = rec + (int64_t)cam_obs[q] * RF::kSize;
      float jc[2 * B], qv[B], tail[4];
      ld_vec4<2 * B>(r + RF::kJc, jc);
      ld_vec4<B>(r + RF::kQ, qv);
      ld_vec4<4>(r + RF::kR - 2, tail);  // Jp[1][1], Jp[1][2], r0, r1
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T j0 = jc[i], j1 = jc[B + i];
        acc[i] += qv[i];
        nrm[i] += j0 * j0 + j1 * j1;
        grd[i] += j0 * tail[2] + j1 * tail[3];
      }
    }
  } else if constexpr (sizeof(T) == 4) {
    // The warp takes observations 32 at a time (thread t still sums
    // observations t, t + 256, ...): it copies the 32 records' Jc, q and r
    // (3B + 2 values) into shared memory, record by record with coalesced
    // loads, and each lane reads its own there.
    // staged: Jc rows [0, 2B), then q [2B, 3B) and r (full record) or r
    // and u (compact record, q = Jc^T u formed here)
    constexpr int NV = kCompact ? 2 * B + 4 : 3 * B + 2, FW = (NV + 31) / 32;
    constexpr int kPitch = NV % 2 == 1 ? NV : NV + 1;  // odd pitch: no bank conflicts
    __shared__ float rs[kRhsThreads / 32][32 * kPitch];
    float* sw = rs[warp];
    const uint32_t q1 = cam_off[c + 1];
    for (uint32_t q0 = cam_off[c] + warp * 32; q0 < q1; q0 += kRhsThreads) {
      const uint32_t q = q0 + lane;
      const bool valid = q < q1;
      const uint32_t o = valid ? cam_obs[q] : 0u;
      const int nv = (int)min(32u, q1 - q0);
      __syncwarp();
      for (int k = 0; k < nv; ++k) {
        const T* r = rec + (int64_t)__shfl_sync(0xffffffffu, o, k) * R::kSize;
#pragma unroll
        for (int f = 0; f < FW; ++f) {
          const int j = lane + 32 * f;
          if (j < NV) {
            if constexpr (kCompact) sw[k * kPitch + j] = r[j < 2 * B ? R::kJc + j : R::kR + (j - 2 * B)];
            else sw[k * kPitch + j] = r[j < 2 * B ? R::kJc + j : j < 3 * B ? R::kQ + (j - 2 * B) : R::kR + (j - 3 * B)];
          }
        }
      }
      __syncwarp();
      if (!valid) continue;
      const float* v = sw + lane * kPitch;
      const T r0 = v[kCompact ? 2 * B : 3 * B], r1 = v[kCompact ? 2 * B + 1 : 3 * B + 1];
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T j0 = v[i], j1 = v[B + i];
        if constexpr (kCompact) acc[i] += j0 * v[2 * B + 2] + j1 * v[2 * B + 3];
        else acc[i] += v[2 * B + i];
        nrm[i] += j0 * j0 + j1 * j1;
        grd[i] += j0 * r0 + j1 * r1;
      }
    }
  } else {
    for (uint32_t q = cam_off[c] + threadIdx.x; q < cam_off[c + 1]; q += kRhsThreads) {
      const T* r = rec + (int64_t)cam_obs[q] * R::kSize;
      const T r0 = r[R::kR], r1 = r[R::kR + 1];
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const T j0 = r[R::kJc + i], j1 = r[R::kJc + B + i];
        if constexpr (kCompact) acc[i] += j0 * r[RecC<B>::kU] + j1 * r[RecC<B>::kU + 1];
        else acc[i] += r[Rec<B>::kQ + i];
        nrm[i] += j0 * j0 + j1 * j1;
        grd[i] += j0 * r0 + j1 * r1;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < B; ++i) {
    acc[i] = warp_sum(acc[i]);
    nrm[i] = warp_sum(nrm[i]);
    grd[i] = warp_sum(grd[i]);
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < B; ++i) {
      part[0][warp][i] = acc[i];
      part[1][warp][i] = nrm[i];
      part[2][warp][i] = grd[i];
    }
  }
  __syncthreads();
  if (threadIdx.x < B) {
    const int i = threadIdx.x;
    T v = T(0);
    double cn = 0.0, g = 0.0;
#pragma unroll
    for (int w = 0; w < kRhsThreads / 32; ++w) {
      v += part[0][w][i];
      cn += (double)part[1][w][i];
      g += (double)part[2][w][i];
    }
    const int ci = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, i);
    if (ci >= 0) {
      rhs[ci] = v;
      const double d = fmin(fmax(cn, dmin), dmax);
      diag_c[ci] = d;
      if (S) S[(int64_t)ci * ld + ci] += (T)(d / *radius);
      if (gmax_shards)
        atomicMax(gmax_shards + (c & (kGmaxShards - 1)),
                  (unsigned long long)__double_as_longlong(fabs(g / scale_c[ci])));
    }
  }
}

// ---------------------------------------------------------------- iterative Schur (PCG)
// Implicit Schur products and a block-Jacobi preconditioner on the camera
// blocks of S (ceres SCHUR_JACOBI, internal/ceres/schur_jacobi_preconditioner.cc;
// implicit products as in internal/ceres/implicit_schur_complement.cc:69-110):
//   S p = (U + D_c^2) p - sum_o W_o V_p(o)^-1 W_o^T p
// with W_o = Jc_o^T Jp_o formed where it is used, from the compact
// observation records (RecC).  The operator data (Jc, Jp, V^-1, U) are in
// the compute type T and the PCG vectors in FP64.  The FP64 path accumulates in FP64; the mixed path forms
// the per-observation products and their sums in FP32 (Kahan-compensated
// where a camera sums thousands of them) and widens the per-camera sums.

// Scalars of the device-resident CG loop (see k_pcg_direction and the other
// k_pcg_* kernels below).
struct PcgState {
  double rho[2];  // r.z of the iterations with even / odd number
  double Q0;      // quadratic model of the previous iteration
  double tol_r;   // |r| termination threshold (r_tolerance |b|; negative = off)
  int it;         // iteration being run (1-based); the count when done
  int done;       // nonzero: the loop has ended
  int failure;    // LINEAR_SOLVER_FAILURE (rho, beta or alpha not usable)
  int pad;
};

// Kahan (compensated) summation: s + v with the lost low part kept in c;
// the sum is s - c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// Camera diagonal blocks U_c = sum Jc^T Jc and the preconditioner block
// S_c = U_c + D_c^2 - sum (W V^-1) W^T (identity on held coordinates), into
// Mblk, which k_cam_inverse then inverts in place.  One block of kCamWarps
// (2, 4 or 8: the handle's camera_warps) warps per camera: warp w takes every
// kCamWarps-th of the camera's observations.  The warp copies an
// observation's Jc, Jp and Jp V^-1 (the first 2B + 12 values of its compact
// record) with coalesced loads into shared memory, Jc as column pairs, the
// next observation's copy in flight while it computes; its lanes take the
// lower triangle's entries, (W V^-1 W^T)_ij = Jc_i^T (Jp V^-1 Jp^T) Jc_j.
// The warps' partial blocks are added in warp order and written to both
// triangles.
template <int B, typename T, int kCamWarps>
__global__ void __launch_bounds__(kCamWarps * 32) k_cam_blocks(const uint32_t* __restrict__ cam_off,
                                                               const uint32_t* __restrict__ cam_obs,
                                                               const T* __restrict__ rec,
                                                               const int32_t* __restrict__ ext_col,
                                                               const int32_t* __restrict__ intr_col,
                                                               const int32_t* __restrict__ cam_group, int K, int64_t nc,
                                                               const double* __restrict__ diag_c,
                                                               const double* __restrict__ radius, T* __restrict__ U,
                                                               double* __restrict__ Mblk) {
  using R = RecC<B>;
  constexpr int NT = B * (B + 1) / 2;       // lower-triangle entries
  constexpr int E = (NT + 31) / 32;         // per lane
  constexpr int NV = 2 * B + 12;            // staged record values: Jc (2B), Jp (6), Jp V^-1 (6)
  constexpr int F = (NV + 31) / 32;         // per lane
  static_assert(R::kJc == 0 && R::kJp == 2 * B && R::kJpV == 2 * B + 6, "record layout: Jc, Jp, Jp V^-1 first");
  // staged layout: jc[i] = (Jc[0][i], Jc[1][i]), then Jp and Jp V^-1 as stored
  constexpr int kJ = 0, kP = 2 * B, kM = 2 * B + 12, kPc = 2 * B + 16, kStage = 4 * B + 16;
  // stage: jc pairs, Jp, Jp V^-1, then M = Jp V^-1 Jp^T (4) and the column
  // pairs P_j = M Jc_j (2B), formed once per observation
  __shared__ __align__(16) T stage[kCamWarps][kStage];
  __shared__ double part[kCamWarps][2][E * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t c = blockIdx.x;
  if (c >= nc) return;
  T* sw = stage[warp];
  // this lane's staged destinations and its entries (i >= j)
  int dst[F];
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const int v = lane + 32 * f;
    if (v < 2 * B) dst[f] = kJ + 2 * (v % B) + v / B;
    else if (v < NV) dst[f] = kP + (v - 2 * B);
    else dst[f] = -1;
  }
  int ei[E], ej[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int idx = lane + 32 * e;
    int i = 0;
    while ((i + 1) * (i + 2) / 2 <= idx) ++i;
    ei[e] = idx < NT ? i : 0;
    ej[e] = idx < NT ? idx - i * (i + 1) / 2 : 0;
  }
  // Observations in flight: two records in registers (pa, pb, used in
  // turn) and the index of the next one to load, so that neither the index
  // load nor the record load waits on the other.
  constexpr int W = kCamWarps;
  const uint32_t q0 = cam_off[c] + warp, q1 = cam_off[c + 1];
  T pa[F], pb[F];
  auto fetch = [&](uint32_t o, T(&p)[F]) {
    const T* r = rec + (int64_t)o * R::kSize;
#pragma unroll
    for (int f = 0; f < F; ++f) p[f] = dst[f] >= 0 ? r[lane + 32 * f] : T(0);
  };
  if (q0 < q1) fetch(cam_obs[q0], pa);
  if (q0 + W < q1) fetch(cam_obs[q0 + W], pb);
  uint32_t onext = q0 + 2 * W < q1 ? cam_obs[q0 + 2 * W] : 0u;
  // FP32: FP32 products and Kahan-compensated FP32 sums (GB300 runs FP64 at
  // a small fraction of the FP32 rate; a camera sums thousands of terms)
  using A = T;
  A su[E], cu[E], ss[E], cs[E];
#pragma unroll
  for (int e = 0; e < E; ++e) su[e] = cu[e] = ss[e] = cs[e] = A(0);
  // observation q from the registers p, which then take observation q + 2W
  auto step = [&](uint32_t q, T(&p)[F]) {
    __syncwarp();
#pragma unroll
    for (int f = 0; f < F; ++f)
      if (dst[f] >= 0) sw[dst[f]] = p[f];
    __syncwarp();
    if (q + 2 * W < q1) {
      fetch(onext, p);
      onext = q + 3 * W < q1 ? cam_obs[q + 3 * W] : 0u;
    }
    if (lane < 4) {
      const int a = lane >> 1, b = lane & 1;
      const T* jp = sw + kP;
      const T* jv = sw + kP + 6;
      sw[kM + lane] = jv[3 * a] * jp[3 * b] + jv[3 * a + 1] * jp[3 * b + 1] + jv[3 * a + 2] * jp[3 * b + 2];
    }
    __syncwarp();
    if (lane < B) {
      const T b0 = sw[kJ + 2 * lane], b1 = sw[kJ + 2 * lane + 1];
      sw[kPc + 2 * lane] = sw[kM] * b0 + sw[kM + 1] * b1;
      sw[kPc + 2 * lane + 1] = sw[kM + 2] * b0 + sw[kM + 3] * b1;
    }
    __syncwarp();
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (lane + 32 * e >= NT) continue;
      const int i = ei[e], j = ej[e];
      const T a0 = sw[kJ + 2 * i], a1 = sw[kJ + 2 * i + 1], b0 = sw[kJ + 2 * j], b1 = sw[kJ + 2 * j + 1];
      const A u = a0 * b0 + a1 * b1;
      const A w = a0 * sw[kPc + 2 * j] + a1 * sw[kPc + 2 * j + 1];
      if constexpr (sizeof(T) == 4) {
        kahan_add(su[e], cu[e], u);
        kahan_add(ss[e], cs[e], u - w);
      } else {
        su[e] += u;
        ss[e] += u - w;
      }
    }
  };
  for (uint32_t q = q0; q < q1; q += 2 * W) {
    step(q, pa);
    if (q + W < q1) step(q + W, pb);
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    part[warp][0][lane + 32 * e] = (double)su[e] - (double)cu[e];
    part[warp][1][lane + 32 * e] = (double)ss[e] - (double)cs[e];
  }
  __syncthreads();
  if (warp != 0) return;
  const double rad = *radius;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int idx = lane + 32 * e;
    if (idx >= NT) continue;
    double u = 0.0, v = 0.0;
#pragma unroll
    for (int w = 0; w < kCamWarps; ++w) {  // warp order: fixed
      u += part[w][0][idx];
      v += part[w][1][idx];
    }
    const int i = ei[e], j = ej[e];
    const int ci = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, i);
    const int cj = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, j);
    if (i == j && ci >= 0) v += diag_c[ci] / rad;
    if (ci < 0 || cj < 0) v = (i == j) ? 1.0 : 0.0;
    U[c * B * B + i * B + j] = U[c * B * B + j * B + i] = (T)u;
    Mblk[c * B * B + i * B + j] = Mblk[c * B * B + j * B + i] = v;
  }
}

// In place: each camera's preconditioner block (row-major B x B) replaced by
// its inverse, FP64 Cholesky and two triangular solves per column; one
// thread per camera.  A block that is not positive definite sets *flag = 4.
template <int B>
__global__ void __launch_bounds__(128) k_cam_inverse(double* __restrict__ Minv, int64_t nc, int* __restrict__ flag) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double A[B * B];
  double* Mi = Minv + c * B * B;
  for (int e = 0; e < B * B; ++e) A[e] = Mi[e];
  {
    bool ok = true;
    for (int j = 0; j < B && ok; ++j) {  // Cholesky, lower, in place
      double d = A[j * B + j];
      for (int t = 0; t < j; ++t) d -= A[j * B + t] * A[j * B + t];
      if (!(d > 0.0)) {
        ok = false;
        break;
      }
      d = sqrt(d);
      A[j * B + j] = d;
      for (int i = j + 1; i < B; ++i) {
        double v = A[i * B + j];
        for (int t = 0; t < j; ++t) v -= A[i * B + t] * A[j * B + t];
        A[i * B + j] = v / d;
      }
    }
    if (!ok) atomicExch(flag, 4);
    for (int col = 0; col < B; ++col) {  // columns of the inverse by two triangular solves
      double y[B];
      for (int i = 0; i < B; ++i) {
        double v = (i == col) ? 1.0 : 0.0;
        for (int t = 0; t < i; ++t) v -= A[i * B + t] * y[t];
        y[i] = ok ? v / A[i * B + i] : 0.0;
      }
      for (int i = B - 1; i >= 0; --i) {
        double v = y[i];
        for (int t = i + 1; t < B; ++t) v -= A[t * B + i] * y[t];
        y[i] = ok ? v / A[i * B + i] : 0.0;
      }
      for (int i = 0; i < B; ++i) Mi[i * B + col] = y[i];
    }
  }
}


// A camera's B operand values (compute type) into v: vector loads where the
// row's size allows them.
template <int B, typename T>
__device__ __forceinline__ void load_cam_row(const T* __restrict__ p, T v[B]) {
  constexpr int bytes = B * (int)sizeof(T);
  if constexpr (bytes % 16 == 0) {
    constexpr int P = 16 / (int)sizeof(T);
#pragma unroll
    for (int i = 0; i < B; i += P) {
      if constexpr (P == 4) {
        const float4 q = *reinterpret_cast<const float4*>(p + i);
        v[i] = q.x;
        v[i + 1] = q.y;
        v[i + 2] = q.z;
        v[i + 3] = q.w;
      } else {
        const double2 q = *reinterpret_cast<const double2*>(p + i);
        v[i] = q.x;
        v[i + 1] = q.y;
      }
    }
  } else if constexpr (bytes % 8 == 0 && sizeof(T) == 4) {
#pragma unroll
    for (int i = 0; i < B; i += 2) {
      const float2 q = *reinterpret_cast<const float2*>(p + i);
      v[i] = q.x;
      v[i + 1] = q.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < B; ++i) v[i] = p[i];
  }
}

// y_p = V_p^-1 sum_{o in p} W_o^T x_c(o), one warp per point group (the
// groups of k_pt_groups: a packed group holds one observation per lane, a
// group of one point is taken 32 observations at a time), W^T x formed as
// Jp^T (Jc x).  A group's compact records are consecutive: the warp copies
// their Jc and Jp (2B + 6 values each) into shared memory with coalesced
// loads, and each lane reads its own observation's there and its camera's
// operand row from xc (the operand gathered per camera by k_pcg_gather_cam).  A grid of at most a few
// waves strides over the groups, so that a launch after the solve has
// stopped costs one flag read per block.
template <int B, typename T>
__global__ void __launch_bounds__(128) k_spmv_point(const uint32_t* __restrict__ pt_off,
                                                    const uint32_t* __restrict__ pt,
                                                    const uint32_t* __restrict__ pt_grp, int64_t n_groups,
                                                    const uint32_t* __restrict__ cam,
                                                    const T* __restrict__ rec, const T* __restrict__ Vinv,
                                                    const T* __restrict__ xc, T* __restrict__ yt,
                                                    const PcgState* __restrict__ ps, int reset_period) {
  using R = RecC<B>;
  // FP32 path: FP32 operand and products and sums (a point has few
  // observations), FP32 point temporaries out
  constexpr int NW = 2 * B + 6;  // staged: Jc (2B), Jp (6)
  constexpr int kPitch = NW % 2 == 1 ? NW : NW + 1;  // odd pitch: no bank conflicts
  static_assert(R::kJc == 0 && R::kJp == 2 * B, "record layout: Jc, Jp first");
  __shared__ T wst[4][32 * kPitch];
  const int lane = threadIdx.x & 31;
  T* sw = wst[(threadIdx.x >> 5) & 3];
  if (ps->done || (reset_period > 0 && ps->it % reset_period != 0)) return;
  const int64_t nw = (gridDim.x * (int64_t)blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < n_groups; w += nw) {
    const uint32_t p0 = pt_grp[w], p1 = pt_grp[w + 1];
    const uint32_t o0 = pt_off[p0], o1 = pt_off[p1];
    T t[3] = {T(0), T(0), T(0)};
    for (uint32_t q0 = o0; q0 < o1; q0 += 32) {
      const int total = (int)min(32u, o1 - q0) * NW;
      const T* base = rec + (int64_t)q0 * R::kSize;
      __syncwarp();
      for (int t0 = 0; t0 < total; t0 += 128) {
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int e = t0 + 32 * u + lane;
          const int k = e / NW;
          if (e < total) v[u] = base[(int64_t)k * R::kSize + (e - k * NW)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int e = t0 + 32 * u + lane;
          const int k = e / NW;
          if (e < total) sw[k * kPitch + (e - k * NW)] = v[u];
        }
      }
      __syncwarp();
      const uint32_t o = q0 + lane;
      if (o < o1) {
        T xr[B];
        load_cam_row<B, T>(xc + (int64_t)cam[o] * B, xr);
        // W^T x = Jp^T (Jc x)
        const T* wr = sw + lane * kPitch;
        T f0 = T(0), f1 = T(0);
#pragma unroll
        for (int i = 0; i < B; ++i) {
          f0 += wr[i] * xr[i];
          f1 += wr[B + i] * xr[i];
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) t[j] += wr[2 * B + j] * f0 + wr[2 * B + 3 + j] * f1;
      }
    }
    uint32_t p;
    if (p1 - p0 == 1) {
#pragma unroll
      for (int j = 0; j < 3; ++j) t[j] = warp_sum(t[j]);
      p = p0;
      if (lane != 0) continue;
    } else {
      // packed: a segmented inclusive scan over each point's lanes; the
      // point's last lane holds its sum
      const uint32_t o = o0 + lane;
      const bool valid = o < o1;
      int head = lane, tail = lane;
      p = 0;
      if (valid) {
        p = pt[o];
        head = (int)(pt_off[p] - o0);
        tail = (int)(pt_off[p + 1] - o0) - 1;
      }
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const bool take = lane - d >= head;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const T u = __shfl_up_sync(0xffffffffu, t[j], d);
          if (take) t[j] += u;
        }
      }
      if (!valid || lane != tail) continue;
    }
    const T* v = Vinv + 6 * (int64_t)p;
    const T row[3][3] = {{v[0], v[1], v[2]}, {v[1], v[3], v[4]}, {v[2], v[4], v[5]}};
#pragma unroll
    for (int j = 0; j < 3; ++j) yt[3 * (int64_t)p + j] = row[j][0] * t[0] + row[j][1] * t[1] + row[j][2] * t[2];
  }
}

// out_c = (U_c + D_c^2) x_c - sum_{o in c} W_o y_p(o).  One block of
// kCamWarps warps per camera, one lane per observation; the warps' sums are
// added in warp order.  part[c] receives x_c . out_c (the partials of p.q).
template <int B, typename T, int kCamWarps>
__global__ void __launch_bounds__(kCamWarps * 32) k_spmv_camera(
    const uint32_t* __restrict__ cam_off, const uint32_t* __restrict__ cam_obs, const uint32_t* __restrict__ pt,
    const T* __restrict__ rec, const T* __restrict__ U, const int32_t* __restrict__ ext_col,
    const int32_t* __restrict__ intr_col, const int32_t* __restrict__ cam_group, int K, int64_t nc,
    const double* __restrict__ diag_c, const double* __restrict__ radius, const double* __restrict__ x,
    const double* __restrict__ y, const float* __restrict__ yf, double* __restrict__ out, double* __restrict__ part,
    const PcgState* __restrict__ ps, int reset_period) {
  using R = RecC<B>;
  __shared__ double red[kCamWarps][B];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t c = blockIdx.x;
  if (ps->done || (reset_period > 0 && ps->it % reset_period != 0)) return;
  if (c >= nc) {
    if (part && threadIdx.x == 0) part[c] = 0.0;
    return;
  }
  double acc[B];
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = 0.0;
  const uint32_t qb = cam_off[c], q1 = cam_off[c + 1];
  if constexpr (sizeof(T) == 4 && R::kSize % 4 == 0) {
    // one observation per lane, its Jc and Jp (2B + 6 values) in 16-byte
    // loads straight from its 16-byte aligned record: W y = Jc^T (Jp y).
    // FP32 products, Kahan-compensated FP32 sums per lane (a camera has
    // thousands of observations), FP64 from the lane sums on.
    constexpr int NL = (2 * B + 6 + 3) / 4 * 4;
    float sa[B], ca[B];
#pragma unroll
    for (int i = 0; i < B; ++i) sa[i] = ca[i] = 0.0f;
    for (uint32_t q = qb + warp * 32 + lane; q < q1; q += kCamWarps * 32) {
      const uint32_t o = cam_obs[q];
      float w[NL];
      ld_vec4<NL>(rec + (int64_t)o * R::kSize, w);
      const float* yp = yf + 3 * (int64_t)pt[o];
      const float y0 = yp[0], y1 = yp[1], y2 = yp[2];
      const float h0 = w[2 * B] * y0 + w[2 * B + 1] * y1 + w[2 * B + 2] * y2;
      const float h1 = w[2 * B + 3] * y0 + w[2 * B + 4] * y1 + w[2 * B + 5] * y2;
#pragma unroll
      for (int i = 0; i < B; ++i) kahan_add(sa[i], ca[i], -(w[i] * h0 + w[B + i] * h1));
    }
#pragma unroll
    for (int i = 0; i < B; ++i) acc[i] = (double)sa[i] - (double)ca[i];
  } else if constexpr (sizeof(T) == 4) {
    // The warp takes its camera's observations 32 at a time, one per lane:
    // it copies the 32 compact records' Jc and Jp (2B + 6 values each) into
    // shared memory with coalesced loads, record by record, and each lane
    // then reads its own: W y = Jc^T (Jp y).  FP32 products,
    // Kahan-compensated FP32 sums per lane (a camera has thousands of
    // observations), FP64 from the lane sums on.
    constexpr int NW = 2 * B + 6, FW = (NW + 31) / 32;
    constexpr int kPitch = NW % 2 == 1 ? NW : NW + 1;  // odd pitch: no bank conflicts
    static_assert(R::kJc == 0 && R::kJp == 2 * B, "record layout: Jc, Jp first");
    __shared__ float wst[kCamWarps][32 * kPitch];
    float* sw = wst[warp];
    float sa[B], ca[B];
#pragma unroll
    for (int i = 0; i < B; ++i) sa[i] = ca[i] = 0.0f;
    for (uint32_t q0 = qb + warp * 32; q0 < q1; q0 += kCamWarps * 32) {
      const uint32_t q = q0 + lane;
      const bool valid = q < q1;
      const uint32_t o = valid ? cam_obs[q] : 0u;
      const int nv = (int)min(32u, q1 - q0);
      __syncwarp();
      for (int k = 0; k < nv; ++k) {
        const T* r = rec + (int64_t)__shfl_sync(0xffffffffu, o, k) * R::kSize;
#pragma unroll
        for (int f = 0; f < FW; ++f) {
          const int v = lane + 32 * f;
          if (v < NW) sw[k * kPitch + v] = r[v];
        }
      }
      __syncwarp();
      if (!valid) continue;
      const float* w = sw + lane * kPitch;
      const float* yp = yf + 3 * (int64_t)pt[o];
      const float y0 = yp[0], y1 = yp[1], y2 = yp[2];
      const float h0 = w[2 * B] * y0 + w[2 * B + 1] * y1 + w[2 * B + 2] * y2;
      const float h1 = w[2 * B + 3] * y0 + w[2 * B + 4] * y1 + w[2 * B + 5] * y2;
#pragma unroll
      for (int i = 0; i < B; ++i) kahan_add(sa[i], ca[i], -(w[i] * h0 + w[B + i] * h1));
    }
#pragma unroll
    for (int i = 0; i < B; ++i) acc[i] = (double)sa[i] - (double)ca[i];
  } else {
    // FP64: one observation per lane straight from its record (the FP64
    // arithmetic bounds this path)
    for (uint32_t q = qb + warp * 32 + lane; q < q1; q += kCamWarps * 32) {
      const uint32_t o = cam_obs[q];
      const T* r = rec + (int64_t)o * R::kSize;
      const double* yp = y + 3 * (int64_t)pt[o];
      const double y0 = yp[0], y1 = yp[1], y2 = yp[2];
      const double h0 = (double)r[R::kJp] * y0 + (double)r[R::kJp + 1] * y1 + (double)r[R::kJp + 2] * y2;
      const double h1 = (double)r[R::kJp + 3] * y0 + (double)r[R::kJp + 4] * y1 + (double)r[R::kJp + 5] * y2;
#pragma unroll
      for (int i = 0; i < B; ++i) acc[i] -= (double)r[R::kJc + i] * h0 + (double)r[R::kJc + B + i] * h1;
    }
  }
#pragma unroll
  for (int i = 0; i < B; ++i) acc[i] = warp_sum(acc[i]);
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < B; ++i) red[warp][i] = acc[i];
  }
  __syncthreads();
  if (warp != 0) return;
  double xo = 0.0;  // this lane's x . out
  if (lane < B) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kCamWarps; ++w) v += red[w][lane];
    const int ci = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, lane);
    if (ci >= 0) {
      double u = diag_c[ci] / *radius * x[ci];
      for (int j = 0; j < B; ++j) {
        const int cj = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, j);
        if (cj >= 0) u += (double)U[c * B * B + lane * B + j] * x[cj];
      }
      out[ci] = v + u;
      xo = x[ci] * (v + u);
    }
  }
  if (!part) return;
  xo = warp_sum(xo);
  if (lane == 0) part[c] = xo;
}

// ---- device-resident CG (ceres ConjugateGradientsSolver::Solve,
// internal/ceres/conjugate_gradients_solver.cc:66-248): the scalars live in a
// PcgState on the device, every kernel of an iteration returns at once when
// `done` is set, and every reduction is a fixed-order sum of per-block
// partials that each consuming block repeats, so no kernel needs the host.

// Fixed-order sum over a block of 256 threads (result in every thread).
__device__ __forceinline__ double block_sum256(double v, double* sh) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < 8; ++w) t += sh[w];
  return t;
}
// Sum of n per-block partials in a fixed order (every thread of a 256-thread block).
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int n, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) v += part[i];
  return block_sum256(v, sh);
}

// The operand of an implicit product gathered per camera: B values in the
// compute type, 0 on held columns (k_spmv_point reads a camera's row as one
// contiguous vector); a no-op on the iterations where that product does not
// run.
template <int B, typename T>
__global__ void __launch_bounds__(256) k_pcg_gather_cam(const double* __restrict__ x, T* __restrict__ xc,
                                                        const int32_t* __restrict__ ext_col,
                                                        const int32_t* __restrict__ intr_col,
                                                        const int32_t* __restrict__ cam_group, int K, int64_t nc,
                                                        const PcgState* __restrict__ ps, int reset_period) {
  if (ps->done || (reset_period > 0 && ps->it % reset_period != 0)) return;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nc * B; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / B;
    const int ci = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, (int)(e - c * B));
    xc[e] = ci >= 0 ? (T)x[ci] : T(0);
  }
}

// The camera step z gathered per camera: B values, 0 on held columns (the
// back substitution reads a camera's row as one contiguous vector).
template <int B, typename T>
__global__ void __launch_bounds__(256) k_gather_cam_rows(const T* __restrict__ z, T* __restrict__ zc,
                                                         const int32_t* __restrict__ ext_col,
                                                         const int32_t* __restrict__ intr_col,
                                                         const int32_t* __restrict__ cam_group, int K, int64_t nc) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nc * B; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / B;
    const int ci = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, (int)(e - c * B));
    zc[e] = ci >= 0 ? z[ci] : T(0);
  }
}

// b = rhs (widened), x = 0, r = b; partials of |b|^2.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_init(const T* __restrict__ rhs, double* __restrict__ b,
                                                  double* __restrict__ x, double* __restrict__ r, int64_t n,
                                                  double* __restrict__ part) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)rhs[i];
    b[i] = v;
    r[i] = v;
    x[i] = 0.0;
    acc += v * v;
  }
  acc = block_sum256(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}
__global__ void __launch_bounds__(256) k_pcg_start(const double* __restrict__ part, int nb, double r_tolerance,
                                                   PcgState* __restrict__ ps) {
  __shared__ double sh[8];
  const double bb = sum_partials(part, nb, sh);
  if (threadIdx.x == 0) {
    ps->rho[0] = ps->rho[1] = 1.0;
    ps->Q0 = 0.0;  // x = 0
    ps->tol_r = r_tolerance * sqrt(bb);
    ps->it = 1;
    ps->failure = 0;
    ps->done = bb > 0.0 ? 0 : 1;  // |b| = 0: x = 0 is the solution
  }
}

// z = M r (block-Jacobi) and partials of r.z; one thread per camera.
template <int B>
__global__ void __launch_bounds__(256) k_pcg_precond(const double* __restrict__ Minv, const int32_t* __restrict__ ext_col,
                                                     const int32_t* __restrict__ intr_col,
                                                     const int32_t* __restrict__ cam_group, int K, int64_t nc,
                                                     const double* __restrict__ r, double* __restrict__ z,
                                                     double* __restrict__ part, const PcgState* __restrict__ ps) {
  __shared__ double sh[8];
  if (ps->done) return;
  double acc = 0.0;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c < nc) {
    int col[B];
    double rv[B];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      col[i] = cam_col(ext_col, intr_col, cam_group, K, (uint32_t)c, i);
      rv[i] = col[i] >= 0 ? r[col[i]] : 0.0;
    }
    const double* Mi = Minv + c * B * B;
#pragma unroll
    for (int i = 0; i < B; ++i) {
      if (col[i] < 0) continue;
      double v = 0.0;
#pragma unroll
      for (int j = 0; j < B; ++j) v += Mi[i * B + j] * rv[j];
      z[col[i]] = v;
      acc += rv[i] * v;
    }
  }
  acc = block_sum256(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// rho = r.z; p = z (first iteration) or z + beta p.
__global__ void __launch_bounds__(256) k_pcg_direction(int64_t n, const double* __restrict__ z, double* __restrict__ p,
                                                       const double* __restrict__ part, int nb,
                                                       PcgState* __restrict__ ps) {
  __shared__ double sh[8];
  if (ps->done) return;
  const double rho = sum_partials(part, nb, sh);
  const int it = ps->it;
  const double last = ps->rho[(it - 1) & 1];
  const double beta = it > 1 ? rho / last : 0.0;
  const bool fail = rho == 0.0 || !isfinite(rho) || (it > 1 && (beta == 0.0 || !isfinite(beta)));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (fail) {
      ps->failure = 1;
      ps->done = 1;
    } else {
      ps->rho[it & 1] = rho;
    }
  }
  if (fail) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = it > 1 ? z[i] + beta * p[i] : z[i];
}

// alpha = rho / p.q; x += alpha p; r -= alpha q (except on residual-reset
// iterations, whose r is recomputed as b - S x).
__global__ void __launch_bounds__(256) k_pcg_step(int64_t n, double* __restrict__ x, double* __restrict__ r,
                                                  const double* __restrict__ p, const double* __restrict__ q,
                                                  const double* __restrict__ part, int nb, int period,
                                                  PcgState* __restrict__ ps) {
  __shared__ double sh[8];
  if (ps->done) return;
  const double pq = sum_partials(part, nb, sh);
  const int it = ps->it;
  const double alpha = ps->rho[it & 1] / pq;
  const bool indefinite = pq <= 0.0 || isinf(pq);
  const bool stop = indefinite || isinf(alpha);
  if (blockIdx.x == 0 && threadIdx.x == 0 && stop) {
    ps->failure = indefinite ? 0 : 1;  // indefinite: no more progress can be made (not a failure)
    ps->done = 1;
  }
  if (stop) return;
  const bool reset = it % period == 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    if (!reset) r[i] -= alpha * q[i];
  }
}

// Residual-reset iterations: r = b - q (q = S x).
__global__ void __launch_bounds__(256) k_pcg_reset(int64_t n, double* __restrict__ r, const double* __restrict__ b,
                                                   const double* __restrict__ q, int period,
                                                   const PcgState* __restrict__ ps) {
  if (ps->done || ps->it % period != 0) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - q[i];
}

// Partials of x.(b + r) (the quadratic model) and r.r.
__global__ void __launch_bounds__(256) k_pcg_model(int64_t n, const double* __restrict__ x, const double* __restrict__ b,
                                                   const double* __restrict__ r, double* __restrict__ part,
                                                   const PcgState* __restrict__ ps) {
  __shared__ double sh[8];
  if (ps->done) return;
  double q = 0.0, rr = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    q += x[i] * (b[i] + r[i]);
    rr += r[i] * r[i];
  }
  q = block_sum256(q, sh);
  rr = block_sum256(rr, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = q;
    part[gridDim.x + blockIdx.x] = rr;
  }
}

// Terminations of the iteration: zeta = it (Q1 - Q0) / Q1 < eta (Nash's
// truncated-Newton rule), |r| <= tol_r, or the iteration limit.
__global__ void __launch_bounds__(256) k_pcg_terminate(const double* __restrict__ part, int nb, double eta,
                                                       int max_iterations, PcgState* __restrict__ ps) {
  __shared__ double sh[8];
  if (ps->done) return;
  const double Q1 = -sum_partials(part, nb, sh);
  const double rr = sum_partials(part + nb, nb, sh);
  if (threadIdx.x == 0) {
    const int it = ps->it;
    const double zeta = it * (Q1 - ps->Q0) / Q1;
    if (zeta < eta) {
      ps->done = 1;
    } else {
      ps->Q0 = Q1;
      if (sqrt(rr) <= ps->tol_r || it >= max_iterations) ps->done = 1;
      else ps->it = it + 1;
    }
  }
}

template <typename T, typename U2>
__global__ void k_convert(const T* a, U2* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (U2)a[i];
}

// ---------------------------------------------------------------- pair-list setup kernels
// Per point: number of ordered observation pairs (a, b) with cam(a) >= cam(b).
__global__ void k_pair_count(const uint32_t* pt_off, const uint32_t* cam, int64_t np, uint32_t* cnt) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    uint32_t n = 0;
    for (uint32_t a = pt_off[p]; a < pt_off[p + 1]; ++a)
      for (uint32_t b = pt_off[p]; b < pt_off[p + 1]; ++b) n += cam[a] >= cam[b];
    cnt[p] = n;
  }
}
__global__ void k_pair_write(const uint32_t* pt_off, const uint32_t* cam, int64_t np, int64_t nc, const uint32_t* pair_off,
                             unsigned long long* pairs, uint32_t* keys, uint32_t* hist) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    uint32_t w = pair_off[p];
    for (uint32_t a = pt_off[p]; a < pt_off[p + 1]; ++a)
      for (uint32_t b = pt_off[p]; b < pt_off[p + 1]; ++b)
        if (cam[a] >= cam[b]) {
          const uint32_t key = (uint32_t)(cam[a] * (uint64_t)nc + cam[b]);
          pairs[w] = ((unsigned long long)a << 32) | b;
          keys[w] = key;
          atomicAdd(&hist[key], 1u);
          ++w;
        }
  }
}
__global__ void k_bucket_scatter64(const unsigned long long* in, const uint32_t* keys, int64_t n, const uint32_t* off,
                                   uint32_t* fill, unsigned long long* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t k = keys[i];
    out[off[k] + atomicAdd(&fill[k], 1u)] = in[i];
  }
}
__global__ void k_segment_sort64(unsigned long long* v, const uint32_t* off, int64_t nseg) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nseg; s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = off[s], e = off[s + 1];
    for (uint32_t i = b + 1; i < e; ++i) {
      const unsigned long long x = v[i];
      uint32_t j = i;
      while (j > b && v[j - 1] > x) {
        v[j] = v[j - 1];
        --j;
      }
      v[j] = x;
    }
  }
}
__global__ void k_nonempty(const uint32_t* off, int64_t nkeys, uint32_t* list, uint32_t* count) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nkeys; k += (int64_t)gridDim.x * blockDim.x)
    if (off[k + 1] > off[k]) list[atomicAdd(count, 1u)] = (uint32_t)k;
}
__global__ void k_iota(uint32_t* v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}
static int key_bits(uint64_t max_key) {
  int b = 1;
  while (b < 32 && (1ull << b) <= max_key) ++b;
  return b;
}
// Camera -> intrinsic group map and the "free intrinsic blocks are private" check.
__global__ void k_cam_groups(const uint32_t* cam, const uint32_t* icam, int64_t no, const uint8_t* intr_var,
                             int32_t* cam_group, uint32_t* group_cam, int* conflict, uint32_t* cam_hist) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < no; o += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cam[o], g = icam[o];
    const int32_t prev = atomicCAS(&cam_group[c], -1, (int32_t)g);
    if (prev != -1 && prev != (int32_t)g) atomicExch(conflict, 1);
    if (intr_var[g]) {
      const uint32_t pc = atomicCAS(&group_cam[g], 0xffffffffu, c);
      if (pc != 0xffffffffu && pc != c) atomicExch(conflict, 1);
    }
    atomicAdd(&cam_hist[c], 1u);
  }
}

// Back substitution from the observation records (no projection is
// recomputed): one warp per point group (k_pt_groups),
//   y_p = V^-1 (g_p - sum E'F z), step = -(z, y), m = J step,
//   model_cost_change += -m.(r + m/2), candidate points.
// z is read per camera (zc: B values per camera, k_gather_cam_rows).  A
// packed group's records are consecutive: the warp copies their Jc, Jp and r
// (2B + 8 values each) into shared memory with coalesced loads, and each lane
// reads its own there.
template <int B, typename T, bool kCompact = false>
__global__ void __launch_bounds__(128) k_backsub_rec(const uint32_t* __restrict__ pt_off, const uint32_t* __restrict__ pt,
                                                     const uint32_t* __restrict__ pt_grp, int64_t n_groups,
                                                     const uint32_t* __restrict__ cam,
                                                     const T* __restrict__ rec, const T* __restrict__ zc,
                                                     const T* __restrict__ Vinv, const T* __restrict__ gp,
                                                     const double* __restrict__ scale_p, const double* __restrict__ pts,
                                                     double* __restrict__ pts_new, double* __restrict__ part_mcc,
                                                     double* __restrict__ part_step, int* __restrict__ flag) {
  using R = RecOf<B, kCompact>;
  // staged values: Jc (2B), Jp (6), r (2)
  constexpr int NV = 2 * B + 8, kPitch = NV + 1;  // odd pitch: no bank conflicts
  __shared__ T rst[4][32 * kPitch];
  __shared__ double smcc[4], sstep[4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  double mcc = 0.0, stp = 0.0;
  // one observation's values: Jc rows, Jp rows and r
  struct View {
    const T* jc;
    const T* jp;
    const T* r;
  };
  // F z of one observation: the camera block's part of J step
  auto fz = [&](const View& v, uint32_t c, T& f0, T& f1) {
    T zr[B];
    load_cam_row<B, T>(zc + (int64_t)c * B, zr);
    f0 = T(0);
    f1 = T(0);
#pragma unroll
    for (int i = 0; i < B; ++i) {
      f0 += v.jc[i] * zr[i];
      f1 += v.jc[B + i] * zr[i];
    }
  };
  // model cost change of one observation from its F z, m = -(F z + E y): m
  // in the compute type (the Jacobian's own precision), -m.(r + m/2) in FP64
  auto obs_mcc = [&](const View& v, T f0, T f1, const T y[3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      f0 += v.jp[j] * y[j];
      f1 += v.jp[3 + j] * y[j];
    }
    const double m0 = -(double)f0, m1 = -(double)f1;
    const double r0 = (double)v.r[0], r1 = (double)v.r[1];
    return -(m0 * (r0 + m0 / 2.0) + m1 * (r1 + m1 / 2.0));
  };
  auto rec_view = [&](uint32_t o) -> View {
    const T* r = rec + (int64_t)o * R::kSize;
    return {r + R::kJc, r + R::kJp, r + R::kR};
  };
  // y_p = V^-1 (g_p - E^T F z) and the candidate point
  auto point_step = [&](uint32_t p, const T t[3], T y[3]) {
    const T* vi = Vinv + 6 * (int64_t)p;
    const T q0 = gp[3 * (int64_t)p] - t[0], q1 = gp[3 * (int64_t)p + 1] - t[1], q2 = gp[3 * (int64_t)p + 2] - t[2];
    y[0] = vi[0] * q0 + vi[1] * q1 + vi[2] * q2;
    y[1] = vi[1] * q0 + vi[3] * q1 + vi[4] * q2;
    y[2] = vi[2] * q0 + vi[4] * q1 + vi[5] * q2;
  };
  if (w < n_groups) {
    const uint32_t p0 = pt_grp[w], p1 = pt_grp[w + 1];
    const uint32_t o0 = pt_off[p0], o1 = pt_off[p1];
    if (p1 - p0 > 1 || (o1 - o0 >= 1 && o1 - o0 <= 32)) {
      // packed: lane i holds observation o0 + i
      T* sr = rst[warp];
      const int total = (int)(o1 - o0) * NV;
      const T* base = rec + (int64_t)o0 * R::kSize;
      for (int e0 = 0; e0 < total; e0 += 128) {
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int e = e0 + 32 * u + lane;
          const int k = e / NV, j = e - k * NV;
          if (e < total)
            v[u] = base[(int64_t)k * R::kSize +
                        (j < 2 * B ? R::kJc + j : j < 2 * B + 6 ? R::kJp + (j - 2 * B) : R::kR + (j - 2 * B - 6))];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int e = e0 + 32 * u + lane;
          const int k = e / NV, j = e - k * NV;
          if (e < total) sr[k * kPitch + j] = v[u];
        }
      }
      __syncwarp();
      const uint32_t o = o0 + lane;
      const bool valid = o < o1;
      const View vw{sr + lane * kPitch, sr + lane * kPitch + 2 * B, sr + lane * kPitch + 2 * B + 6};
      T t[3] = {T(0), T(0), T(0)};
      T f0 = T(0), f1 = T(0);
      uint32_t p = 0;
      int head = lane, tail = lane;
      if (valid) {
        p = pt[o];
        head = (int)(pt_off[p] - o0);
        tail = (int)(pt_off[p + 1] - o0) - 1;
        fz(vw, cam[o], f0, f1);
#pragma unroll
        for (int j = 0; j < 3; ++j) t[j] = vw.jp[j] * f0 + vw.jp[3 + j] * f1;
      }
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const bool take = lane - d >= head;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const T y = __shfl_up_sync(0xffffffffu, t[j], d);
          if (take) t[j] += y;
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) t[j] = __shfl_sync(0xffffffffu, t[j], tail);
      if (valid) {
        T y[3];
        point_step(p, t, y);
        mcc = obs_mcc(vw, f0, f1, y);
        if (lane == head) {
          if (!isfinite(y[0]) || !isfinite(y[1]) || !isfinite(y[2])) atomicExch(flag, 3);
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const double d = -(double)y[j] * scale_p[3 * (int64_t)p + j];
            pts_new[3 * (int64_t)p + j] = pts[3 * (int64_t)p + j] + d;
            stp += d * d;
          }
        }
      }
    } else {
      // one point (no observation, or more than 32)
      const uint32_t p = p0;
      T t[3] = {T(0), T(0), T(0)};
      for (uint32_t o = o0 + lane; o < o1; o += 32) {
        const View vw = rec_view(o);
        T f0, f1;
        fz(vw, cam[o], f0, f1);
#pragma unroll
        for (int j = 0; j < 3; ++j) t[j] += vw.jp[j] * f0 + vw.jp[3 + j] * f1;
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) t[j] = warp_sum(t[j]);
      T y[3];
      point_step(p, t, y);
      if (!isfinite(y[0]) || !isfinite(y[1]) || !isfinite(y[2])) {
        if (lane == 0) atomicExch(flag, 3);
      }
      for (uint32_t o = o0 + lane; o < o1; o += 32) {
        const View vw = rec_view(o);
        T f0, f1;
        fz(vw, cam[o], f0, f1);
        mcc += obs_mcc(vw, f0, f1, y);
      }
      if (lane < 3) {
        const double d = -(double)y[lane] * scale_p[3 * (int64_t)p + lane];
        pts_new[3 * (int64_t)p + lane] = pts[3 * (int64_t)p + lane] + d;
        stp = d * d;
      }
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

// FP64 camera poses of ext (one thread per camera).
__global__ void k_cam_pose(const double* __restrict__ ext, int64_t nc, double* __restrict__ pose) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double E[6], q[12];
#pragma unroll
  for (int i = 0; i < 6; ++i) E[i] = ext[6 * c + i];
  pose_matrix<double>(E, q);
#pragma unroll
  for (int i = 0; i < 12; ++i) pose[12 * c + i] = q[i];
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
    if (P.pose) {
      residual_pose<M, double>(Kp, P.pose + 12 * (int64_t)c, X, ob.x, ob.y, r);
    } else {
      double dJe[2][6], dJk[2][K], dJx[2][3];
      residual<M, double, false>(Kp, E, X, ob.x, ob.y, r, dJe, dJk, dJx, (double*)nullptr);
    }
    double sr1;
    const double cst = robust<double>(P.loss_type, P.loss_a, r[0] * r[0] + r[1] * r[1], &sr1);
    if (!isfinite(cst)) atomicExch(nonfinite, 1);
    if (P.rc_out) P.rc_out[o] = make_float4((float)(r[0] * sr1), (float)(r[1] * sr1), (float)sr1, 0.0f);
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
  double *pose = nullptr, *pose2 = nullptr;  // FP64 poses of ext / ext2 (mixed path)
  float *ext_f = nullptr, *intr_f = nullptr, *pts_f = nullptr;  // FP32 copies of ext, intr, pts (mixed path)
  float4* rcache = nullptr;  // mixed path: residual cache, [2][no] (current parameters, candidate)
  float* pcg_yf = nullptr;  // mixed path: FP32 point temporaries of the implicit product
  char* pcg_xc = nullptr;   // the implicit product's operand per camera (B values, compute type)
  char* zc = nullptr;       // the camera step per camera (B values, compute type; back substitution)
  float *scale_cf = nullptr, *scale_pf = nullptr;               // FP32 copies of the Jacobi scales
  uint32_t *pt_grp = nullptr, *pgrp_cnt = nullptr, *pgrp_off = nullptr;  // point groups (k_pt_groups)
  int64_t n_pgrp = 0;
  int nb_pgrp = 1;  // blocks of the per-group kernels (4 groups per block)
  double2* obs;
  uint32_t *cam, *icam, *pt, *pt_off;
  int32_t *ext_col, *intr_col;
  uint8_t* intr_var;
  double *cn_c, *cn_p, *g_c, *g_p, *scale_c, *scale_p, *diag_c, *diag_p;
  double* radius;
  unsigned long long* gmax_bits;
  unsigned long long* gmax_shards;  // gradient max norm of the fused linearisation (kGmaxShards slots)
  int *flag, *nonfinite;
  void *S, *rhs, *zsol, *Linv, *Vinv, *gpv, *Wbuf, *What;
  double *part_mcc, *part_step_p, *part_step_c, *part_cost, *part_x, *scalars;
  int nb_obs, nb_pt, nb_cam, nb_x;
  // atomic-free Schur build (pair list in the handle's pair arena)
  bool pair_path = false;
  int64_t n_blocks = 0;  // work items of the pair kernel
  int64_t n_merges = 0;
  void* pair_items = nullptr;
  void* pair_merges = nullptr;
  void* pair_partial = nullptr;
  uint32_t *blocks = nullptr, *blk_off = nullptr, *cam_off = nullptr, *cam_obs = nullptr;
  unsigned long long* pairs = nullptr;
  int32_t* cam_group = nullptr;
  void* rec = nullptr;
  bool dense = true;
  int schur_build = GBBA_SCHUR_BUILD_AUTO;  // gbba_options::schur_build
  double t_origin = 0.0;                     // start of the gbba_solve call (trace times)
  // iterative Schur (PCG) state
  double *pcg_x = nullptr, *pcg_r = nullptr, *pcg_z = nullptr, *pcg_p = nullptr, *pcg_q = nullptr, *pcg_b = nullptr;
  double *pcg_y = nullptr, *pcg_minv = nullptr, *pcg_part = nullptr;
  int64_t pcg_part_n = 0;  // per-block partials of one reduction (two arrays of this size)
  PcgState* pcg_state = nullptr;
  cudaGraphExec_t pcg_graph = nullptr;  // one chunk of CG iterations
  int64_t pcg_chunk_launches = 0;
  void* pcg_u = nullptr;
  int nb_pcg = 0;
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
  P.pose = nullptr;
  P.ext_f = P.intr_f = P.pts_f = P.scale_cf = P.scale_pf = nullptr;
  P.rc = nullptr;
  P.rc_out = nullptr;
  return P;
}

// Carve the workspace (run twice: once against a Planner for the size).
template <typename A>
static void carve(A& a, Solve& s, size_t tsize) {
  s.ext = a.template take<double>(6 * s.nc);
  s.intr = a.template take<double>(s.k * s.ni);
  s.pts = a.template take<double>(3 * s.np);
  s.ext2 = a.template take<double>(6 * s.nc);
  s.pose = a.template take<double>(12 * s.nc);
  s.pose2 = a.template take<double>(12 * s.nc);
  s.ext_f = a.template take<float>(6 * s.nc);
  s.intr_f = a.template take<float>((int64_t)s.k * s.ni);
  s.pts_f = a.template take<float>(3 * s.np);
  s.scale_cf = a.template take<float>(s.n_red + 1);
  s.scale_pf = a.template take<float>(3 * s.np);
  s.rcache = a.template take<float4>(tsize == 4 ? 2 * s.no : 0);
  if (tsize != 4) s.rcache = nullptr;
  s.intr2 = a.template take<double>(s.k * s.ni);
  s.pts2 = a.template take<double>(3 * s.np);
  s.obs = a.template take<double2>(s.no);
  s.cam = a.template take<uint32_t>(s.no);
  s.icam = a.template take<uint32_t>(s.no);
  s.pt = a.template take<uint32_t>(s.no);
  s.pt_off = a.template take<uint32_t>(s.np + 1);
  s.pt_grp = a.template take<uint32_t>(s.np + 1);
  s.pgrp_cnt = a.template take<uint32_t>(ceil_div(s.np, kGroupChunk) + 1);
  s.pgrp_off = a.template take<uint32_t>(ceil_div(s.np, kGroupChunk) + 1);
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
  s.gmax_shards = a.template take<unsigned long long>(kGmaxShards);
  s.flag = a.template take<int>(1);
  s.nonfinite = a.template take<int>(1);
  const int64_t n_s = s.dense ? s.n_pad : 0;
  s.S = a.template take<char>((size_t)n_s * n_s * tsize);
  s.rhs = a.template take<char>((size_t)s.n_pad * tsize);
  s.zsol = a.template take<char>((size_t)s.n_pad * tsize);
  s.Linv = a.template take<char>((size_t)n_s * kDenseTile * tsize);
  s.Vinv = a.template take<char>((size_t)s.np * 6 * tsize);
  s.gpv = a.template take<char>((size_t)s.np * 3 * tsize);
  s.part_mcc = a.template take<double>(s.nb_pt);
  s.part_step_p = a.template take<double>(s.nb_pt);
  s.part_step_c = a.template take<double>(s.nb_cam);
  s.part_cost = a.template take<double>(s.nb_obs);
  s.part_x = a.template take<double>(s.nb_x);
  s.scalars = a.template take<double>(8);
}

void scan_offsets(gbba_handle* h, const uint32_t* counts, uint32_t* off, int64_t n, uint32_t* tmp_chunks,
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

static void setup_pairs(gbba_handle* h, Solve& s, size_t tsize);
static void setup_atomic_path(gbba_handle* h, Solve& s, size_t tsize);

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
  s.schur_build = o->schur_build;
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
  s.n_pad = ceil_div(std::max<int64_t>(n_max, 1), kDenseTile) * kDenseTile;
  s.dense = o->linear_solver == GBBA_SOLVER_DENSE_SCHUR ||
            (o->linear_solver == GBBA_SOLVER_AUTO && s.n_pad <= (int64_t)o->dense_schur_max_size + 64);
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
  s.n_pad = ceil_div(std::max<int64_t>(col, 1), kDenseTile) * kDenseTile;

  // counting sort of observations by point (input order kept within a point)
  scan_offsets(h, counts, s.pt_off, np, chunks, st);
  k_scatter<<<grid, 256, 0, st>>>(idx_in + 2 * no, no, s.pt_off, fill, perm);
  check_launch(h);
  k_segment_sort<<<std::max(1, (int)std::min<int64_t>(ceil_div(np, 256), h->sm_count * 8)), 256, 0, st>>>(perm, s.pt_off, np);
  check_launch(h);
  k_gather<<<grid, 256, 0, st>>>(perm, no, obs_in, idx_in, idx_in + no, idx_in + 2 * no, s.obs, s.cam, s.icam, s.pt);
  check_launch(h);
  // point groups of the Schur point kernel
  if (np > 0) {
    const int64_t nch = ceil_div(np, kGroupChunk);
    const unsigned gb = (unsigned)ceil_div(nch, 128);
    k_pt_groups<<<gb, 128, 0, st>>>(s.pt_off, np, nullptr, s.pgrp_cnt, 0);
    check_launch(h);
    scan_offsets(h, s.pgrp_cnt, s.pgrp_off, nch, chunks, st);
    k_pt_groups<<<gb, 128, 0, st>>>(s.pt_off, np, s.pgrp_off, s.pt_grp, 1);
    check_launch(h);
    uint32_t ng = 0;
    GBBA_CUDA(cudaMemcpyAsync(&ng, s.pgrp_off + nch, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    s.n_pgrp = ng;
    s.nb_pgrp = (int)std::max<int64_t>(1, ceil_div(s.n_pgrp * 32, 128));
  }
  copy_in(s.ext, P->extrinsics, sizeof(double) * 6 * nc, P->memory, st);
  copy_in(s.intr, P->intrinsics, sizeof(double) * s.k * ni, P->memory, st);
  copy_in(s.pts, P->points, sizeof(double) * 3 * np, P->memory, st);
  GBBA_CUDA(cudaMemcpyAsync(s.ext_col, ecol.data(), sizeof(int32_t) * ecol.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(s.intr_col, icol.data(), sizeof(int32_t) * icol.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(s.intr_var, ivar.data(), ni, cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaStreamSynchronize(st));  // the host vectors above go out of scope
  setup_pairs(h, s, tsize);
}


// Pair list and camera CSR of the atomic-free Schur build.  Applies when the
// dense solver is used, every free intrinsic block is private to one camera
// and every camera uses one intrinsic group; otherwise the point-major kernel
// with atomics is used.
static void setup_atomic_path(gbba_handle* h, Solve& s, size_t tsize) {
  GBBA_REQUIRE(s.dense, GBBA_ERROR_NOT_SUPPORTED,
               "the iterative Schur solver needs every free intrinsic block to belong to one camera");
  s.pair_path = false;
  Arena& A = h->pair_arena;
  const size_t w = (size_t)s.no * (6 + s.k) * 3 * tsize;
  A.reset();
  A.reserve(2 * (w + 256) + 4096);
  s.Wbuf = A.take<char>(w);
  s.What = A.take<char>(w);
}

static void setup_pairs(gbba_handle* h, Solve& s, size_t tsize) {
  s.pair_path = false;
  const int64_t nc = s.nc, ni = s.ni, np = s.np, no = s.no;
  const bool want_pairs = s.dense;
  if ((s.schur_build == GBBA_SCHUR_BUILD_POINT_ATOMIC && s.dense) || nc > 0x7fffffffLL || no > 0x7fffffffLL ||
      (want_pairs && (nc > 8192 || nc * nc > (int64_t)1 << 26))) {
    setup_atomic_path(h, s, tsize);
    return;
  }
  cudaStream_t st = s.st;
  const int64_t nk = want_pairs ? nc * nc : 0;
  const int64_t n_pcg = s.dense ? 0 : s.n_pad;
  const int B = 6 + s.k;
  size_t phase2_guess = 0;
  for (int attempt = 0; attempt < 3; ++attempt) {
    Arena& A = h->pair_arena;
    Planner p1;
    p1.take<int32_t>(nc);
    p1.take<uint32_t>(ni);
    p1.take<int>(2);
    p1.take<uint32_t>(nc + 1);
    p1.take<uint32_t>(nc + 1);
    p1.take<uint32_t>(nc + 1);
    p1.take<uint32_t>(no);
    p1.take<uint32_t>(ceil_div(std::max(np, nk) + 1, 1024) + 1);
    p1.take<uint32_t>(np + 1);
    p1.take<uint32_t>(np + 1);
    p1.take<char>((size_t)no * (s.dense ? 9 * B + 8 : 2 * B + 16) * tsize);
    // PCG vectors (x, r, z, p, q, b), point temporaries, camera blocks
    p1.take<double>(6 * n_pcg);
    p1.take<double>(3 * np);
    p1.take<char>((size_t)(n_pcg ? nc : 0) * B * tsize);
    p1.take<float>(tsize == 4 && n_pcg ? 3 * np : 0);
    p1.take<double>((size_t)nc * B * B);
    p1.take<char>((size_t)(n_pcg ? nc : 0) * B * B * tsize);
    p1.take<char>((size_t)nc * B * tsize);
    p1.take<double>(2 * std::max<int64_t>(4096, nc + 1));  // PCG partial sums (one per camera block at most)
    p1.take<PcgState>(1);
    size_t cam_sort_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cam_sort_bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)no, 0, key_bits(nc));
    p1.take<uint32_t>(no);  // sorted camera keys
    p1.take<uint32_t>(no);  // iota
    p1.take<char>(cam_sort_bytes);
    A.reset();
    A.reserve(p1.used + phase2_guess + 4096);
    s.cam_group = A.take<int32_t>(nc);
    uint32_t* group_cam = A.take<uint32_t>(ni);
    int* conflict = A.take<int>(2);
    uint32_t* cam_hist = A.take<uint32_t>(nc + 1);
    s.cam_off = A.take<uint32_t>(nc + 1);
    uint32_t* cam_fill = A.take<uint32_t>(nc + 1);
    s.cam_obs = A.take<uint32_t>(no);
    uint32_t* chunks = A.take<uint32_t>(ceil_div(std::max(np, nk) + 1, 1024) + 1);
    uint32_t* pcnt = A.take<uint32_t>(np + 1);
    uint32_t* pair_off = A.take<uint32_t>(np + 1);
    s.rec = A.take<char>((size_t)no * (s.dense ? 9 * B + 8 : 2 * B + 16) * tsize);
    s.pcg_x = A.take<double>(n_pcg);
    s.pcg_r = A.take<double>(n_pcg);
    s.pcg_z = A.take<double>(n_pcg);
    s.pcg_p = A.take<double>(n_pcg);
    s.pcg_q = A.take<double>(n_pcg);
    s.pcg_b = A.take<double>(n_pcg);
    s.pcg_y = A.take<double>(3 * np);
    s.pcg_xc = A.take<char>((size_t)(n_pcg ? nc : 0) * B * tsize);
    s.pcg_yf = A.take<float>(tsize == 4 && n_pcg ? 3 * np : 0);
    if (!n_pcg) s.pcg_xc = nullptr;
    if (!(tsize == 4 && n_pcg)) s.pcg_yf = nullptr;
    s.pcg_minv = A.take<double>((size_t)nc * B * B);
    s.pcg_u = A.take<char>((size_t)(n_pcg ? nc : 0) * B * B * tsize);
    s.zc = A.take<char>((size_t)nc * B * tsize);
    s.pcg_part_n = std::max<int64_t>(4096, nc + 1);
    s.pcg_part = A.take<double>(2 * s.pcg_part_n);
    s.pcg_state = A.take<PcgState>(1);
    s.nb_pcg = 256;
    uint32_t* cam_keys = A.take<uint32_t>(no);
    uint32_t* iota = A.take<uint32_t>(no);
    void* cam_sort_tmp = A.take<char>(cam_sort_bytes);
    GBBA_CUDA(cudaMemsetAsync(s.cam_group, 0xff, sizeof(int32_t) * nc, st));
    GBBA_CUDA(cudaMemsetAsync(group_cam, 0xff, sizeof(uint32_t) * ni, st));
    GBBA_CUDA(cudaMemsetAsync(conflict, 0, sizeof(int) * 2, st));
    GBBA_CUDA(cudaMemsetAsync(cam_hist, 0, sizeof(uint32_t) * (nc + 1), st));
    GBBA_CUDA(cudaMemsetAsync(cam_fill, 0, sizeof(uint32_t) * (nc + 1), st));
    const int grid = s.nb_obs;
    k_cam_groups<<<grid, 256, 0, st>>>(s.cam, s.icam, no, s.intr_var, s.cam_group, group_cam, conflict, cam_hist);
    check_launch(h);
    k_pair_count<<<std::max(1, (int)std::min<int64_t>(ceil_div(np, 128), h->sm_count * 16)), 128, 0, st>>>(s.pt_off, s.cam, np, pcnt);
    check_launch(h);
    scan_offsets(h, pcnt, pair_off, np, chunks, st);
    int hconf = 0;
    uint32_t total = 0;
    GBBA_CUDA(cudaMemcpyAsync(&hconf, conflict, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaMemcpyAsync(&total, pair_off + np, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    if (hconf) {
      setup_atomic_path(h, s, tsize);
      return;
    }
    Planner p2;
    if (!want_pairs) total = 0;
    size_t pair_sort_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, pair_sort_bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const unsigned long long*)nullptr, (unsigned long long*)nullptr, (int)total, 0,
                                    key_bits(nk));
    p2.take<char>(pair_sort_bytes);
    p2.take<uint32_t>(total);
    p2.take<unsigned long long>(total);
    p2.take<uint32_t>(total);
    p2.take<uint32_t>(nk + 1);
    p2.take<uint32_t>(nk + 1);
    p2.take<uint32_t>(nk + 1);
    p2.take<unsigned long long>(total);
    p2.take<uint32_t>(nk);
    p2.take<uint32_t>(1);
    if (A.used + p2.used + 4096 > A.capacity) {  // grow and redo phase 1
      phase2_guess = p2.used + (A.used > p1.used ? A.used - p1.used : 0);
      A.release();
      continue;
    }
    // camera CSR: observation lists per camera in ascending (point) order, by a
    // stable radix sort of the observations on their camera
    scan_offsets(h, cam_hist, s.cam_off, nc, chunks, st);
    k_iota<<<grid, 256, 0, st>>>(iota, no);
    check_launch(h);
    {
      size_t bytes = cam_sort_bytes;
      GBBA_CUDA(cub::DeviceRadixSort::SortPairs(cam_sort_tmp, bytes, s.cam, cam_keys, iota, s.cam_obs, (int)no, 0,
                                                key_bits(nc), st));
      count_launch(h, 4);
    }
    if (!want_pairs) {
      s.pair_path = true;
      s.n_blocks = 0;
      return;
    }
    // pair list bucketed by camera pair
    unsigned long long* tmp = A.take<unsigned long long>(total);
    uint32_t* keys = A.take<uint32_t>(total);
    uint32_t* hist = A.take<uint32_t>(nk + 1);
    s.blk_off = A.take<uint32_t>(nk + 1);
    uint32_t* fill = A.take<uint32_t>(nk + 1);
    s.pairs = A.take<unsigned long long>(total);
    s.blocks = A.take<uint32_t>(nk);
    uint32_t* count = A.take<uint32_t>(1);
    GBBA_CUDA(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * (nk + 1), st));
    GBBA_CUDA(cudaMemsetAsync(fill, 0, sizeof(uint32_t) * (nk + 1), st));
    GBBA_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), st));
    void* pair_sort_tmp = A.take<char>(pair_sort_bytes);
    uint32_t* keys_sorted = A.take<uint32_t>(total);
    k_pair_write<<<std::max(1, (int)std::min<int64_t>(ceil_div(np, 128), h->sm_count * 16)), 128, 0, st>>>(
        s.pt_off, s.cam, np, nc, pair_off, tmp, keys, hist);
    check_launch(h);
    scan_offsets(h, hist, s.blk_off, nk, chunks, st);
    if (total > 0) {  // stable: pairs stay in generation (point) order inside a block
      size_t bytes = pair_sort_bytes;
      GBBA_CUDA(cub::DeviceRadixSort::SortPairs(pair_sort_tmp, bytes, keys, keys_sorted, tmp, s.pairs, (int)total, 0,
                                                key_bits(nk), st));
      count_launch(h, 4);
    }
    // work items: chunks of at most `chunk` (<= kPairChunk) pairs per camera-pair block
    const uint32_t chunk = (uint32_t)std::min(std::max(h->pair_chunk, 1), kPairChunk);
    std::vector<uint32_t> hoff(nk + 1);
    GBBA_CUDA(cudaMemcpyAsync(hoff.data(), s.blk_off, sizeof(uint32_t) * (nk + 1), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    std::vector<PairItem> items;
    std::vector<PairMerge> merges;
    int32_t slots = 0;
    for (int64_t key = 0; key < nk; ++key) {
      const uint32_t b = hoff[key], e = hoff[key + 1];
      if (e == b) continue;
      const uint32_t nch = (e - b + chunk - 1) / chunk;
      if (nch == 1) {
        items.push_back(PairItem{(uint32_t)key, b, e, -1});
        continue;
      }
      merges.push_back(PairMerge{(uint32_t)key, (uint32_t)slots, nch});
      for (uint32_t c = 0; c < nch; ++c)
        items.push_back(PairItem{(uint32_t)key, b + c * chunk, std::min(e, b + (c + 1) * chunk), slots++});
    }
    Arena& I = h->item_arena;
    I.reset();
    I.reserve(sizeof(PairItem) * items.size() + sizeof(PairMerge) * merges.size() + (size_t)slots * B * B * tsize +
              4096);
    s.pair_items = I.take<PairItem>(items.size());
    s.pair_merges = I.take<PairMerge>(merges.size());
    s.pair_partial = I.take<char>((size_t)slots * B * B * tsize);
    GBBA_CUDA(cudaMemcpyAsync(s.pair_items, items.data(), sizeof(PairItem) * items.size(), cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaMemcpyAsync(s.pair_merges, merges.data(), sizeof(PairMerge) * merges.size(), cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    s.n_blocks = (int64_t)items.size();
    s.n_merges = (int64_t)merges.size();
    s.pair_path = true;
    return;
  }
  // every attempt fell short of the pair list's size: never continue with a
  // half-built workspace
  throw Error{GBBA_ERROR_OUT_OF_MEMORY, "camera-pair workspace could not be sized"};
}

// Block-Jacobi PCG on the implicit Schur complement: ceres's CG
// (conjugate_gradients_solver.cc:66-248) with the per-solve options the LM
// strategy passes (levenberg_marquardt_strategy.cc:88-96: q_tolerance = eta,
// r_tolerance = -1, i.e. the residual-norm test off), the residual recomputed
// as b - S x every options.refinement_interval iterations (ceres's
// residual_reset_period), FP64 vectors and reductions over the stored FP32 /
// FP64 operator blocks.  The loop runs on the device: the host launches
// chunks of kPcgChunk iterations (replayed from a CUDA graph) and reads the
// `done` flag once per chunk.
constexpr int kPcgChunk = 4;

template <int M, typename T>
static void pcg_solve(Solve& s, const gbba_options* o, gbba_summary* sum) {
  gbba_handle* h = s.h;
  cudaStream_t st = s.st;
  constexpr int B = 6 + Model<M>::K;
  const int64_t n = s.n_red;
  const int nbv = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), s.nb_pcg));
  const int nbc = (int)std::max<int64_t>(1, ceil_div(s.nc, 256));      // k_pcg_precond blocks
  const int nbs = (int)std::max<int64_t>(1, s.nc);  // k_spmv_camera blocks (one per camera)
  // k_spmv_point blocks: at most 8 waves of 16 blocks per SM, striding over the point groups
  const int nbp = (int)std::max<int64_t>(1, std::min<int64_t>(s.nb_pgrp, (int64_t)h->sm_count * 16 * 8));
  const int nbx = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(s.nc * B, 256), 1024));  // k_pcg_gather_cam
  const int period = std::max(1, o->refinement_interval);
  PcgState* ps = s.pcg_state;
  double* part_a = s.pcg_part;                 // r.z, then p.q
  double* part_b = s.pcg_part + s.pcg_part_n;  // |b|^2, then the model and r.r
  k_pcg_init<T><<<nbv, 256, 0, st>>>((const T*)s.rhs, s.pcg_b, s.pcg_x, s.pcg_r, n, part_b);
  check_launch(h);
  k_pcg_start<<<1, 256, 0, st>>>(part_b, nbv, -1.0, ps);
  check_launch(h);
  auto spmv = [&](const double* x, double* out, double* part, int reset) {
    if (s.np > 0) {
      k_pcg_gather_cam<B, T><<<nbx, 256, 0, st>>>(x, (T*)s.pcg_xc, s.ext_col, s.intr_col, s.cam_group, s.k, s.nc,
                                                  ps, reset);
      check_launch(h);
      k_spmv_point<B, T><<<nbp, 128, 0, st>>>(s.pt_off, s.pt, s.pt_grp, s.n_pgrp, s.cam, (const T*)s.rec,
                                              (const T*)s.Vinv, (const T*)s.pcg_xc,
                                              sizeof(T) == 4 ? (T*)s.pcg_yf : (T*)s.pcg_y, ps, reset);
      check_launch(h);
    }
    auto cam = [&](auto warps) {
      constexpr int W = decltype(warps)::value;
      k_spmv_camera<B, T, W><<<(unsigned)nbs, W * 32, 0, st>>>(
          s.cam_off, s.cam_obs, s.pt, (const T*)s.rec, (const T*)s.pcg_u, s.ext_col, s.intr_col, s.cam_group, s.k,
          s.nc, s.diag_c, s.radius, x, s.pcg_y, s.pcg_yf, out, part, ps, reset);
    };
    if (h->camera_warps == 2) cam(std::integral_constant<int, 2>());
    else if (h->camera_warps == 8) cam(std::integral_constant<int, 8>());
    else cam(std::integral_constant<int, 4>());
    check_launch(h);
  };
  auto iteration = [&]() {
    k_pcg_precond<B><<<nbc, 256, 0, st>>>(s.pcg_minv, s.ext_col, s.intr_col, s.cam_group, s.k, s.nc, s.pcg_r,
                                          s.pcg_z, part_a, ps);
    check_launch(h);
    k_pcg_direction<<<nbv, 256, 0, st>>>(n, s.pcg_z, s.pcg_p, part_a, nbc, ps);
    check_launch(h);
    spmv(s.pcg_p, s.pcg_q, part_a, 0);
    k_pcg_step<<<nbv, 256, 0, st>>>(n, s.pcg_x, s.pcg_r, s.pcg_p, s.pcg_q, part_a, nbs, period, ps);
    check_launch(h);
    spmv(s.pcg_x, s.pcg_q, nullptr, period);  // residual reset: q = S x (only when it % period == 0)
    k_pcg_reset<<<nbv, 256, 0, st>>>(n, s.pcg_r, s.pcg_b, s.pcg_q, period, ps);
    check_launch(h);
    k_pcg_model<<<nbv, 256, 0, st>>>(n, s.pcg_x, s.pcg_b, s.pcg_r, part_b, ps);
    check_launch(h);
    k_pcg_terminate<<<1, 256, 0, st>>>(part_b, nbv, o->eta, o->max_linear_solver_iterations, ps);
    check_launch(h);
  };
  // one chunk of iterations as a graph, captured on first use in this solve
  if (o->use_cuda_graphs && !s.pcg_graph) {
    const int64_t l0 = h->launches;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      for (int i = 0; i < kPcgChunk; ++i) iteration();
      GBBA_CUDA(cudaStreamEndCapture(st, &g));
      GBBA_CUDA(cudaGraphInstantiate(&s.pcg_graph, g, 0));
      cudaGraphDestroy(g);
      s.pcg_chunk_launches = h->launches - l0;
    } else {
      cudaGetLastError();
    }
    h->launches = l0;  // captured, not yet run
  }
  int* hdone = reinterpret_cast<int*>(h->pinned + 160);
  for (int launched = 0;; launched += kPcgChunk) {
    if (s.pcg_graph) {
      GBBA_CUDA(cudaGraphLaunch(s.pcg_graph, st));
      count_launch(h, (int)s.pcg_chunk_launches);
    } else {
      for (int i = 0; i < kPcgChunk; ++i) iteration();
    }
    GBBA_CUDA(cudaMemcpyAsync(hdone, &ps->done, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    // the device stops at max_linear_solver_iterations; this bound only
    // guards against a state that never reports done
    if (*hdone || launched > o->max_linear_solver_iterations + kPcgChunk) break;
  }
  PcgState* hs = reinterpret_cast<PcgState*>(h->pinned + 168);
  GBBA_CUDA(cudaMemcpyAsync(hs, ps, sizeof(PcgState), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaStreamSynchronize(st));
  sum->linear_solver_iterations += hs->it;
  if (hs->failure) GBBA_CUDA(cudaMemsetAsync(s.flag, 5, sizeof(int), st));
  k_convert<double, T><<<nbv, 256, 0, st>>>(s.pcg_x, (T*)s.zsol, n);
  check_launch(h);
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

  // The mixed path evaluates its FP64 residuals from per-camera FP64 poses
  // (a 3x3 product per observation instead of the Rodrigues sine/cosine):
  // s.pose for the current parameters, s.pose2 for the evaluated ones.
  constexpr bool kPose = sizeof(T) == 4;
  const unsigned nb_cam_pose = (unsigned)std::max<int64_t>(1, ceil_div(s.nc, 128));
  auto to_float = [&](const double* src, float* dst, int64_t n) {
    if (n <= 0) return;
    k_convert<double, float><<<(unsigned)std::min<int64_t>(ceil_div(n, 256), 1024), 256, 0, st>>>(src, dst, n);
    check_launch(h);
  };
  auto launch_cost = [&](const double* e, const double* i, const double* p) {
    Prob Pc = make_prob(s, e, i, p, o);
    // the mixed path's residual cache: current parameters in slot 0, the
    // candidate in slot 1 (copied to slot 0 when the step is accepted)
    if (kPose && s.rcache) Pc.rc_out = s.rcache + (e == s.ext ? 0 : s.no);
    if (kPose && s.nc > 0) {
      k_cam_pose<<<nb_cam_pose, 128, 0, st>>>(e, s.nc, s.pose2);
      check_launch(h);
      Pc.pose = s.pose2;
    }
    k_cost<M><<<s.nb_obs, 256, 0, st>>>(Pc, e, i, p, s.part_cost, s.nonfinite);
    check_launch(h);
  };
  // gradient max norm and x norm at the current point; scale on first use
  auto linearize = [&](bool first, double* gmax, double* xnorm) {
    Prob P = make_prob(s, s.ext, s.intr, s.pts, o);
    if (kPose && s.nc > 0) {
      k_cam_pose<<<nb_cam_pose, 128, 0, st>>>(s.ext, s.nc, s.pose);
      check_launch(h);
      P.pose = s.pose;
    }
    if (kPose) {
      to_float(s.ext, s.ext_f, 6 * s.nc);
      to_float(s.intr, s.intr_f, (int64_t)s.k * s.ni);
      to_float(s.pts, s.pts_f, 3 * s.np);
      P.ext_f = s.ext_f;
      P.intr_f = s.intr_f;
      P.pts_f = s.pts_f;
    }
    GBBA_CUDA(cudaMemsetAsync(s.cn_c, 0, sizeof(double) * (s.n_red + 1), st));
    GBBA_CUDA(cudaMemsetAsync(s.g_c, 0, sizeof(double) * (s.n_red + 1), st));
    GBBA_CUDA(cudaMemsetAsync(s.cn_p, 0, sizeof(double) * 3 * s.np, st));
    GBBA_CUDA(cudaMemsetAsync(s.g_p, 0, sizeof(double) * 3 * s.np, st));
    GBBA_CUDA(cudaMemsetAsync(s.gmax_bits, 0, sizeof(unsigned long long), st));
    // deterministic sums: largest terms, scales, fixed-point sums, back to FP64
    auto ull = [](double* p) { return reinterpret_cast<unsigned long long*>(p); };
    const double nobs = (double)std::max<int64_t>(1, s.no);
    const unsigned gc = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(s.n_red, 256), 1024));
    const unsigned gp = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(3 * s.np, 256), 4096));
    k_linearize_max<M, T><<<s.nb_obs, 256, 0, st>>>(P, ull(s.cn_c), ull(s.cn_p), ull(s.g_c), ull(s.g_p));
    check_launch(h);
    if (s.n_red > 0) {
      k_linearize_exp<<<gc, 256, 0, st>>>(s.n_red, nobs, ull(s.cn_c), ull(s.g_c), s.diag_c);
      check_launch(h);
    }
    if (s.np > 0) {
      k_linearize_exp<<<gp, 256, 0, st>>>(3 * s.np, nobs, ull(s.cn_p), ull(s.g_p), s.diag_p);
      check_launch(h);
    }
    k_linearize<M, T><<<s.nb_obs, 256, 0, st>>>(P, s.cn_c, s.cn_p, s.g_c, s.g_p, s.diag_c, s.diag_p);
    check_launch(h);
    if (s.n_red > 0) {
      k_linearize_conv<<<gc, 256, 0, st>>>(s.n_red, s.cn_c, s.g_c, s.diag_c);
      check_launch(h);
    }
    if (s.np > 0) {
      k_linearize_conv<<<gp, 256, 0, st>>>(3 * s.np, s.cn_p, s.g_p, s.diag_p);
      check_launch(h);
    }
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
    if (kPose && first) {
      to_float(s.scale_c, s.scale_cf, s.n_red);
      to_float(s.scale_p, s.scale_pf, 3 * s.np);
    }
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
  // Fused linearisation (pair path): after an accepted step only the poses,
  // the FP32 copies and the x norm are refreshed here; the LM diagonal and
  // the gradient at the new point come out of the next Schur phase
  // (k_schur_point_rec, k_rhs_camera), so no separate Jacobian pass runs.
  const bool fused = s.pair_path;
  auto refresh = [&]() {
    if (kPose && s.nc > 0) {
      k_cam_pose<<<nb_cam_pose, 128, 0, st>>>(s.ext, s.nc, s.pose);
      check_launch(h);
    }
    if (kPose) {
      to_float(s.ext, s.ext_f, 6 * s.nc);
      to_float(s.intr, s.intr_f, (int64_t)s.k * s.ni);
      to_float(s.pts, s.pts_f, 3 * s.np);
    }
    k_xnorm<<<gx, 256, 0, st>>>(s.ext, s.ext_col, n_e, s.intr, s.intr_var, s.k, n_i, s.pts, 3 * s.np, s.part_x);
    check_launch(h);
    k_reduce3<<<1, 256, 0, st>>>(s.part_x, gx, s.part_x, 0, s.part_x, 0, s.part_x, 0, s.scalars + 4);
    check_launch(h);
  };
  // gradient max norm of the last Schur phase (reads its shards; synchronises)
  auto read_gmax = [&]() -> double {
    unsigned long long* hb = reinterpret_cast<unsigned long long*>(pin + 64);
    GBBA_CUDA(cudaMemcpyAsync(hb, s.gmax_shards, sizeof(unsigned long long) * kGmaxShards, cudaMemcpyDeviceToHost,
                              st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    double m = 0.0;
    for (int i = 0; i < kGmaxShards; ++i) m = std::max(m, __builtin_bit_cast(double, (long long)hb[i]));
    return m;
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
  auto trace = [&](int i, double c) {
    if (o->trace_capacity > i && i >= 0) {
      if (o->trace_cost) o->trace_cost[i] = c;
      if (o->trace_time_s) o->trace_time_s[i] = now_s() - s.t_origin;
    }
  };
  trace(0, cost);
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
  // The launch sequence of one LM iteration, in five phases separated by the
  // timing events.  Parameters are read from s.ext/s.intr/s.pts and the
  // candidate is written to s.ext2/s.intr2/s.pts2 (an accepted candidate is
  // copied back), so the sequence is invariant and is captured once into CUDA
  // graphs that every iteration replays.
  Prob P = make_prob(s, s.ext, s.intr, s.pts, o);
  if (kPose && s.nc > 0) P.pose = s.pose;  // refreshed by linearize() after every accepted step
  // gradient norm of the fused linearisation: only with a gradient tolerance
  unsigned long long* const gshards = o->gradient_tolerance > 0.0 ? s.gmax_shards : nullptr;
  if (kPose) {
    P.ext_f = s.ext_f;
    P.intr_f = s.intr_f;
    P.pts_f = s.pts_f;
    P.scale_cf = s.scale_cf;
    P.scale_pf = s.scale_pf;
    P.rc = s.rcache;  // residuals of the current parameters from the last cost pass
  }
  const int nb_back = s.pair_path ? s.nb_pgrp : s.nb_pt;  // blocks (partials) of the back substitution
  auto record_phase = [&](int ph) {
    switch (ph) {
      case 0:
        if (s.pair_path) GBBA_CUDA(cudaMemsetAsync(s.gmax_shards, 0, sizeof(unsigned long long) * kGmaxShards, st));
        if (s.dense) {
          GBBA_CUDA(cudaMemsetAsync(S, 0, sizeof(T) * s.n_pad * s.n_pad, st));
          k_schur_init<T><<<(unsigned)std::min<int64_t>(ceil_div(s.n_pad, 256), 1024), 256, 0, st>>>(
              S, rhs, s.n_red, s.n_pad, s.diag_c, s.radius, s.pair_path ? 1 : 0);
          check_launch(h);
        } else {
          GBBA_CUDA(cudaMemsetAsync(rhs, 0, sizeof(T) * s.n_pad, st));
        }
        break;
      case 1:
        if (s.np > 0 && s.pair_path) {
          constexpr int B = 6 + Model<M>::K;
          // the point kernel with or without the FP64 re-inversion, writing
          // the full record (dense path: camera-pair products) or the
          // compact one (iterative path)
          auto point_rec = [&](auto fp64_inverse) {
            constexpr bool kInv = decltype(fp64_inverse)::value;
            if (s.dense)
              k_schur_point_rec<M, T, kInv, false><<<(unsigned)ceil_div(s.n_pgrp * 32, 128), 128, 0, st>>>(
                  P, s.pt_grp, s.n_pgrp, s.scale_c, s.scale_p, s.diag_p, o->min_lm_diagonal, o->max_lm_diagonal,
                  gshards, s.radius, (T*)s.Vinv, (T*)s.gpv, (T*)s.rec, s.flag);
            else
              k_schur_point_rec<M, T, kInv, true><<<(unsigned)ceil_div(s.n_pgrp * 32, 128), 128, 0, st>>>(
                  P, s.pt_grp, s.n_pgrp, s.scale_c, s.scale_p, s.diag_p, o->min_lm_diagonal, o->max_lm_diagonal,
                  gshards, s.radius, (T*)s.Vinv, (T*)s.gpv, (T*)s.rec, s.flag);
          };
          if (kPose && (o->mixed_flags & GBBA_MIXED_FP64_POINT_INVERSE))
            point_rec(std::true_type());
          else
            point_rec(std::false_type());
          check_launch(h);
          if (s.dense && s.n_blocks > 0) {
            if (kPose && (o->mixed_flags & GBBA_MIXED_KAHAN_SCHUR))
              k_schur_pairs<B, T, true><<<(unsigned)ceil_div(s.n_blocks * 32, 128), 128, 0, st>>>(
                  (const PairItem*)s.pair_items, s.n_blocks, s.pairs, (const T*)s.rec, s.ext_col, s.intr_col,
                  s.cam_group, s.k, s.nc, S, s.n_pad, (T*)s.pair_partial);
            else
              k_schur_pairs<B, T><<<(unsigned)ceil_div(s.n_blocks * 32, 128), 128, 0, st>>>(
                  (const PairItem*)s.pair_items, s.n_blocks, s.pairs, (const T*)s.rec, s.ext_col, s.intr_col,
                  s.cam_group, s.k, s.nc, S, s.n_pad, (T*)s.pair_partial);
            check_launch(h);
            if (s.n_merges > 0) {
              k_pair_merge<B, T><<<(unsigned)ceil_div(s.n_merges * 32, 128), 128, 0, st>>>(
                  (const PairMerge*)s.pair_merges, s.n_merges, (const T*)s.pair_partial, s.ext_col, s.intr_col,
                  s.cam_group, s.k, s.nc, S, s.n_pad);
              check_launch(h);
            }
          }
          if (s.nc > 0) {
            auto rhs_cam = [&](auto compact) {
              k_rhs_camera<B, T, decltype(compact)::value><<<(unsigned)s.nc, kRhsThreads, 0, st>>>(
                  s.cam_off, s.cam_obs, (const T*)s.rec, s.ext_col, s.intr_col, s.cam_group, s.k, s.nc, rhs,
                  s.scale_c, s.diag_c, o->min_lm_diagonal, o->max_lm_diagonal, s.radius, s.dense ? S : nullptr,
                  s.n_pad, gshards);
            };
            if (s.dense) rhs_cam(std::false_type());
            else rhs_cam(std::true_type());
            check_launch(h);
          }
          if (!s.dense && s.nc > 0) {
            auto cam_blocks = [&](auto warps) {
              constexpr int W = decltype(warps)::value;
              k_cam_blocks<B, T, W><<<(unsigned)s.nc, W * 32, 0, st>>>(
                  s.cam_off, s.cam_obs, (const T*)s.rec, s.ext_col, s.intr_col, s.cam_group, s.k, s.nc, s.diag_c,
                  s.radius, (T*)s.pcg_u, s.pcg_minv);
            };
            if (h->camera_warps == 2) cam_blocks(std::integral_constant<int, 2>());
            else if (h->camera_warps == 8) cam_blocks(std::integral_constant<int, 8>());
            else cam_blocks(std::integral_constant<int, 4>());
            check_launch(h);
            k_cam_inverse<B><<<(unsigned)ceil_div(s.nc, 128), 128, 0, st>>>(s.pcg_minv, s.nc, s.flag);
            check_launch(h);
          }
        } else if (s.np > 0) {
          k_schur_point<M, T><<<s.nb_pt, 128, 0, st>>>(P, s.scale_c, s.scale_p, s.diag_p, s.radius, S, s.n_pad, rhs,
                                                        (T*)s.Vinv, (T*)s.gpv, (T*)s.Wbuf, (T*)s.What, s.flag);
          check_launch(h);
        }
        break;
      case 2:
        if (s.dense) dense_cholesky_solve<T>(h, S, s.n_pad, rhs, z, (T*)s.Linv, s.flag, st);
        else pcg_solve<M, T>(s, o, sum);
        break;
      case 3:
        if (s.np > 0 && s.pair_path) {
          constexpr int B = 6 + Model<M>::K;
          k_gather_cam_rows<B, T>
              <<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(s.nc * B, 256), 1024)), 256, 0, st>>>(
                  z, (T*)s.zc, s.ext_col, s.intr_col, s.cam_group, s.k, s.nc);
          check_launch(h);
          auto backsub = [&](auto compact) {
            k_backsub_rec<B, T, decltype(compact)::value><<<s.nb_pgrp, 128, 0, st>>>(
                s.pt_off, s.pt, s.pt_grp, s.n_pgrp, s.cam, (const T*)s.rec, (const T*)s.zc, (const T*)s.Vinv,
                (const T*)s.gpv, s.scale_p, s.pts, s.pts2, s.part_mcc, s.part_step_p, s.flag);
          };
          if (s.dense) backsub(std::false_type());
          else backsub(std::true_type());
          check_launch(h);
        } else if (s.np > 0) {
          k_backsub<M, T><<<s.nb_pt, 128, 0, st>>>(P, s.scale_c, s.scale_p, z, (T*)s.Vinv, (T*)s.gpv, s.pts2,
                                                    s.part_mcc, s.part_step_p, s.flag);
          check_launch(h);
        }
        k_cam_candidate<T><<<s.nb_cam, 256, 0, st>>>(s.ext, s.intr, s.ext2, s.intr2, s.ext_col, s.intr_col, n_e, n_i, z,
                                                     s.scale_c, s.part_step_c);
        check_launch(h);
        break;
      default:
        launch_cost(s.ext2, s.intr2, s.pts2);
        k_reduce3<<<1, 256, 0, st>>>(s.part_mcc, s.np > 0 ? nb_back : 0, s.part_step_p, s.np > 0 ? nb_back : 0,
                                     s.part_step_c, s.nb_cam, s.part_cost, s.nb_obs, s.scalars);
        check_launch(h);
        break;
    }
  };
  int64_t phase_launches[5] = {0, 0, 0, 0, 0};
  cudaGraphExec_t graphs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  dense_cholesky_prepare<T>();
  if (o->use_cuda_graphs) {
    for (int ph = 0; ph < 5; ++ph) {
      // Phase 2 (the linear solve) is launched directly every iteration: the
      // PCG loop is host-driven, and the dense factorisation relies on the
      // per-launch stream priority of its panel chain, which a graph replay
      // does not reproduce (medium workload: 4.59 ms replayed, 4.50 ms
      // launched directly).
      if (ph == 2) continue;
      const int64_t l0 = h->launches;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        break;
      }
      record_phase(ph);
      GBBA_CUDA(cudaStreamEndCapture(st, &g));
      GBBA_CUDA(cudaGraphInstantiate(&graphs[ph], g, 0));
      cudaGraphDestroy(g);
      phase_launches[ph] = h->launches - l0;
      h->launches = l0;  // captured, not yet run
    }
  }
  auto run_phase = [&](int ph) {
    if (graphs[ph]) {
      GBBA_CUDA(cudaGraphLaunch(graphs[ph], st));
      count_launch(h, (int)phase_launches[ph]);
    } else {
      const int64_t l0 = h->launches;
      record_phase(ph);
      phase_launches[ph] = h->launches - l0;
    }
  };
  // On the fused path the gradient at an accepted point is checked after the
  // next Schur phase (before that phase's step is used), and, when the
  // iteration limit ends the solve right after an accepted step, by one
  // more Schur phase: the same terminations as ceres's check right after
  // the step is accepted.
  bool need_grad = false;
  const bool check_grad = o->gradient_tolerance > 0.0;
  while (term < 0) {
    if (iteration >= o->max_num_iterations) {
      term = GBBA_NO_CONVERGENCE;
      if (fused && need_grad && check_grad) {
        pin[2] = radius;
        GBBA_CUDA(cudaMemcpyAsync(s.radius, pin + 2, sizeof(double), cudaMemcpyHostToDevice, st));
        run_phase(0);
        run_phase(1);
        if (read_gmax() <= o->gradient_tolerance) term = GBBA_CONVERGENCE;
      }
      break;
    }
    pin[2] = radius;
    GBBA_CUDA(cudaMemcpyAsync(s.radius, pin + 2, sizeof(double), cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaMemsetAsync(s.flag, 0, sizeof(int), st));
    GBBA_CUDA(cudaMemsetAsync(s.nonfinite, 0, sizeof(int), st));
    GBBA_CUDA(cudaEventRecord(ev[0], st));
    run_phase(0);
    GBBA_CUDA(cudaEventRecord(ev[4], st));
    run_phase(1);
    GBBA_CUDA(cudaEventRecord(ev[1], st));
    if (fused && need_grad && check_grad) {
      need_grad = false;
      if (read_gmax() <= o->gradient_tolerance) {
        term = GBBA_CONVERGENCE;
        break;
      }
    }
    need_grad = false;
    run_phase(2);
    GBBA_CUDA(cudaEventRecord(ev[5], st));
    run_phase(3);
    GBBA_CUDA(cudaEventRecord(ev[2], st));
    run_phase(4);
    GBBA_CUDA(cudaEventRecord(ev[3], st));
    sum->schur_kernel_launches += phase_launches[1];
    sum->factor_launches += (int32_t)phase_launches[2];
    Scalars* hs = reinterpret_cast<Scalars*>(pin + 8);
    GBBA_CUDA(cudaMemcpyAsync(hs, s.scalars, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaMemcpyAsync(&hs->flag, s.flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaMemcpyAsync(&hs->nonfinite, s.nonfinite, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (fused) GBBA_CUDA(cudaMemcpyAsync(pin + 20, s.scalars + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    if (fused) x_norm = std::sqrt(pin[20]);
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
    trace(iteration, cost);
    if (success) {
      ++sum->num_successful_steps;
      radius = radius / std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * relative_decrease - 1.0, 3));
      radius = std::min(o->max_trust_region_radius, radius);
      decrease_factor = 2.0;
      GBBA_CUDA(cudaMemcpyAsync(s.ext, s.ext2, sizeof(double) * n_e, cudaMemcpyDeviceToDevice, st));
      GBBA_CUDA(cudaMemcpyAsync(s.intr, s.intr2, sizeof(double) * n_i, cudaMemcpyDeviceToDevice, st));
      GBBA_CUDA(cudaMemcpyAsync(s.pts, s.pts2, sizeof(double) * 3 * s.np, cudaMemcpyDeviceToDevice, st));
      if (kPose && s.rcache)
        GBBA_CUDA(cudaMemcpyAsync(s.rcache, s.rcache + s.no, sizeof(float4) * s.no, cudaMemcpyDeviceToDevice, st));
      if (fused) {
        refresh();
        need_grad = true;
      } else {
        const double tj = now_s();
        linearize(false, &gmax, &x_norm);
        sum->jacobian_time_s += now_s() - tj;
        if (gmax <= o->gradient_tolerance) term = GBBA_CONVERGENCE;
      }
    } else {
      ++sum->num_unsuccessful_steps;
      radius = radius / decrease_factor;  // StepRejected and StepIsInvalid
      decrease_factor *= 2.0;
      if (radius < o->min_trust_region_radius) term = GBBA_CONVERGENCE;
    }
  }
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  for (int i = 0; i < 5; ++i)
    if (graphs[i]) cudaGraphExecDestroy(graphs[i]);
  if (s.pcg_graph) {
    cudaGraphExecDestroy(s.pcg_graph);
    s.pcg_graph = nullptr;
  }
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
  s.t_origin = t0;
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
  // Mixed path: FP32 steps can end the LM early through ceres's stopping rule
  // (a poor but accepted step with |dcost| <= 1e-6 cost).  When the mixed run
  // reports convergence, a short plain-FP64 run from its solution, with
  // tolerances 1000x tighter, finishes at the FP64 minimum.
  if (st == GBBA_SUCCESS && sum->usable && sum->termination_type == GBBA_CONVERGENCE &&
      o->precision == GBBA_PRECISION_MIXED && o->fp64_polish_iterations > 0) {
    gbba_options o2 = *o;
    o2.precision = GBBA_PRECISION_FP64;
    o2.max_num_iterations = o->fp64_polish_iterations;
    o2.function_tolerance = o->function_tolerance * 1e-3;
    o2.parameter_tolerance = o->parameter_tolerance * 1e-3;
    o2.trace_cost = o2.trace_time_s = nullptr;
    o2.trace_capacity = 0;
    gbba_summary s2{};
    const gbba_status st2 = solve_impl(h, P, &o2, &s2);
    if (st2 == GBBA_SUCCESS && s2.usable) {
      sum->final_cost = s2.final_cost;
      sum->num_iterations += s2.num_iterations;
      sum->num_successful_steps += s2.num_successful_steps;
      sum->num_unsuccessful_steps += s2.num_unsuccessful_steps;
      sum->termination_type = s2.termination_type;
      sum->jacobian_time_s += s2.jacobian_time_s;
      sum->linear_solver_time_s += s2.linear_solver_time_s;
      sum->residual_time_s += s2.residual_time_s;
      sum->linear_solver_iterations += s2.linear_solver_iterations;
    }
  }
  sum->total_time_s = now_s() - t0;
  return st;
}

}  // namespace gbba
