// Batched local bundle adjustment: thousands of independent problems in one
// launch (gbba_solve_batched).
//
// Each problem is an independent ceres-style LM solve (the same semantics as
// gbba_solve: Jacobi scaling, LM diagonal, Schur elimination, step quality and
// radius update, ceres's terminations -- trust_region_minimizer.cc,
// levenberg_marquardt_strategy.cc).  Local windows are small (<= 40 cameras,
// reduced camera system <= 256 unknowns), so one CTA owns one problem for its
// whole solve:
//   - in FP32 the lower triangle of S lives in shared memory (n(n+1)/2
//     values, <= 131.6 KB);
//   - in FP64 (the plain FP64 path and the mixed path's FP64 polish) S lives
//     in a per-CTA slice of global memory (L2-resident): an FP64 S of
//     n = 256 would not fit shared memory;
//   - every sum the Schur build scatters (S, rhs, column norms, gradient) is
//     accumulated in fixed point, integers under atomics: integer addition is
//     associative, so the result does not depend on the order in which warps
//     reach an entry and a solve is bitwise repeatable.  The scales are
//     powers of two: S_ij is scaled by 2^(e_i + e_j), e_i chosen from a bound
//     on column i's norm, so that each entry keeps the resolution of its own
//     columns (int32 entries of S in FP32, int64 in FP64); the vectors take
//     one scale per window (int64).  A build that finds a column norm above
//     the bound it was scaled for runs again with the norms it found;
//   - the cost pass runs one thread per observation (FP64 residuals from the
//     window's FP64 poses in shared memory);
//   - the Schur build runs one warp per point (V, V^-1, g_p, W, W V^-1) and
//     also forms the column norms and the gradient of its Jacobian (the LM
//     diagonal and ceres's gradient check): the FP64 path's sums in the
//     global slice, the FP32 path's in shared memory;
//   - the Cholesky factorisation and both triangular solves run where S
//     lives; every thread evaluates the step and takes the same accept /
//     reject decision.
// CTAs never wait on each other, so the launch cannot deadlock; the hardware
// schedules the next problem onto an SM as soon as one finishes (problems are
// ordered largest first to shorten the tail).
#include <math_constants.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gbba_device.cuh"
#include "gbba_internal.h"

namespace gbba {

void scan_offsets(gbba_handle* h, const uint32_t* counts, uint32_t* off, int64_t n, uint32_t* tmp_chunks,
                  cudaStream_t st);
__global__ void k_scatter(const uint32_t* pt, int64_t no, const uint32_t* off, uint32_t* fill, uint32_t* perm);
__global__ void k_segment_sort(uint32_t* perm, const uint32_t* off, int64_t np);

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

constexpr int kNMax = 256;  // largest reduced camera system of a batched problem
// doubles of a CTA's global scratch slice: column norms, gradient, rhs, S
constexpr int64_t kGlobalSlice = 3 * kNMax + kNMax * (kNMax + 1) / 2;

struct BProb {
  uint32_t o0, o1;  // observations (sorted by point)
  uint32_t x0, x1;  // points
  uint32_t c0, nc;  // cameras
  uint32_t g0, ni;  // intrinsic groups
  uint32_t n;       // reduced camera-side size
  uint32_t pad;
};

struct BOut {
  double initial_cost, final_cost;
  int32_t iterations, successful, unsuccessful, termination, usable, status;
};

struct BArgs {
  const BProb* probs;
  const uint32_t* order;
  double *ext, *intr, *pts, *ext2, *intr2, *pts2;
  const double2* obs;
  const uint32_t *cam, *icam, *pt_off, *pt_s;  // pt_s: point of each (sorted) observation
  const int32_t *ext_col, *intr_col;  // problem-local reduced columns (-1 = held)
  const uint8_t* intr_var;
  double* scale_p;
  void *Vinv, *gp, *wscratch;  // compute type
  double* gscr;                // kGlobalSlice doubles per CTA
  // FP32 path: FP32 copies of the current parameters and of the point
  // scales, and per observation the corrected residual and sqrt(rho') of the
  // FP64 cost evaluation at the current parameters and at the candidate
  // ([2][total_obs])
  float *ext_f, *intr_f, *pts_f, *scale_pf;
  float4* rcache;
  int64_t total_obs;
  int max_views;
  BOut* out;
  // options
  int max_iterations, max_invalid, jacobi, loss_type;
  double loss_a, ftol, gtol, ptol, r0, rmax, rmin, min_rel, dmin, dmax;
};

// One observation's scratch slot (compute type values): W = Jc^T Jp and
// W V^-1 (B x 3 each, row i = camera parameter i), the scaled camera Jacobian
// Jc (2 x B) and, in a window with one intrinsic group, the observation's
// U_kk lower triangle, intrinsic rhs correction and intrinsic gradient
// Jc_k^T r.  Parts start on 4-value
// (16-byte) boundaries.  The back substitution reuses the slot for Jc z and
// the residual (4 doubles) and Jp (6 values).
__host__ __device__ constexpr int rnd4(int v) { return (v + 3) & ~3; }
template <int K>
struct Slot {
  static constexpr int B = 6 + K, KK = K * (K + 1) / 2;
  static constexpr int kW = 0, kWh = rnd4(3 * B), kJ = kWh + rnd4(3 * B), kU = kJ + rnd4(2 * B), kQ = kU + KK,
                       kG = kQ + K;
  static constexpr int kSize = rnd4(kG + K);
  static_assert(kSize >= 8 + 6, "back substitution entries fit the slot");
};

template <typename T>
__device__ __forceinline__ void ld18(const T* p, T v[18]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) ld4<T>(p + 4 * q, v + 4 * q);
  v[16] = p[16];
  v[17] = p[17];
}

// NS: values of S held in shared memory (1 when S lives in global memory).
constexpr int kPoseCams = 64;  // larger windows evaluate residuals by Rodrigues and read columns from global memory
template <typename T, int NS, int N>
struct Shared {
  double pose[2][kPoseCams * 12];  // FP64 poses of ext (0) and of the candidate ext2 (1)
  int32_t ecol[kPoseCams * 6];     // the window's extrinsic columns (-1 = held)
  int32_t kcol[8];                 // one intrinsic group: its columns
  T S[NS];
  T rhs[N];
  T z[N];
  T zs[N];  // the camera step in the original parameterisation, z * scale_c
  double scale_c[N];
  double diag_c[N];
  float scale_cf[N];  // FP32 path: scale_c
  // FP32 path: fixed-point sums of rhs, column norms and gradient of the
  // Schur build's Jacobian
  long long fxv[3][N];
  double fx[4];    // scales of the column norms, gradient and rhs (fx[0] unused)
  int fxk[4];      // their exponents
  double cbnd[N];  // per column: bound on its scaled column norm the scales are chosen for
  T fxs[N];        // per column: the power-of-two factor of S's fixed-point scale (FP32)
  T fxi[N];        // its inverse
  int32_t fxe[N];  // its exponent (FP64)
  int fxbits;      // S's budget: 2^(2 e_i) bound_i < 2^fxbits
  int fxbad;       // a term out of range or not finite (FP64)
  double red[kWarps];
  double bcast[8];
  int flag;
};
template <typename SS>
struct SharedOf {
  static constexpr bool kGlobalS = sizeof(SS) == 8;
  using type = Shared<SS, kGlobalS ? 1 : kNMax * (kNMax + 1) / 2, kNMax>;
};

__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }

__device__ __forceinline__ double block_sum(double v, double* red, double* out) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kWarps; ++w) s += red[w];
    *out = s;
  }
  __syncthreads();
  return *out;
}
__device__ __forceinline__ double block_max(double v, double* red, double* out) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kWarps; ++w) s = fmax(s, red[w]);
    *out = s;
  }
  __syncthreads();
  return *out;
}

// Exponent of the power of two 2^e with bound * 2^e <= 2^bits (0 for a
// bound that is not a positive finite number), clamped to [-lim, lim].
__device__ __forceinline__ int pow2_exp(double bound, int bits, int lim) {
  if (!(bound > 0.0) || !isfinite(bound)) return 0;
  int e;
  frexp(bound, &e);  // bound < 2^e
  return max(-lim, min(lim, bits - e));
}
// Exponent e of a column's factor 2^e with 2^(2e) * bound < 2^bits (lim for
// a bound that is not a positive number), clamped to [-lim, lim].  S_ij is
// accumulated scaled by 2^(e_i + e_j).  Every term added to S_ij is an entry
// of a per-observation U or a W_x V^-1 W_y^T of two observations x, y of one
// point, and U >= W_x V^-1 W_x^T: with every column norm within its bound,
// Cauchy-Schwarz (over the observations, then over the points) keeps the
// partial sums within (1 + m) sqrt(bound_i bound_j), m the most
// observations of one point that touch one column.  So the scaled sums stay
// below (1 + m) 2^bits, and each entry's resolution follows its own columns
// instead of the largest column of the window.
__device__ __forceinline__ int col_exp(double bound, int bits, int lim) {
  if (!(bound > 0.0)) return lim;
  if (!isfinite(bound)) return -lim;
  int be;
  frexp(bound, &be);  // bound < 2^be
  return max(-lim, min(lim, (bits - be) >> 1));
}
// v * 2^k rounded to the nearest integer (ties away from zero) with integer
// operations only (FP64 arithmetic is slow on this GPU); a result that
// would reach 2^62 sets bit 0 of *bad, a value that is not finite bit 1,
// and either gives 0.  Any rounding rule serves: a sum of integers does not
// depend on the order.
__device__ __forceinline__ long long fx_round(double v, int k, int* bad) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)(b >> 52) & 0x7ff;
  const int sh = ex - 1075 + k;  // |v| 2^k = m 2^sh, m < 2^53
  if (ex == 0x7ff || sh > 9) {
    atomicOr(bad, ex == 0x7ff ? 2 : 1);
    return 0;
  }
  const long long m = ex ? (long long)((b & 0xfffffffffffffull) | 0x10000000000000ull) : 0ll;
  const int rs = min(max(-sh, 0), 63);
  const long long ml = m << max(sh, 0);
  const long long r = rs ? (ml + (1ll << (rs - 1))) >> rs : ml;
  return (b >> 63) ? -r : r;
}
__device__ __forceinline__ void fx_add(long long* p, double v, int k, int* bad) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)fx_round(v, k, bad));
}
__device__ __forceinline__ void fx_add(long long* p, float v, float scale) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)__float2ll_rn(v * scale));
}

// Linearisation of observation o (point p) at the current parameters: the
// corrected residual rr and Jacobian blocks (compute type) and the reduced
// columns of its camera-side parameters.
//   FP64: residual, robust correction and Jacobian evaluated here from the
//   FP64 parameters.
//   FP32: the corrected residual and sqrt(rho') come from the cost
//   evaluation's cache at the same parameters (rc), the Jacobian from the
//   FP32 parameter copies (it does not depend on the observed point), so
//   that no FP64 arithmetic is left.
template <int M, typename T>
__device__ __forceinline__ void obs_lin(const BArgs& a, int64_t o, uint32_t p, const float4* rc, T rr[2],
                                        T Jc[2][6 + Model<M>::K], T Jp[2][3], int col[6 + Model<M>::K]) {
  constexpr int K = Model<M>::K;
  const uint32_t c = a.cam[o], g = a.icam[o];
  T Je[2][6], Jk[2][K], Jx[2][3], s;
  if constexpr (sizeof(T) == 8) {
    double Ed[6], Kd[K], Xd[3], r[2];
#pragma unroll
    for (int i = 0; i < 6; ++i) Ed[i] = a.ext[6 * (int64_t)c + i];
#pragma unroll
    for (int i = 0; i < K; ++i) Kd[i] = a.intr[K * (int64_t)g + i];
#pragma unroll
    for (int i = 0; i < 3; ++i) Xd[i] = a.pts[3 * (int64_t)p + i];
    const double2 ob = a.obs[o];
    residual<M, double, true>(Kd, Ed, Xd, ob.x, ob.y, r, Je, Jk, Jx, (double*)nullptr);
    double sr1;
    robust<double>(a.loss_type, a.loss_a, r[0] * r[0] + r[1] * r[1], &sr1);
    rr[0] = r[0] * sr1;
    rr[1] = r[1] * sr1;
    s = sr1;
  } else {
    T Ef[6], Kf[K], Xf[3], rf[2];
#pragma unroll
    for (int i = 0; i < 6; ++i) Ef[i] = a.ext_f[6 * (int64_t)c + i];
#pragma unroll
    for (int i = 0; i < K; ++i) Kf[i] = a.intr_f[K * (int64_t)g + i];
#pragma unroll
    for (int i = 0; i < 3; ++i) Xf[i] = a.pts_f[3 * (int64_t)p + i];
    residual<M, T, true>(Kf, Ef, Xf, T(0), T(0), rf, Je, Jk, Jx, (T*)nullptr);
    const float4 q = rc[o];
    rr[0] = q.x;
    rr[1] = q.y;
    s = q.z;
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) col[j] = a.ext_col[6 * (int64_t)c + j];
#pragma unroll
  for (int j = 0; j < K; ++j) col[6 + j] = a.intr_col[K * (int64_t)g + j];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int j = 0; j < 6; ++j) Jc[i][j] = Je[i][j] * s;
#pragma unroll
    for (int j = 0; j < K; ++j) Jc[i][6 + j] = Jk[i][j] * s;
#pragma unroll
    for (int j = 0; j < 3; ++j) Jp[i][j] = Jx[i][j] * s;
  }
}

// T: Jacobians and point blocks; SS: the shared-memory S, its factor and the step.
template <int M, typename T, typename SS>
__global__ void __launch_bounds__(kThreads, 1) k_lm_batched(BArgs a) {
  constexpr int K = Model<M>::K;
  constexpr int B = 6 + K;
  constexpr bool kGS = SharedOf<SS>::kGlobalS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename SharedOf<SS>::type& sh = *reinterpret_cast<typename SharedOf<SS>::type*>(smem_raw);
  const uint32_t pid = a.order[blockIdx.x];
  const BProb P = a.probs[pid];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = (int)P.n;
  T* Vinv = (T*)a.Vinv;
  T* gpv = (T*)a.gp;
  // per-warp scratch, one slot per observation of the warp's current point;
  // one more slot holds per-point sums
  using SL = Slot<K>;
  constexpr int KK = SL::KK;
  T* wsc = (T*)a.wscratch + ((int64_t)blockIdx.x * kWarps + warp) * (int64_t)(a.max_views + 1) * SL::kSize;
  // global slice: column norms [kNMax], gradient [kNMax], rhs [kNMax], S (FP64)
  double* gsl = a.gscr + (int64_t)blockIdx.x * kGlobalSlice;
  double* g_acc = gsl;
  double* g_grad = gsl + kNMax;
  double* g_rhs = gsl + 2 * kNMax;
  double* g_S = gsl + 3 * kNMax;
  // S and rhs accessors: shared memory in FP32, the global slice (through L2:
  // global reductions do not update L1) in FP64
  auto Sld = [&](int i) -> SS {
    if constexpr (kGS) return (SS)__ldcg(g_S + i);
    else return sh.S[i];
  };
  auto Sst = [&](int i, SS v) {
    if constexpr (kGS) __stcg(g_S + i, (double)v);
    else sh.S[i] = v;
  };
  // Fixed-point accumulation of the Schur build (scales set before each
  // build): S as int64 in the global slice (FP64) or int32 in shared memory
  // (FP32), scaled per column pair; rhs, the column norms (Nadd) and the
  // gradient (Gadd) of the scaled Jacobian as int64 in the global slice
  // (FP64) or in shared memory (FP32), one scale each.  FP32 scales as
  // factors, FP64 ones as exponents (integer rounding).
  float fxf[4] = {1.f, 1.f, 1.f, 1.f};  // the FP32 path's copy of the vector scales
  int fxk[4] = {0, 0, 0, 0};            // the FP64 path's copy of their exponents
  // a column's factor of S's scale (a register copy: the atomics below
  // keep the compiler from reusing a shared-memory load)
  struct ColScale {
    SS s;
    int e;
  };
  auto cscale = [&](int i) -> ColScale {
    if constexpr (kGS) return {SS(0), sh.fxe[i]};
    else return {sh.fxs[i], 0};
  };
  // S_ij (i >= j) += v, scaled by the columns' factors
  auto Sadd_s = [&](int i, int j, SS v, ColScale fi, ColScale fj) {
    const int e = tri(i, j);
    if constexpr (kGS) fx_add(reinterpret_cast<long long*>(g_S + e), (double)v, fi.e + fj.e, &sh.fxbad);
    else atomicAdd(reinterpret_cast<int*>(&sh.S[e]), __float2int_rn((float)v * (fi.s * fj.s)));
  };
  auto Sadd = [&](int i, int j, SS v) { Sadd_s(i, j, v, cscale(i), cscale(j)); };
  auto Nadd = [&](int i, T v) {
    if constexpr (kGS) fx_add(reinterpret_cast<long long*>(g_acc + i), (double)v, fxk[1], &sh.fxbad);
    else {
      if (!isfinite((float)v)) atomicOr(&sh.fxbad, 2);
      fx_add(&sh.fxv[1][i], (float)v, fxf[1]);
    }
  };
  auto Gadd = [&](int i, T v) {
    if constexpr (kGS) fx_add(reinterpret_cast<long long*>(g_grad + i), (double)v, fxk[2], &sh.fxbad);
    else fx_add(&sh.fxv[2][i], (float)v, fxf[2]);
  };
  auto Radd = [&](int i, SS v) {
    if constexpr (kGS) fx_add(reinterpret_cast<long long*>(g_rhs + i), (double)v, fxk[3], &sh.fxbad);
    else fx_add(&sh.fxv[0][i], (float)v, fxf[3]);
  };

  const bool use_pose = P.nc <= (uint32_t)kPoseCams;
  // reduced column of camera c's extrinsic parameter j (-1 = held)
  auto ecol = [&](uint32_t c, int j) -> int {
    return use_pose ? sh.ecol[6 * (c - P.c0) + j] : a.ext_col[6 * (int64_t)c + j];
  };
  // The 6x6 extrinsic block of S for observations u (camera cu) and w (camera
  // cw <= cu) of one point: -(W V^-1)_u W_w^T, plus U_ee = Jc_e^T Jc_e when u
  // is the observation's own pair; a diagonal block keeps its lower triangle.
  auto ext_block = [&](const T* base, uint32_t u, uint32_t w, uint32_t cu, uint32_t cw, bool own) {
    const T* Su = base + (int64_t)u * SL::kSize;
    const T* Sw = base + (int64_t)w * SL::kSize;
    int ci[6], cj[6];
    ColScale fi[6], fj[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      ci[j] = ecol(cu, j);
      cj[j] = ecol(cw, j);
      fi[j] = ci[j] >= 0 ? cscale(ci[j]) : ColScale{};
      fj[j] = cj[j] >= 0 ? cscale(cj[j]) : ColScale{};
    }
    // W_w (and for an observation's own pair its Jc_e) in registers; the
    // rows of (W V^-1)_u are read as they are used (FP64: register budget)
    T ww[18], j0[6], j1[6];
    ld18<T>(Sw + SL::kW, ww);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      j0[j] = own ? Sw[SL::kJ + j] : T(0);
      j1[j] = own ? Sw[SL::kJ + B + j] : T(0);
    }
    T hu[18];
    if constexpr (sizeof(T) == 4) ld18<T>(Su + SL::kWh, hu);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (ci[i] < 0) continue;
      if constexpr (sizeof(T) != 4) {
#pragma unroll
        for (int k = 0; k < 3; ++k) hu[3 * i + k] = Su[SL::kWh + 3 * i + k];
      }
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        if (cj[j] < 0 || cj[j] > ci[i]) continue;
        const T s = j0[i] * j0[j] + j1[i] * j1[j] -
                    (hu[3 * i] * ww[3 * j] + hu[3 * i + 1] * ww[3 * j + 1] + hu[3 * i + 2] * ww[3 * j + 2]);
        Sadd_s(ci[i], cj[j], (SS)s, fi[i], fj[j]);
      }
    }
  };
  // residual cache (FP32 path): slot `cur` holds the current parameters'
  constexpr bool kCache = sizeof(T) == 4;
  int cur = 0;
  auto rc_cur = [&]() -> const float4* { return kCache ? a.rcache + (int64_t)cur * a.total_obs : nullptr; };
  // FP32 path: FP32 copies of the window's parameters (ext, intr, pts)
  auto make_f32 = [&](const double* ext, const double* intr, const double* pts) {
    if constexpr (kCache) {
      for (uint32_t i = tid; i < 6 * P.nc; i += kThreads) a.ext_f[6 * (int64_t)P.c0 + i] = (float)ext[6 * (int64_t)P.c0 + i];
      for (uint32_t i = tid; i < K * P.ni; i += kThreads) a.intr_f[K * (int64_t)P.g0 + i] = (float)intr[K * (int64_t)P.g0 + i];
      for (uint32_t i = tid; i < 3 * (P.x1 - P.x0); i += kThreads)
        a.pts_f[3 * (int64_t)P.x0 + i] = (float)pts[3 * (int64_t)P.x0 + i];
    }
  };
  // scales in the compute type
  auto csc = [&](int i) -> T {
    if constexpr (kCache) return sh.scale_cf[i];
    else return sh.scale_c[i];
  };
  auto psc = [&](uint32_t p, int j) -> T {
    if constexpr (kCache) return a.scale_pf[3 * (int64_t)p + j];
    else return a.scale_p[3 * (int64_t)p + j];
  };
  // poses of ext (slot 0) or ext2 (slot 1); the barrier makes them visible
  auto make_poses = [&](const double* ext, int slot) {
    if (use_pose) {
      for (uint32_t c = tid; c < P.nc; c += kThreads) {
        double E[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) E[i] = ext[6 * ((int64_t)P.c0 + c) + i];
        pose_matrix<double>(E, &sh.pose[slot][12 * c]);
      }
    }
    __syncthreads();
  };
  auto cost_at = [&](const double* ext, const double* intr, const double* pts, bool* finite) -> double {
    const double* pz = !use_pose ? nullptr : ext == a.ext ? sh.pose[0] : sh.pose[1];
    float4* wc = kCache ? a.rcache + (int64_t)(ext == a.ext ? cur : cur ^ 1) * a.total_obs : nullptr;
    double acc = 0.0;
    // one thread per observation: the cost needs no per-point sums
    const uint32_t oz = a.pt_off[P.x1];
    for (uint32_t o = a.pt_off[P.x0] + tid; o < oz; o += kThreads) {
      const uint32_t p = a.pt_s[o], c = a.cam[o], g = a.icam[o];
      double E[6], Kp[K], X[3], r[2], dJe[2][6], dJk[2][K], dJx[2][3];
      for (int i = 0; i < 6; ++i) E[i] = ext[6 * (int64_t)c + i];
      for (int i = 0; i < K; ++i) Kp[i] = intr[K * (int64_t)g + i];
      for (int i = 0; i < 3; ++i) X[i] = pts[3 * (int64_t)p + i];
      const double2 ob = a.obs[o];
      if (pz) residual_pose<M, double>(Kp, pz + 12 * (c - P.c0), X, ob.x, ob.y, r);
      else residual<M, double, false>(Kp, E, X, ob.x, ob.y, r, dJe, dJk, dJx, (double*)nullptr);
      double sr1;
      acc += robust<double>(a.loss_type, a.loss_a, r[0] * r[0] + r[1] * r[1], &sr1);
      if (wc) wc[o] = make_float4((float)(r[0] * sr1), (float)(r[1] * sr1), (float)sr1, 0.f);
    }
    const double c = block_sum(acc, sh.red, &sh.bcast[0]);
    *finite = isfinite(c);
    return c;
  };

  // norm of the variable parameters (parameter tolerance)
  auto param_norm = [&]() -> double {
    double xs = 0.0;
    for (uint32_t i = tid; i < 6 * P.nc; i += kThreads) {
      const int64_t j = 6 * (int64_t)P.c0 + i;
      if (a.ext_col[j] >= 0) xs += a.ext[j] * a.ext[j];
    }
    for (uint32_t i = tid; i < K * P.ni; i += kThreads) {
      const int64_t j = K * (int64_t)P.g0 + i;
      if (a.intr_var[j / K]) xs += a.intr[j] * a.intr[j];
    }
    for (uint32_t i = tid; i < 3 * (P.x1 - P.x0); i += kThreads) {
      const double v = a.pts[3 * (int64_t)P.x0 + i];
      xs += v * v;
    }
    return sqrt(block_sum(xs, sh.red, &sh.bcast[2]));
  };
  // Jacobi scale (first) and gradient max norm at the current parameters.
  // After the first linearisation the Schur build forms the LM diagonal and
  // the gradient from its own Jacobian; this pass only runs again to check
  // the gradient of an accepted last step at the iteration limit.
  auto linearize = [&](bool first) -> double {
    // Column norms and gradient are fixed-point sums (order-independent).
    // Pass 1 finds the largest single term of each, which with the window's
    // observation count bounds every partial sum; pass 2 accumulates.
    double mc = 0.0, mg = 0.0;
    for (uint32_t p = P.x0 + warp; p < P.x1; p += kWarps) {
      for (uint32_t o = a.pt_off[p] + lane; o < a.pt_off[p + 1]; o += 32) {
        T rr[2], Jc[2][B], Jp[2][3];
        int col[B];
        obs_lin<M, T>(a, o, p, rc_cur(), rr, Jc, Jp, col);
#pragma unroll
        for (int j = 0; j < B; ++j) {
          if (col[j] < 0) continue;
          const double x0 = Jc[0][j], x1 = Jc[1][j];
          mc = fmax(mc, x0 * x0 + x1 * x1);
          mg = fmax(mg, fabs(x0 * (double)rr[0] + x1 * (double)rr[1]));
        }
      }
    }
    mc = block_max(mc, sh.red, &sh.bcast[5]);
    mg = block_max(mg, sh.red, &sh.bcast[6]);
    const double nobs = (double)(a.pt_off[P.x1] - a.pt_off[P.x0]);
    const int kc = pow2_exp(mc * nobs, 62, 1000), kg = pow2_exp(mg * nobs, 62, 1000);
    for (int i = tid; i < n; i += kThreads) {
      __stcg(reinterpret_cast<long long*>(g_acc + i), 0ll);
      __stcg(reinterpret_cast<long long*>(g_grad + i), 0ll);
    }
    __syncthreads();
    double gm = 0.0;
    for (uint32_t p = P.x0 + warp; p < P.x1; p += kWarps) {
      double cp[3] = {0, 0, 0}, gp3[3] = {0, 0, 0};
      for (uint32_t o = a.pt_off[p] + lane; o < a.pt_off[p + 1]; o += 32) {
        T rr[2], Jc[2][B], Jp[2][3];
        int col[B];
        obs_lin<M, T>(a, o, p, rc_cur(), rr, Jc, Jp, col);
        const double r[2] = {(double)rr[0], (double)rr[1]};
#pragma unroll
        for (int j = 0; j < B; ++j) {
          if (col[j] < 0) continue;
          const double x0 = Jc[0][j], x1 = Jc[1][j];
          fx_add(reinterpret_cast<long long*>(g_acc + col[j]), x0 * x0 + x1 * x1, kc, &sh.fxbad);
          fx_add(reinterpret_cast<long long*>(g_grad + col[j]), x0 * r[0] + x1 * r[1], kg, &sh.fxbad);
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const double x0 = Jp[0][j], x1 = Jp[1][j];
          cp[j] += x0 * x0 + x1 * x1;
          gp3[j] += x0 * r[0] + x1 * r[1];
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        cp[j] = warp_sum(cp[j]);
        gp3[j] = warp_sum(gp3[j]);
      }
      if (lane < 3) {
        const double c = lane == 0 ? cp[0] : lane == 1 ? cp[1] : cp[2];
        if (first) {
          const double sc = a.jacobi ? 1.0 / (1.0 + sqrt(c)) : 1.0;
          a.scale_p[3 * (int64_t)p + lane] = sc;
          if constexpr (kCache) a.scale_pf[3 * (int64_t)p + lane] = (float)sc;
        }
        gm = fmax(gm, fabs(lane == 0 ? gp3[0] : lane == 1 ? gp3[1] : gp3[2]));
      }
    }
    __syncthreads();
    for (int i = tid; i < n; i += kThreads) {
      __stcg(g_acc + i, ldexp((double)__ldcg(reinterpret_cast<const long long*>(g_acc + i)), -kc));
      __stcg(g_grad + i, ldexp((double)__ldcg(reinterpret_cast<const long long*>(g_grad + i)), -kg));
    }
    __syncthreads();
    for (int i = tid; i < n; i += kThreads) {
      if (first) {
        sh.scale_c[i] = a.jacobi ? 1.0 / (1.0 + sqrt(__ldcg(g_acc + i))) : 1.0;
        sh.scale_cf[i] = (float)sh.scale_c[i];
      }
      gm = fmax(gm, fabs(__ldcg(g_grad + i)));
    }
    return block_max(gm, sh.red, &sh.bcast[1]);
  };

  // the window's column maps, fixed for the whole solve (made visible by make_poses' barrier)
  if (use_pose)
    for (uint32_t i = tid; i < 6 * P.nc; i += kThreads) sh.ecol[i] = a.ext_col[6 * (int64_t)P.c0 + i];
  if (tid < 8) sh.kcol[tid] = P.ni == 1 && tid < K ? a.intr_col[K * (int64_t)P.g0 + tid] : -1;
  make_f32(a.ext, a.intr, a.pts);
  bool finite = true;
  make_poses(a.ext, 0);
  double cost = cost_at(a.ext, a.intr, a.pts, &finite);
  BOut res;
  res.initial_cost = cost;
  res.final_cost = cost;
  res.iterations = res.successful = res.unsuccessful = 0;
  res.status = 0;
  if (!finite) {
    if (tid == 0) {
      res.termination = GBBA_FAILURE;
      res.usable = 0;
      res.status = GBBA_ERROR_NUMERICAL;
      a.out[pid] = res;
    }
    return;
  }
  {
    // the most observations of one point that touch one column: of one
    // camera (extrinsic columns; in a one-group window also the intrinsic
    // ones, whose terms are summed per point first) or of one intrinsic
    // group; S's sums stay below (1 + m) 2^fxbits
    int mult = 1;
    for (uint32_t p = P.x0 + warp; p < P.x1; p += kWarps) {
      const uint32_t ob = a.pt_off[p], oe = a.pt_off[p + 1];
      for (uint32_t x = ob + lane; x < oe; x += 32) {
        const uint32_t cx = a.cam[x], gx = a.icam[x];
        int nc = 0, ng = 0;
        for (uint32_t y = ob; y < oe; ++y) {
          nc += a.cam[y] == cx;
          ng += a.icam[y] == gx;
        }
        mult = max(mult, P.ni == 1 ? nc : max(nc, ng));
      }
    }
    mult = (int)block_max((double)mult, sh.red, &sh.bcast[7]);
    // one bit spare below int32 / int64
    if (tid == 0) sh.fxbits = (kGS ? 61 : 30) - (32 - __clz(mult));  // 32 - clz(m) = ceil(log2(1 + m))
    __syncthreads();
  }
  double gmax = linearize(true), xnorm = param_norm();
  {
    // bounds on the scaled column norms for the first build's fixed-point scales
    for (int i = tid; i < n; i += kThreads) sh.cbnd[i] = __ldcg(g_acc + i) * sh.scale_c[i] * sh.scale_c[i];
    __syncthreads();
  }
  bool check_grad = false;  // an accepted step's gradient is checked by the next Schur build
  int term = gmax <= a.gtol ? GBBA_CONVERGENCE : -1;
  double radius = a.r0, decrease = 2.0;
  int invalid = 0, iter = 0;
  while (term < 0) {
    if (iter >= a.max_iterations) {
      term = GBBA_NO_CONVERGENCE;
      if (check_grad && linearize(false) <= a.gtol) term = GBBA_CONVERGENCE;
      break;
    }
    // ---- S = sum F'F - sum (F'E) V^-1 (E'F) + diag(D_c^2), rhs, and from
    // the same Jacobian the column norms (LM diagonal) and the gradient, in
    // fixed point: S_ij scaled by 2^(e_i + e_j), e_i chosen for a column
    // norm of up to 4 cbnd[i] (col_exp gives the bound on S's sums); the
    // vectors with one scale for the window.  A build that finds a column
    // above its bound runs again.
    const double irad_d = 1.0 / radius;
    T gmt = T(0);  // gradient max norm (unscaled) over this thread's points
    double cover = 0.0;  // largest column norm / its bound of the last build
    for (int attempt = 0;; ++attempt) {
    {
      double cb = 0.0;
      for (int i = tid; i < n; i += kThreads) {
        const int e = col_exp(4.0 * sh.cbnd[i], sh.fxbits, kGS ? 500 : 60);
        sh.fxe[i] = e;
        sh.fxs[i] = (SS)ldexp(1.0, e);
        sh.fxi[i] = (SS)ldexp(1.0, -e);
        cb = fmax(cb, sh.cbnd[i]);
      }
      cb = block_max(cb, sh.red, &sh.bcast[7]);
      if (tid == 0) {
        const double G = 2.0 * sqrt(4.0 * cb * (2.0 * cost + 1e-300));
        const int lim = kGS ? 1000 : 120;
        sh.fxk[1] = pow2_exp(4.0 * cb, 60, lim);
        sh.fxk[2] = pow2_exp(G, 58, lim);
        sh.fxk[3] = pow2_exp(4.0 * G, 58, lim);
        for (int q = 1; q < 4; ++q) sh.fx[q] = ldexp(1.0, sh.fxk[q]);
        sh.flag = 0;
        sh.fxbad = 0;
      }
    }
    for (int i = tid; i < n * (n + 1) / 2; i += kThreads) Sst(i, SS(0));
    for (int i = tid; i < n; i += kThreads) {
      if constexpr (kGS) {
        __stcg(g_rhs + i, 0.0);
        __stcg(g_acc + i, 0.0);
        __stcg(g_grad + i, 0.0);
      } else {
        sh.fxv[0][i] = sh.fxv[1][i] = sh.fxv[2][i] = 0;
      }
    }
    gmt = T(0);
    __syncthreads();
#pragma unroll
    for (int q = 1; q < 4; ++q) {
      fxf[q] = (float)sh.fx[q];
      fxk[q] = sh.fxk[q];
    }
    // One intrinsic group per window (the local-BA case): the intrinsic
    // columns are common to every observation, so their terms factor through
    // per-point sums (no observation pairs):
    //   S_kk += sum_o U_kk - (sum_x W_kx V^-1)(sum_y W_ky)^T,
    //   S_k,c(y) += U_ke(y) - (sum_x W_kx V^-1) W_ey^T  (one lane per observation y),
    // and only the 6x6 extrinsic blocks need the observation pairs (one lane
    // per pair; an observation's own pair carries its U_ee).
    const bool one_group = P.ni == 1;
    const T irad = T(irad_d), dmin = (T)a.dmin, dmax = (T)a.dmax;
    for (uint32_t p = P.x0 + warp; p < P.x1; p += kWarps) {
      const uint32_t ob = a.pt_off[p], oe = a.pt_off[p + 1], m = oe - ob;
      const T sp[3] = {psc(p, 0), psc(p, 1), psc(p, 2)};
      T v[6] = {}, g[3] = {};
      for (uint32_t o = ob + lane; o < oe; o += 32) {
        T rr[2], Jc[2][B], Jp[2][3];
        int col[B];
        obs_lin<M, T>(a, o, p, rc_cur(), rr, Jc, Jp, col);
#pragma unroll
        for (int j = 0; j < B; ++j) {
          const T s = col[j] >= 0 ? csc(col[j]) : T(0);
          Jc[0][j] *= s;
          Jc[1][j] *= s;
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          Jp[0][j] *= sp[j];
          Jp[1][j] *= sp[j];
        }
        const T r0 = rr[0], r1 = rr[1];
        v[0] += Jp[0][0] * Jp[0][0] + Jp[1][0] * Jp[1][0];
        v[1] += Jp[0][0] * Jp[0][1] + Jp[1][0] * Jp[1][1];
        v[2] += Jp[0][0] * Jp[0][2] + Jp[1][0] * Jp[1][2];
        v[3] += Jp[0][1] * Jp[0][1] + Jp[1][1] * Jp[1][1];
        v[4] += Jp[0][1] * Jp[0][2] + Jp[1][1] * Jp[1][2];
        v[5] += Jp[0][2] * Jp[0][2] + Jp[1][2] * Jp[1][2];
#pragma unroll
        for (int j = 0; j < 3; ++j) g[j] += Jp[0][j] * r0 + Jp[1][j] * r1;
        T* W = wsc + (int64_t)(o - ob) * SL::kSize;
#pragma unroll
        for (int i = 0; i < B; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) W[SL::kW + i * 3 + j] = Jc[0][i] * Jp[0][j] + Jc[1][i] * Jp[1][j];
#pragma unroll
        for (int i = 0; i < B; ++i) {
          W[SL::kJ + i] = Jc[0][i];
          W[SL::kJ + B + i] = Jc[1][i];
        }
        // column norms and gradient of the scaled Jacobian (the intrinsic
        // columns of a one-group window through the per-point sums: every
        // observation shares them)
#pragma unroll
        for (int j = 0; j < B; ++j) {
          if (col[j] < 0) continue;
          const T x0 = Jc[0][j], x1 = Jc[1][j];
          if (one_group && j >= 6) {
            W[SL::kG + (j - 6)] = x0 * r0 + x1 * r1;
            continue;
          }
          Nadd(col[j], x0 * x0 + x1 * x1);
          Gadd(col[j], x0 * r0 + x1 * r1);
        }
        if (one_group) {
          // the observation's U_kk lower triangle (held columns are skipped at the reduction)
#pragma unroll
          for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j <= i; ++j)
              W[SL::kU + i * (i + 1) / 2 + j] = Jc[0][6 + i] * Jc[0][6 + j] + Jc[1][6 + i] * Jc[1][6 + j];
        } else {
#pragma unroll
          for (int i = 0; i < B; ++i) {
            const int ci = col[i];
            if (ci < 0) continue;
#pragma unroll
            for (int j = 0; j <= i; ++j) {
              const int cj = col[j];
              if (cj < 0) continue;
              const T u = Jc[0][i] * Jc[0][j] + Jc[1][i] * Jc[1][j];
              Sadd(max(ci, cj), min(ci, cj), (SS)u);
            }
          }
        }
      }
#pragma unroll
      for (int i = 0; i < 6; ++i) v[i] = warp_sum(v[i]);
#pragma unroll
      for (int i = 0; i < 3; ++i) g[i] = warp_sum(g[i]);
#pragma unroll
      for (int j = 0; j < 3; ++j) gmt = fmax(gmt, fabs(g[j] / sp[j]));
      // point block damped by its own LM diagonal clamp(diag V) / radius
      const T a00 = v[0] + fmin(fmax(v[0], dmin), dmax) * irad, a11 = v[3] + fmin(fmax(v[3], dmin), dmax) * irad,
              a22 = v[5] + fmin(fmax(v[5], dmin), dmax) * irad;
      const T l00 = sqrt(a00), l10 = v[1] / l00, l20 = v[2] / l00;
      const T d1 = a11 - l10 * l10;
      const T l11 = sqrt(d1), l21 = (v[4] - l20 * l10) / l11;
      const T d2 = a22 - l20 * l20 - l21 * l21;
      const T l22 = sqrt(d2);
      const T i00 = T(1) / l00, i11 = T(1) / l11, i22 = T(1) / l22;
      const T i10 = -l10 * i00 * i11, i21 = -l21 * i11 * i22, i20 = -(l20 * i00 + l21 * i10) * i22;
      const T vi[6] = {i00 * i00 + i10 * i10 + i20 * i20, i10 * i11 + i20 * i21, i20 * i22,
                       i11 * i11 + i21 * i21, i21 * i22, i22 * i22};
      if (!(a00 > T(0)) || !(d1 > T(0)) || !(d2 > T(0)) || !isfinite((double)vi[0])) sh.flag = 2;
      if (lane == 0) {
#pragma unroll
        for (int i = 0; i < 6; ++i) Vinv[6 * (int64_t)p + i] = vi[i];
#pragma unroll
        for (int i = 0; i < 3; ++i) gpv[3 * (int64_t)p + i] = g[i];
      }
      const T Vf[3][3] = {{vi[0], vi[1], vi[2]}, {vi[1], vi[3], vi[4]}, {vi[2], vi[4], vi[5]}};
      for (uint32_t o = ob + lane; o < oe; o += 32) {
        T* W = wsc + (int64_t)(o - ob) * SL::kSize;
        const uint32_t c = a.cam[o], gi = a.icam[o];
#pragma unroll
        for (int i = 0; i < B; ++i) {
          T y[3];
#pragma unroll
          for (int j = 0; j < 3; ++j)
            y[j] = W[SL::kW + i * 3] * Vf[0][j] + W[SL::kW + i * 3 + 1] * Vf[1][j] + W[SL::kW + i * 3 + 2] * Vf[2][j];
#pragma unroll
          for (int j = 0; j < 3; ++j) W[SL::kWh + i * 3 + j] = y[j];
          const T q = -(y[0] * g[0] + y[1] * g[1] + y[2] * g[2]);
          if (one_group && i >= 6) {
            W[SL::kQ + (i - 6)] = q;
            continue;
          }
          const int ci = i < 6 ? ecol(c, i) : a.intr_col[K * (int64_t)gi + (i - 6)];
          if (ci >= 0) Radd(ci, (SS)q);
        }
      }
      __syncwarp();
      if (one_group) {
        // per-point sums over the observations, Wh_K = sum W_k V^-1 and
        // W_K = sum W_k (K x 3 each), kept in the warp's extra scratch slot
        T* sums = wsc + (int64_t)a.max_views * SL::kSize;
        for (int e = lane; e < 3 * K; e += 32) {
          T hs = T(0), ws = T(0);
          for (uint32_t x = 0; x < m; ++x) {
            const T* Wx = wsc + (int64_t)x * SL::kSize;
            hs += Wx[SL::kWh + 18 + e];
            ws += Wx[SL::kW + 18 + e];
          }
          sums[e] = hs;
          sums[3 * K + e] = ws;
        }
        // the point's U_kk (its diagonal: the column norms), intrinsic rhs
        // correction and intrinsic gradient: sums over its observations' slots
        for (int e = lane; e < KK + 2 * K; e += 32) {
          T acc = T(0);
          for (uint32_t x = 0; x < m; ++x) acc += wsc[(int64_t)x * SL::kSize + SL::kU + e];
          if (e < KK) {
            int i = 0;
            while ((i + 1) * (i + 2) / 2 <= e) ++i;
            const int j = e - i * (i + 1) / 2;
            if (sh.kcol[i] >= 0 && sh.kcol[j] >= 0) {
              Sadd(sh.kcol[i], sh.kcol[j], (SS)acc);
              if (i == j) Nadd(sh.kcol[i], acc);
            }
          } else if (e < KK + K) {
            if (sh.kcol[e - KK] >= 0) Radd(sh.kcol[e - KK], (SS)acc);
          } else if (sh.kcol[e - KK - K] >= 0) {
            Gadd(sh.kcol[e - KK - K], acc);
          }
        }
        __syncwarp();
        // S_kk -= Wh_K W_K^T (lower triangle of the K x K block)
        for (int e = lane; e < KK; e += 32) {
          int i = 0;
          while ((i + 1) * (i + 2) / 2 <= e) ++i;
          const int j = e - i * (i + 1) / 2;
          const int ci = sh.kcol[i], cj = sh.kcol[j];
          if (ci < 0 || cj < 0) continue;
          const T sacc = sums[3 * i] * sums[3 * K + 3 * j] + sums[3 * i + 1] * sums[3 * K + 3 * j + 1] +
                         sums[3 * i + 2] * sums[3 * K + 3 * j + 2];
          Sadd(ci, cj, (SS)(-sacc));
        }
        // S_k,c(y) += U_ke(y) - Wh_K W_ey^T: one lane per observation y
        // (intrinsic columns follow every extrinsic column: lower triangle)
        for (uint32_t y = lane; y < m; y += 32) {
          const T* Wy = wsc + (int64_t)y * SL::kSize;
          const uint32_t cy = a.cam[ob + y];
          int cj[6];
#pragma unroll
          for (int j = 0; j < 6; ++j) cj[j] = ecol(cy, j);
          if (cj[0] < 0 && cj[1] < 0 && cj[2] < 0 && cj[3] < 0 && cj[4] < 0 && cj[5] < 0) continue;
          ColScale fj[6];
#pragma unroll
          for (int j = 0; j < 6; ++j) fj[j] = cj[j] >= 0 ? cscale(cj[j]) : ColScale{};
          T wy[18], j0[6], j1[6];
          ld18<T>(Wy + SL::kW, wy);
#pragma unroll
          for (int j = 0; j < 6; ++j) {
            j0[j] = Wy[SL::kJ + j];
            j1[j] = Wy[SL::kJ + B + j];
          }
#pragma unroll
          for (int i = 0; i < K; ++i) {
            const int ci = sh.kcol[i];
            if (ci < 0) continue;
            const T s0 = sums[3 * i], s1 = sums[3 * i + 1], s2 = sums[3 * i + 2];
            const T k0 = Wy[SL::kJ + 6 + i], k1 = Wy[SL::kJ + B + 6 + i];
            const ColScale fi = cscale(ci);
#pragma unroll
            for (int j = 0; j < 6; ++j) {
              if (cj[j] < 0) continue;
              const T val = k0 * j0[j] + k1 * j1[j] - (s0 * wy[3 * j] + s1 * wy[3 * j + 1] + s2 * wy[3 * j + 2]);
              Sadd_s(ci, cj[j], (SS)val, fi, fj[j]);
            }
          }
        }
        // extrinsic blocks: one lane per unordered observation pair x >= y
        const uint32_t nq = m * (m + 1) / 2;
        for (uint32_t q = lane; q < nq; q += 32) {
          uint32_t x = (uint32_t)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
          while ((x + 1) * (x + 2) / 2 <= q) ++x;
          while (x * (x + 1) / 2 > q) --x;
          const uint32_t y = q - x * (x + 1) / 2;
          const uint32_t cx = a.cam[ob + x], cy = a.cam[ob + y];
          if (cx >= cy) ext_block(wsc, x, y, cx, cy, x == y);
          else ext_block(wsc, y, x, cy, cx, false);
          if (cx == cy && x != y) ext_block(wsc, y, x, cy, cx, false);  // a camera that sees the point twice
        }
      } else {
        for (uint32_t x = 0; x < m; ++x) {
          const uint32_t oa = ob + x;
          const uint32_t ca = a.cam[oa], ga = a.icam[oa];
          const T* Wha = wsc + (int64_t)x * SL::kSize + SL::kWh;
          for (uint32_t y = 0; y < m; ++y) {
            const uint32_t obb = ob + y;
            const uint32_t cb = a.cam[obb], gb = a.icam[obb];
            const T* Wb = wsc + (int64_t)y * SL::kSize + SL::kW;
            for (int e = lane; e < B * B; e += 32) {
              const int i = e / B, j = e % B;
              const int ci = i < 6 ? ecol(ca, i) : a.intr_col[K * (int64_t)ga + (i - 6)];
              const int cj = j < 6 ? ecol(cb, j) : a.intr_col[K * (int64_t)gb + (j - 6)];
              if (ci < 0 || cj < 0 || cj > ci) continue;
              Sadd(ci, cj,
                   (SS)(-(Wha[3 * i] * Wb[3 * j] + Wha[3 * i + 1] * Wb[3 * j + 1] + Wha[3 * i + 2] * Wb[3 * j + 2])));
            }
          }
        }
      }
      __syncwarp();
    }
    __syncthreads();
    // the column norms against the bounds the build was scaled for; the
    // next build (this one again, or the next iteration's) takes the norms
    // found as its bounds
    {
      double cm = 0.0;
      for (int i = tid; i < n; i += kThreads) {
        const long long v = kGS ? __ldcg(reinterpret_cast<const long long*>(g_acc + i)) : sh.fxv[1][i];
        const double c = (double)v / sh.fx[1];
        const bool sat = v >= (1ll << 62) || v < 0;
        cm = fmax(cm, sat ? CUDART_INF : c / (4.0 * sh.cbnd[i]));
        sh.cbnd[i] = sat ? 65536.0 * sh.cbnd[i] + 1e-300 : c;
      }
      cover = block_max(cm, sh.red, &sh.bcast[7]);
      if (sh.fxbad & 1) cover = CUDART_INF;
    }
    // (a point block that failed to factor, or a Jacobian that is not
    // finite, invalidates the step whatever the scales)
    if (cover <= 1.0 || attempt >= 16 || sh.flag != 0 || (sh.fxbad & 2)) break;
    }  // build attempts
    if ((cover > 1.0 || (sh.fxbad & 2)) && tid == 0 && sh.flag == 0) sh.flag = 4;  // the step is invalid
    // back to floating point: S in place, a row per warp
    for (int i = warp; i < n; i += kWarps) {
      const SS si = sh.fxi[i];
      for (int j = lane; j <= i; j += 32) {
        const SS inv = si * sh.fxi[j];  // a power of two: exact
        if constexpr (kGS)
          __stcg(g_S + tri(i, j), (double)__ldcg(reinterpret_cast<const long long*>(g_S + tri(i, j))) * inv);
        else
          sh.S[tri(i, j)] = (float)(*reinterpret_cast<const int*>(&sh.S[tri(i, j)])) * inv;
      }
    }
    __syncthreads();
    // LM diagonal D_c^2 = clamp(column norms), rhs = gradient + Schur
    // correction, gradient max norm of this linearisation
    double gm = (double)gmt;
    for (int i = tid; i < n; i += kThreads) {
      long long vr, vn, vg;
      if constexpr (kGS) {
        vr = __ldcg(reinterpret_cast<const long long*>(g_rhs + i));
        vn = __ldcg(reinterpret_cast<const long long*>(g_acc + i));
        vg = __ldcg(reinterpret_cast<const long long*>(g_grad + i));
      } else {
        vr = sh.fxv[0][i];
        vn = sh.fxv[1][i];
        vg = sh.fxv[2][i];
      }
      const double acc = (double)vn / sh.fx[1];
      const double gi = (double)vg / sh.fx[2];
      const double d = fmin(fmax(acc, a.dmin), a.dmax);
      sh.diag_c[i] = d;
      Sst(tri(i, i), Sld(tri(i, i)) + (SS)(d / radius));
      sh.rhs[i] = (SS)(gi + (double)vr / sh.fx[3]);
      gm = fmax(gm, fabs(gi / sh.scale_c[i]));
    }
    gmax = block_max(gm, sh.red, &sh.bcast[1]);
    // ceres checks the gradient right after an accepted step
    if (check_grad) {
      check_grad = false;
      if (gmax <= a.gtol) {
        term = GBBA_CONVERGENCE;
        break;
      }
    }
    // ---- Cholesky of S (outer-product elimination, one barrier per column)
    for (int j = 0; j < n; ++j) {
      SS d = Sld(tri(j, j));
      if (!(d > SS(0)) || !isfinite((double)d)) {
        d = SS(1);
        if (tid == 0) {
          sh.flag = 1;
          Sst(tri(j, j), d);
        }
      }
      const SS invd = SS(1) / d;
      // trailing update of the lower triangle: rows by warp, columns by lane
      for (int i = j + 1 + warp; i < n; i += kWarps) {
        const SS sij = Sld(tri(i, j)) * invd;
        const int ri = tri(i, 0);
        for (int l = j + 1 + lane; l <= i; l += 32) Sst(ri + l, Sld(ri + l) - sij * Sld(tri(l, j)));
      }
      __syncthreads();
    }
    for (int j = tid; j < n; j += kThreads) sh.z[j] = sqrt(Sld(tri(j, j)));
    __syncthreads();
    for (int i = warp; i < n; i += kWarps) {
      const int ri = tri(i, 0);
      for (int j = lane; j < i; j += 32) Sst(ri + j, Sld(ri + j) / sh.z[j]);
    }
    __syncthreads();
    for (int j = tid; j < n; j += kThreads) Sst(tri(j, j), sh.z[j]);
    __syncthreads();
    // forward L y = rhs (column oriented), then backward L^T z = y; z holds the solution
    for (int j = 0; j < n; ++j) {
      const SS yj = sh.rhs[j] / Sld(tri(j, j));
      for (int i = j + 1 + tid; i < n; i += kThreads) sh.rhs[i] -= Sld(tri(i, j)) * yj;
      __syncthreads();
      if (tid == 0) sh.rhs[j] = yj;
      __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {
      const SS xj = sh.rhs[j] / Sld(tri(j, j));
      for (int i = tid; i < j; i += kThreads) sh.rhs[i] -= Sld(tri(j, i)) * xj;
      __syncthreads();
      if (tid == 0) sh.z[j] = xj;
      __syncthreads();
    }
    // camera step in the original parameterisation
    for (int j = tid; j < n; j += kThreads) sh.zs[j] = (SS)((double)sh.z[j] * sh.scale_c[j]);
    __syncthreads();
    // ---- back substitution, model cost change, candidate points.  The
    // first pass over a point's observations keeps each one's Jc z, residual
    // and Jp in its scratch slot for the second pass.
    double mcc = 0.0, stp = 0.0;
    for (uint32_t p = P.x0 + warp; p < P.x1; p += kWarps) {
      const uint32_t ob = a.pt_off[p], oe = a.pt_off[p + 1];
      const T sp[3] = {psc(p, 0), psc(p, 1), psc(p, 2)};
      T t[3] = {};
      for (uint32_t o = ob + lane; o < oe; o += 32) {
        T rr[2], Jc[2][B], Jp[2][3];
        int col[B];
        obs_lin<M, T>(a, o, p, rc_cur(), rr, Jc, Jp, col);
        T f0 = T(0), f1 = T(0);
#pragma unroll
        for (int i = 0; i < B; ++i) {
          if (col[i] < 0) continue;
          const T zi = sh.zs[col[i]];
          f0 += Jc[0][i] * zi;
          f1 += Jc[1][i] * zi;
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) t[j] += (Jp[0][j] * f0 + Jp[1][j] * f1) * sp[j];
        T* d = wsc + (int64_t)(o - ob) * SL::kSize;
        d[0] = f0;
        d[1] = f1;
        d[2] = rr[0];
        d[3] = rr[1];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          d[4 + j] = Jp[0][j];
          d[7 + j] = Jp[1][j];
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) t[j] = warp_sum(t[j]);
      const T* vi = Vinv + 6 * (int64_t)p;
      const T q0 = gpv[3 * (int64_t)p] - t[0], q1 = gpv[3 * (int64_t)p + 1] - t[1], q2 = gpv[3 * (int64_t)p + 2] - t[2];
      const T y[3] = {vi[0] * q0 + vi[1] * q1 + vi[2] * q2, vi[1] * q0 + vi[3] * q1 + vi[4] * q2,
                      vi[2] * q0 + vi[4] * q1 + vi[5] * q2};
      if (!isfinite((double)y[0]) || !isfinite((double)y[1]) || !isfinite((double)y[2])) sh.flag = 3;
      const T ys[3] = {y[0] * sp[0], y[1] * sp[1], y[2] * sp[2]};
      // model cost change: each term in the compute type, the sum in FP64
      for (uint32_t o = ob + lane; o < oe; o += 32) {
        const T* d = wsc + (int64_t)(o - ob) * SL::kSize;
        const T m0 = -(d[0] + d[4] * ys[0] + d[5] * ys[1] + d[6] * ys[2]);
        const T m1 = -(d[1] + d[7] * ys[0] + d[8] * ys[1] + d[9] * ys[2]);
        mcc += (double)(-(m0 * (d[2] + m0 / T(2)) + m1 * (d[3] + m1 / T(2))));
      }
      if (lane < 3) {
        const double dx = -(double)(lane == 0 ? y[0] : lane == 1 ? y[1] : y[2]) * a.scale_p[3 * (int64_t)p + lane];
        a.pts2[3 * (int64_t)p + lane] = a.pts[3 * (int64_t)p + lane] + dx;
        stp += dx * dx;
      }
      __syncwarp();
    }
    for (uint32_t i = tid; i < 6 * P.nc; i += kThreads) {
      const int64_t j = 6 * (int64_t)P.c0 + i;
      const int col = a.ext_col[j];
      const double d = col >= 0 ? -(double)sh.z[col] * sh.scale_c[col] : 0.0;
      a.ext2[j] = a.ext[j] + d;
      stp += d * d;
    }
    for (uint32_t i = tid; i < K * P.ni; i += kThreads) {
      const int64_t j = K * (int64_t)P.g0 + i;
      const int col = a.intr_col[j];
      const double d = col >= 0 ? -(double)sh.z[col] * sh.scale_c[col] : 0.0;
      a.intr2[j] = a.intr[j] + d;
      stp += d * d;
    }
    mcc = block_sum(mcc, sh.red, &sh.bcast[3]);
    stp = block_sum(stp, sh.red, &sh.bcast[4]);
    __threadfence_block();
    make_poses(a.ext2, 1);
    bool cfinite = true;
    const double new_cost_raw = cost_at(a.ext2, a.intr2, a.pts2, &cfinite);
    ++iter;
    // ---- step evaluation (TrustRegionMinimizer), identical in every thread
    const bool solved = sh.flag == 0;
    const bool valid = solved && isfinite(mcc) && mcc >= 0.0;
    bool success = false;
    double rel = 0.0;
    if (!valid) {
      if (++invalid >= a.max_invalid) {
        term = GBBA_FAILURE;
        break;
      }
    } else {
      invalid = 0;
      const double new_cost = cfinite ? new_cost_raw : 1.7976931348623157e308;
      if (sqrt(stp) <= a.ptol * (xnorm + a.ptol)) {
        term = GBBA_CONVERGENCE;
        break;
      }
      const double change = cost - new_cost;
      if (fabs(change) <= a.ftol * cost) {
        term = GBBA_CONVERGENCE;
        break;
      }
      rel = change / mcc;
      success = rel > a.min_rel;
      if (success) cost = new_cost;
    }
    if (success) {
      ++res.successful;
      const double f = 1.0 - (2.0 * rel - 1.0) * (2.0 * rel - 1.0) * (2.0 * rel - 1.0);
      radius = fmin(a.rmax, radius / fmax(1.0 / 3.0, f));
      decrease = 2.0;
      for (uint32_t i = tid; i < 3 * (P.x1 - P.x0); i += kThreads) a.pts[3 * (int64_t)P.x0 + i] = a.pts2[3 * (int64_t)P.x0 + i];
      for (uint32_t i = tid; i < 6 * P.nc; i += kThreads) a.ext[6 * (int64_t)P.c0 + i] = a.ext2[6 * (int64_t)P.c0 + i];
      for (uint32_t i = tid; i < K * P.ni; i += kThreads) a.intr[K * (int64_t)P.g0 + i] = a.intr2[K * (int64_t)P.g0 + i];
      if (use_pose)
        for (uint32_t i = tid; i < 12 * P.nc; i += kThreads) sh.pose[0][i] = sh.pose[1][i];
      make_f32(a.ext2, a.intr2, a.pts2);
      cur ^= 1;  // the candidate's residual cache becomes the current one
      __syncthreads();
      xnorm = param_norm();
      check_grad = true;
    } else {
      ++res.unsuccessful;
      radius /= decrease;
      decrease *= 2.0;
      if (radius < a.rmin) term = GBBA_CONVERGENCE;
    }
  }
  if (tid == 0) {
    res.termination = term;
    res.usable = term != GBBA_FAILURE ? 1 : 0;
    res.final_cost = cost;
    res.iterations = res.successful + res.unsuccessful;
    a.out[pid] = res;
  }
}

}  // namespace

// Host side of gbba_solve_batched.
gbba_status solve_batched_impl(gbba_handle* h, const gbba_problem* probs, int32_t np_, const gbba_options* o,
                               gbba_summary* sums) {
  const auto t0 = std::chrono::steady_clock::now();
  const int model = probs[0].camera_model;
  const int mem = probs[0].memory;
  const int k = model == kPinholeF ? 1 : model == kRadialK3 ? 6 : 8;
  const bool fp64 = o->precision == GBBA_PRECISION_FP64;
  const int nmax = kNMax;
  cudaStream_t st = h->active;
  // sizes, offsets and problem-local reduced column maps (host)
  std::vector<BProb> bp(np_);
  int64_t tc = 0, tg = 0, tx = 0, to = 0;
  for (int i = 0; i < np_; ++i) {
    const gbba_problem& P = probs[i];
    GBBA_REQUIRE(P.camera_model == model && P.memory == mem, GBBA_ERROR_INVALID_ARGUMENT,
                 "all problems of a batch must share the camera model and memory kind");
    bp[i].c0 = (uint32_t)tc; bp[i].nc = (uint32_t)P.num_cameras;
    bp[i].g0 = (uint32_t)tg; bp[i].ni = (uint32_t)P.num_intrinsics;
    bp[i].x0 = (uint32_t)tx; bp[i].x1 = (uint32_t)(tx + P.num_points);
    bp[i].o0 = (uint32_t)to; bp[i].o1 = (uint32_t)(to + P.num_observations);
    tc += P.num_cameras; tg += P.num_intrinsics; tx += P.num_points; to += P.num_observations;
  }
  GBBA_REQUIRE(to < 0xffffffffLL && tx < 0xffffffffLL, GBBA_ERROR_TOO_LARGE, "batch too large");
  auto host_copy = [&](void* dst, const void* src, size_t bytes) {
    if (!bytes) return;
    if (mem == GBBA_MEMORY_HOST) std::memcpy(dst, src, bytes);
    else GBBA_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  };
  // index arrays and column maps are assembled on the host (global indices)
  std::vector<uint32_t> cam(to), icam(to), pt(to);
  std::vector<int32_t> ecol(6 * tc, -1), icol(k * tg, -1);
  std::vector<uint8_t> ivar(tg, 0);
  int max_views = 1;
  for (int i = 0; i < np_; ++i) {
    const gbba_problem& P = probs[i];
    const int64_t no = P.num_observations;
    host_copy(&cam[bp[i].o0], P.camera_index, 4 * no);
    host_copy(&icam[bp[i].o0], P.intrinsic_index, 4 * no);
    host_copy(&pt[bp[i].o0], P.point_index, 4 * no);
    std::vector<uint8_t> cc(P.num_cameras, 0), ic(P.num_intrinsics, 0), cu(P.num_cameras, 0), iu(P.num_intrinsics, 0);
    if (P.camera_constant) host_copy(cc.data(), P.camera_constant, P.num_cameras);
    if (P.intrinsic_constant) host_copy(ic.data(), P.intrinsic_constant, P.num_intrinsics);
    std::vector<int> views(P.num_points, 0);
    for (int64_t q = 0; q < no; ++q) {
      uint32_t& c = cam[bp[i].o0 + q];
      uint32_t& g = icam[bp[i].o0 + q];
      uint32_t& x = pt[bp[i].o0 + q];
      GBBA_REQUIRE(c < P.num_cameras && g < P.num_intrinsics && x < P.num_points, GBBA_ERROR_INVALID_ARGUMENT,
                   "observation index out of range");
      cu[c] = 1;
      iu[g] = 1;
      max_views = std::max(max_views, ++views[x]);
      c += bp[i].c0;
      g += bp[i].g0;
      x += bp[i].x0;
    }
    int n = 0;
    for (int64_t c = 0; c < P.num_cameras; ++c) {
      if (!cu[c] || cc[c]) continue;
      for (int j = 0; j < 6; ++j)
        if (!(P.extrinsic_fixed_mask & (1u << j))) ecol[6 * (bp[i].c0 + c) + j] = n++;
    }
    for (int64_t g = 0; g < P.num_intrinsics; ++g) {
      if (!iu[g] || ic[g]) continue;
      for (int j = 0; j < k; ++j)
        if (!(P.intrinsic_fixed_mask & (1u << j))) {
          icol[k * (bp[i].g0 + g) + j] = n++;
          ivar[bp[i].g0 + g] = 1;
        }
    }
    GBBA_REQUIRE(n <= nmax, GBBA_ERROR_TOO_LARGE, "a batched problem's reduced camera system exceeds the per-CTA limit");
    bp[i].n = (uint32_t)n;
  }
  // problems ordered by observation count, largest first
  std::vector<uint32_t> order(np_);
  for (int i = 0; i < np_; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t x, uint32_t y) { return (bp[x].o1 - bp[x].o0) > (bp[y].o1 - bp[y].o0); });
  const int slot_values = k == 1 ? Slot<1>::kSize : k == 6 ? Slot<6>::kSize : Slot<8>::kSize;
  const size_t tsize = 8;  // FP64-sized: the mixed path ends with an FP64 polish
  Planner pl;
  auto plan = [&](auto& A) {
    struct Ptrs {
      double *ext, *intr, *pts, *ext2, *intr2, *pts2, *obs_in, *scale_p;
      double2* obs;
      uint32_t *cam, *icam, *pt, *cam_s, *icam_s, *counts, *off, *fill, *chunks, *perm, *order;
      int32_t *ecol, *icol;
      uint8_t* ivar;
      BProb* probs;
      BOut* out;
      void *Vinv, *gp, *wsc;
      double* gscr;
      float4* rcache;
      float *ext_f, *intr_f, *pts_f, *scale_pf;
      uint32_t* pt_s;
    } q;
    q.ext = A.template take<double>(6 * tc); q.intr = A.template take<double>(k * tg); q.pts = A.template take<double>(3 * tx);
    q.ext2 = A.template take<double>(6 * tc); q.intr2 = A.template take<double>(k * tg); q.pts2 = A.template take<double>(3 * tx);
    q.obs_in = A.template take<double>(2 * to); q.obs = A.template take<double2>(to);
    q.scale_p = A.template take<double>(3 * tx);
    q.cam = A.template take<uint32_t>(to); q.icam = A.template take<uint32_t>(to); q.pt = A.template take<uint32_t>(to);
    q.cam_s = A.template take<uint32_t>(to); q.icam_s = A.template take<uint32_t>(to);
    q.counts = A.template take<uint32_t>(tx + 1); q.off = A.template take<uint32_t>(tx + 1);
    q.fill = A.template take<uint32_t>(tx + 1); q.chunks = A.template take<uint32_t>(ceil_div(tx + 1, 1024) + 1);
    q.perm = A.template take<uint32_t>(to); q.order = A.template take<uint32_t>(np_);
    q.ecol = A.template take<int32_t>(6 * tc); q.icol = A.template take<int32_t>(k * tg); q.ivar = A.template take<uint8_t>(tg);
    q.probs = A.template take<BProb>(np_); q.out = A.template take<BOut>(2 * np_);
    q.Vinv = A.template take<char>(6 * tx * tsize); q.gp = A.template take<char>(3 * tx * tsize);
    q.wsc = A.template take<char>((size_t)np_ * kWarps * (max_views + 1) * slot_values * tsize);
    q.gscr = A.template take<double>((size_t)np_ * kGlobalSlice);
    q.rcache = A.template take<float4>((size_t)2 * std::max<int64_t>(to, 1));
    q.ext_f = A.template take<float>(6 * tc); q.intr_f = A.template take<float>(k * tg);
    q.pts_f = A.template take<float>(3 * tx); q.scale_pf = A.template take<float>(3 * tx);
    q.pt_s = A.template take<uint32_t>(to);
    return q;
  };
  plan(pl);
  h->arena.reset();
  h->arena.reserve(pl.used + 4096);
  auto q = plan(h->arena);
  // parameters and observations, packed
  std::vector<double> hbuf;
  auto upload_packed = [&](double* dst, int field_doubles, int64_t total, auto count_of, auto ptr_of) {
    if (mem == GBBA_MEMORY_DEVICE) {
      for (int i = 0; i < np_; ++i) {
        const int64_t cnt = count_of(i) * field_doubles;
        if (cnt) GBBA_CUDA(cudaMemcpyAsync(dst, ptr_of(i), 8 * cnt, cudaMemcpyDeviceToDevice, st));
        dst += cnt;
      }
      return;
    }
    hbuf.resize(total * field_doubles);
    int64_t w = 0;
    for (int i = 0; i < np_; ++i) {
      const int64_t cnt = count_of(i) * field_doubles;
      std::memcpy(&hbuf[w], ptr_of(i), 8 * cnt);
      w += cnt;
    }
    GBBA_CUDA(cudaMemcpyAsync(dst, hbuf.data(), 8 * w, cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
  };
  upload_packed(q.ext, 6, tc, [&](int i) { return probs[i].num_cameras; }, [&](int i) { return (const void*)probs[i].extrinsics; });
  upload_packed(q.intr, k, tg, [&](int i) { return probs[i].num_intrinsics; }, [&](int i) { return (const void*)probs[i].intrinsics; });
  upload_packed(q.pts, 3, tx, [&](int i) { return probs[i].num_points; }, [&](int i) { return (const void*)probs[i].points; });
  upload_packed(q.obs_in, 2, to, [&](int i) { return probs[i].num_observations; }, [&](int i) { return (const void*)probs[i].observations; });
  GBBA_CUDA(cudaMemcpyAsync(q.cam, cam.data(), 4 * to, cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.icam, icam.data(), 4 * to, cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.pt, pt.data(), 4 * to, cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.ecol, ecol.data(), 4 * ecol.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.icol, icol.data(), 4 * icol.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.ivar, ivar.data(), ivar.size(), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.probs, bp.data(), sizeof(BProb) * np_, cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemcpyAsync(q.order, order.data(), 4 * np_, cudaMemcpyHostToDevice, st));
  // sort observations by (global) point, input order kept inside a point
  std::vector<uint32_t> counts(tx + 1, 0);
  for (int64_t i = 0; i < to; ++i) counts[pt[i]]++;
  GBBA_CUDA(cudaMemcpyAsync(q.counts, counts.data(), 4 * (tx + 1), cudaMemcpyHostToDevice, st));
  GBBA_CUDA(cudaMemsetAsync(q.fill, 0, 4 * (tx + 1), st));
  scan_offsets(h, q.counts, q.off, tx, q.chunks, st);
  const int grid = std::max(1, std::min<int>((int)ceil_div(std::max<int64_t>(to, 1), 256), h->sm_count * 8));
  if (to > 0) {
    k_scatter<<<grid, 256, 0, st>>>(q.pt, to, q.off, q.fill, q.perm);
    check_launch(h);
    k_segment_sort<<<std::max(1, (int)std::min<int64_t>(ceil_div(tx, 256), h->sm_count * 8)), 256, 0, st>>>(q.perm, q.off, tx);
    check_launch(h);
  }
  // gather
  {
    std::vector<uint32_t> hperm(to);
    GBBA_CUDA(cudaMemcpyAsync(hperm.data(), q.perm, 4 * to, cudaMemcpyDeviceToHost, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    std::vector<uint32_t> c2(to), g2(to), p2(to);
    for (int64_t i = 0; i < to; ++i) {
      c2[i] = cam[hperm[i]];
      g2[i] = icam[hperm[i]];
      p2[i] = pt[hperm[i]];
    }
    GBBA_CUDA(cudaMemcpyAsync(q.cam_s, c2.data(), 4 * to, cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaMemcpyAsync(q.icam_s, g2.data(), 4 * to, cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaMemcpyAsync(q.pt_s, p2.data(), 4 * to, cudaMemcpyHostToDevice, st));
    std::vector<double> ob(2 * to);
    if (mem == GBBA_MEMORY_HOST) {
      for (int64_t i = 0; i < to; ++i) {
        ob[2 * i] = hbuf[2 * hperm[i]];
        ob[2 * i + 1] = hbuf[2 * hperm[i] + 1];
      }
    } else {
      std::vector<double> raw(2 * to);
      GBBA_CUDA(cudaMemcpyAsync(raw.data(), q.obs_in, 16 * to, cudaMemcpyDeviceToHost, st));
      GBBA_CUDA(cudaStreamSynchronize(st));
      for (int64_t i = 0; i < to; ++i) {
        ob[2 * i] = raw[2 * hperm[i]];
        ob[2 * i + 1] = raw[2 * hperm[i] + 1];
      }
    }
    GBBA_CUDA(cudaMemcpyAsync(q.obs, ob.data(), 16 * to, cudaMemcpyHostToDevice, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
  }
  BArgs a;
  a.probs = q.probs; a.order = q.order;
  a.ext = q.ext; a.intr = q.intr; a.pts = q.pts; a.ext2 = q.ext2; a.intr2 = q.intr2; a.pts2 = q.pts2;
  a.obs = q.obs; a.cam = q.cam_s; a.icam = q.icam_s; a.pt_off = q.off;
  a.ext_col = q.ecol; a.intr_col = q.icol; a.intr_var = q.ivar;
  a.scale_p = q.scale_p; a.Vinv = q.Vinv; a.gp = q.gp; a.wscratch = q.wsc; a.gscr = q.gscr;
  a.rcache = q.rcache; a.total_obs = to;
  a.ext_f = q.ext_f; a.intr_f = q.intr_f; a.pts_f = q.pts_f; a.scale_pf = q.scale_pf; a.pt_s = q.pt_s;
  a.max_views = max_views; a.out = q.out;
  a.max_iterations = o->max_num_iterations; a.max_invalid = o->max_num_consecutive_invalid_steps;
  a.jacobi = o->jacobi_scaling; a.loss_type = o->loss_type; a.loss_a = o->loss_scale;
  a.ftol = o->function_tolerance; a.gtol = o->gradient_tolerance; a.ptol = o->parameter_tolerance;
  a.r0 = o->initial_trust_region_radius; a.rmax = o->max_trust_region_radius; a.rmin = o->min_trust_region_radius;
  a.min_rel = o->min_relative_decrease; a.dmin = o->min_lm_diagonal; a.dmax = o->max_lm_diagonal;
  cudaEvent_t e0, e1;
  GBBA_CUDA(cudaEventCreate(&e0));
  GBBA_CUDA(cudaEventCreate(&e1));
  GBBA_CUDA(cudaEventRecord(e0, st));
  BArgs* base = &a;
  auto launch = [&](auto kern, size_t smem) {
    if (np_ <= 0) return;
    GBBA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<np_, kThreads, smem, st>>>(*base);
    check_launch(h);
  };
  // FP64: S in the global slice (small shared footprint); mixed: FP32 S in
  // shared memory
  const size_t sm64 = sizeof(SharedOf<double>::type), sm32 = sizeof(SharedOf<float>::type);
  if (fp64) {
    if (model == kPinholeF) launch(k_lm_batched<kPinholeF, double, double>, sm64);
    else if (model == kRadialK3) launch(k_lm_batched<kRadialK3, double, double>, sm64);
    else launch(k_lm_batched<kBrownT2, double, double>, sm64);
  } else {
    if (model == kPinholeF) launch(k_lm_batched<kPinholeF, float, float>, sm32);
    else if (model == kRadialK3) launch(k_lm_batched<kRadialK3, float, float>, sm32);
    else launch(k_lm_batched<kBrownT2, float, float>, sm32);
  }
  // Mixed path: the FP64 kernel continues from the mixed solution (its own
  // LM restart, at most fp64_polish_iterations iterations, tolerances 1000x
  // tighter), so that the final iterates carry FP64 Jacobians and steps and
  // end at the minimum rather than anywhere inside the stopping band
  // |dcost| <= 1e-6 cost.
  const bool polish = !fp64 && o->fp64_polish_iterations > 0;
  BArgs pol = a;
  if (polish) {
    pol.out = q.out + np_;
    pol.max_iterations = o->fp64_polish_iterations;
    pol.ftol = a.ftol * 1e-3;  // converge past ceres's 1e-6 stopping band
    pol.ptol = a.ptol * 1e-3;
    base = &pol;
    if (model == kPinholeF) launch(k_lm_batched<kPinholeF, double, double>, sm64);
    else if (model == kRadialK3) launch(k_lm_batched<kRadialK3, double, double>, sm64);
    else launch(k_lm_batched<kBrownT2, double, double>, sm64);
  }
  GBBA_CUDA(cudaEventRecord(e1, st));
  std::vector<BOut> out(2 * np_);
  GBBA_CUDA(cudaMemcpyAsync(out.data(), q.out, sizeof(BOut) * 2 * np_, cudaMemcpyDeviceToHost, st));
  // write back refined parameters of the usable problems
  std::vector<double> he(6 * tc), hi(k * tg), hx(3 * tx);
  GBBA_CUDA(cudaMemcpyAsync(he.data(), q.ext, 8 * he.size(), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaMemcpyAsync(hi.data(), q.intr, 8 * hi.size(), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaMemcpyAsync(hx.data(), q.pts, 8 * hx.size(), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  gbba_status status = GBBA_SUCCESS;
  for (int i = 0; i < np_; ++i) {
    if (polish && out[np_ + i].status == 0) {
      const BOut& f = out[np_ + i];
      out[i].final_cost = f.final_cost;
      out[i].iterations += f.iterations;
      out[i].successful += f.successful;
      out[i].unsuccessful += f.unsuccessful;
      if (f.termination != GBBA_FAILURE) {
        out[i].termination = f.termination;
        out[i].usable = 1;
      }
    }
    gbba_summary& s = sums[i];
    std::memset(&s, 0, sizeof(s));
    s.initial_cost = out[i].initial_cost;
    s.final_cost = out[i].final_cost;
    s.num_iterations = out[i].iterations;
    s.num_successful_steps = out[i].successful;
    s.num_unsuccessful_steps = out[i].unsuccessful;
    s.termination_type = out[i].termination;
    s.usable = out[i].usable;
    s.reduced_system_size = bp[i].n;
    s.total_time_s = total;
    s.linear_solver_time_s = ms * 1e-3;  // the whole batched launch
    if (out[i].status != 0 && status == GBBA_SUCCESS) status = (gbba_status)out[i].status;
    if (!s.usable) continue;
    const gbba_problem& P = probs[i];
    auto put = [&](double* dst, const double* src, size_t count) {
      if (!count) return;
      if (mem == GBBA_MEMORY_HOST) std::memcpy(dst, src, 8 * count);
      else GBBA_CUDA(cudaMemcpyAsync(dst, src, 8 * count, cudaMemcpyHostToDevice, st));
    };
    put(P.extrinsics, &he[6 * (int64_t)bp[i].c0], 6 * P.num_cameras);
    put(P.intrinsics, &hi[k * (int64_t)bp[i].g0], k * P.num_intrinsics);
    put(P.points, &hx[3 * (int64_t)bp[i].x0], 3 * P.num_points);
  }
  GBBA_CUDA(cudaStreamSynchronize(st));
  return status;
}

}  // namespace gbba
