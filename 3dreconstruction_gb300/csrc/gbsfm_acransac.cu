// AC-RANSAC hypothesis scoring (include/gbsfm.h, gbsfm_acransac_score): the
// per-model body of ACRANSAC's main loop
// (libs/feature/include/mvg/feature/estimator_acransac.h:170-200) for a batch
// of candidate resection models, one CTA per model:
//   1. the squared reprojection error of every correspondence
//      (ResectionSquaredResidualError, libs/sfm/include/mvg/sfm/sfm_robust.h:
//      197-204) as a 64-bit key (the bits of a non-negative double order like
//      the double) with the correspondence index as payload;
//   2. a bitonic sort of the (key, index) pairs in shared memory (a per-CTA
//      global slice above 8192 correspondences): the pairs are distinct, so
//      the result is std::sort's order of (error, index) pairs;
//   3. bestNFA (estimator_acransac.h:75-97) as a block-wide argmin over k,
//      the smallest k winning ties as the reference's strict '<' scan does.
// The logcombi tables (:40-65, float-rounded as the reference stores them)
// are built on the device from a table of log10(i), summed in the
// reference's order.
#include <math_constants.h>

#include <cfloat>
#include <cstring>

#include "../../include/gbsfm.h"
#include "gbba_internal.h"

namespace gbba {
namespace {

constexpr int kScoreThreads = 512;
constexpr int64_t kSmemPairs = 8192;  // 8192 x 12 B = 96 KB of keys and indices

__global__ void __launch_bounds__(256) k_log10_table(int64_t n, double* __restrict__ lg) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x)
    lg[i] = i > 0 ? log10((double)i) : 0.0;
}

// logcombi(k, n): 0 for k >= n or k <= 0, else the sum over i = 1..min(k, n-k)
// of log10(n - i + 1) - log10(i), in that order.
__device__ double logcombi(int64_t k, int64_t n, const double* __restrict__ lg) {
  if (k >= n || k <= 0) return 0.0;
  if (n - k < k) k = n - k;
  double r = 0.0;
  for (int64_t i = 1; i <= k; ++i) r += lg[n - i + 1] - lg[i];
  return r;
}

// logc_n[k] = logcombi(k, n), logc_k[m] = logcombi(sample_size, m), k, m in 0..n.
__global__ void __launch_bounds__(256) k_logcombi(int64_t n, int sample_size, const double* __restrict__ lg,
                                                  float* __restrict__ logc_n, float* __restrict__ logc_k) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
    logc_n[i] = (float)logcombi(i, n, lg);
    logc_k[i] = (float)logcombi(sample_size, i, lg);
  }
}

// |Project(P, X) - x|^2 with Project = (P [X; 1]).head(2) / z, the products
// and sums kept apart (no contraction) in the order of the matrix rows.
__device__ __forceinline__ double resection_error(const double* __restrict__ m, double X0, double X1, double X2,
                                                  double x, double y) {
  double h[3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    h[r] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[4 * r], X0), __dmul_rn(m[4 * r + 1], X1)),
                               __dmul_rn(m[4 * r + 2], X2)),
                     m[4 * r + 3]);
  const double dx = h[0] / h[2] - x, dy = h[1] / h[2] - y;
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

__device__ __forceinline__ bool pair_less(unsigned long long ka, uint32_t va, unsigned long long kb, uint32_t vb) {
  return ka < kb || (ka == kb && va < vb);
}

// Ascending bitonic sort of p (a power of two) pairs.
__device__ void bitonic_sort(unsigned long long* keys, uint32_t* vals, int64_t p) {
  for (int64_t size = 2; size <= p; size <<= 1) {
    for (int64_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (int64_t t = threadIdx.x; t < p / 2; t += blockDim.x) {
        const int64_t i = 2 * t - (t & (stride - 1));  // lower element of the t-th compared pair
        const int64_t j = i + stride;
        const bool up = (i & size) == 0;
        const unsigned long long ki = keys[i], kj = keys[j];
        const uint32_t vi = vals[i], vj = vals[j];
        if (pair_less(kj, vj, ki, vi) == up) {
          keys[i] = kj;
          keys[j] = ki;
          vals[i] = vj;
          vals[j] = vi;
        }
      }
      __syncthreads();
    }
  }
}

struct ScoreArgs {
  int64_t n, h, p;
  const double *x2d, *x3d, *models;
  const float *logc_n, *logc_k;
  int sample_size;
  double loge0, logalpha0, mult_error, max_threshold;
  double* nfa;
  int32_t* inliers;
  double* error_max;
  uint32_t* order;
  unsigned long long* scratch_keys;  // global slices when p > kSmemPairs
  uint32_t* scratch_vals;
};

__global__ void __launch_bounds__(kScoreThreads) k_acransac_score(ScoreArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double sh_model[12];
  __shared__ double sh_best[kScoreThreads / 32];
  __shared__ int64_t sh_best_k[kScoreThreads / 32];
  unsigned long long* keys;
  uint32_t* vals;
  if (a.p <= kSmemPairs) {
    keys = reinterpret_cast<unsigned long long*>(smem);
    vals = reinterpret_cast<uint32_t*>(smem + sizeof(unsigned long long) * a.p);
  } else {
    keys = a.scratch_keys + blockIdx.x * a.p;
    vals = a.scratch_vals + blockIdx.x * a.p;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t m = blockIdx.x; m < a.h; m += gridDim.x) {
    if (threadIdx.x < 12) sh_model[threadIdx.x] = a.models[12 * m + threadIdx.x];
    __syncthreads();
    for (int64_t i = threadIdx.x; i < a.p; i += blockDim.x) {
      if (i < a.n) {
        const double e = resection_error(sh_model, a.x3d[3 * i], a.x3d[3 * i + 1], a.x3d[3 * i + 2], a.x2d[2 * i],
                                         a.x2d[2 * i + 1]);
        // +0.0 for -0.0 so that the bit order is the double order
        keys[i] = (unsigned long long)__double_as_longlong(e + 0.0);
        vals[i] = (uint32_t)i;
      } else {
        keys[i] = ~0ull;
        vals[i] = 0xffffffffu;
      }
    }
    __syncthreads();
    bitonic_sort(keys, vals, a.p);
    // bestNFA: k = sample_size + 1 .. n while e[k-1] <= max_threshold
    double best = CUDART_INF;
    int64_t best_k = a.sample_size;
    for (int64_t k = a.sample_size + 1 + threadIdx.x; k <= a.n; k += blockDim.x) {
      const double e = __longlong_as_double((long long)keys[k - 1]);
      if (!(e <= a.max_threshold)) break;  // sorted: every later k fails too
      const double logalpha = a.logalpha0 + a.mult_error * log10(e + (double)FLT_MIN);
      const double v = a.loge0 + logalpha * (double)(k - a.sample_size) + (double)a.logc_n[k] + (double)a.logc_k[k];
      if (v < best) {  // k ascends per thread: the first of equal values stays
        best = v;
        best_k = k;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int64_t ok = __shfl_xor_sync(0xffffffffu, best_k, o);
      if (ob < best || (ob == best && ok < best_k)) {
        best = ob;
        best_k = ok;
      }
    }
    if (lane == 0) {
      sh_best[warp] = best;
      sh_best_k[warp] = best_k;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < kScoreThreads / 32; ++w)
        if (sh_best[w] < best || (sh_best[w] == best && sh_best_k[w] < best_k)) {
          best = sh_best[w];
          best_k = sh_best_k[w];
        }
      const bool found = best < CUDART_INF;
      a.nfa[m] = best;
      a.inliers[m] = (int32_t)(found ? best_k : a.sample_size);
      a.error_max[m] = found ? __longlong_as_double((long long)keys[best_k - 1]) : CUDART_INF;
    }
    if (a.order)
      for (int64_t i = threadIdx.x; i < a.n; i += blockDim.x) a.order[m * a.n + i] = vals[i];
    __syncthreads();
  }
}

int64_t next_pow2(int64_t n) {
  int64_t p = 2;
  while (p < n) p <<= 1;
  return p;
}

PerDeviceOnce g_score_smem;

}  // namespace
}  // namespace gbba

using namespace gbba;

extern "C" gbba_status gbsfm_acransac_score(gbba_handle* h, const gbsfm_acransac_params* prm, int64_t num_points,
                                            const double* x2d, const double* x3d, int64_t num_models,
                                            const double* models, double* nfa, int32_t* num_inliers,
                                            double* error_max, uint32_t* order, int32_t memory) {
  if (!prm || prm->sample_size < 1 || prm->max_models < 1 || num_models < 0 || num_points <= prm->sample_size)
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (num_models > 0 && (!x2d || !x3d || !models || !nfa || !num_inliers || !error_max))
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (num_points > 0x7fffffffLL) return GBBA_ERROR_TOO_LARGE;
  return sfm_guard(h, [&]() {
    if (num_models == 0) return GBBA_SUCCESS;
    const int64_t n = num_points, p = next_pow2(n);
    const unsigned grid = (unsigned)std::min<int64_t>(num_models, (int64_t)h->sm_count * 2);
    const bool in_smem = p <= kSmemPairs;
    const size_t smem = in_smem ? (size_t)p * (sizeof(unsigned long long) + sizeof(uint32_t)) : 0;
    const size_t scratch = in_smem ? 0 : (size_t)grid * p * (sizeof(unsigned long long) + sizeof(uint32_t));
    h->arena.reset();
    h->arena.reserve(sizeof(double) * (5 * n + 12 * num_models + 3 * num_models + n + 1) + 2 * sizeof(float) * (n + 1) +
                     sizeof(int32_t) * num_models + (order ? sizeof(uint32_t) * num_models * n : 0) + scratch +
                     256 * 16);
    ScoreArgs a;
    a.n = n;
    a.h = num_models;
    a.p = p;
    a.x2d = in_view(h, x2d, 2 * n, memory);
    a.x3d = in_view(h, x3d, 3 * n, memory);
    a.models = in_view(h, models, 12 * num_models, memory);
    a.nfa = out_view(h, nfa, num_models, memory);
    a.inliers = out_view(h, num_inliers, num_models, memory);
    a.error_max = out_view(h, error_max, num_models, memory);
    a.order = out_view(h, order, num_models * n, memory);
    double* lg = h->arena.take<double>(n + 1);
    float* logc_n = h->arena.take<float>(n + 1);
    float* logc_k = h->arena.take<float>(n + 1);
    a.logc_n = logc_n;
    a.logc_k = logc_k;
    a.scratch_keys = in_smem ? nullptr : h->arena.take<unsigned long long>(grid * p);
    a.scratch_vals = in_smem ? nullptr : h->arena.take<uint32_t>(grid * p);
    a.sample_size = prm->sample_size;
    // loge0 = log10(MAX_MODELS * (nData - sample_size)) (estimator_acransac.h:147)
    a.loge0 = log10((double)prm->max_models * (double)(n - prm->sample_size));
    a.logalpha0 = prm->logalpha0;
    a.mult_error = prm->mult_error;
    a.max_threshold = prm->max_threshold;
    if (in_smem && smem > 48 * 1024)
      g_score_smem.run([&]() {
        GBBA_CUDA(cudaFuncSetAttribute(k_acransac_score, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(kSmemPairs * (sizeof(unsigned long long) + sizeof(uint32_t)))));
      });
    KernelTimer timer(h);
    k_log10_table<<<grid_for(h, n + 1, 256), 256, 0, h->active>>>(n, lg);
    check_launch(h);
    k_logcombi<<<grid_for(h, n + 1, 256), 256, 0, h->active>>>(n, prm->sample_size, lg, logc_n, logc_k);
    check_launch(h);
    k_acransac_score<<<grid, kScoreThreads, smem, h->active>>>(a);
    check_launch(h);
    timer.stop();
    out_back(h, nfa, a.nfa, num_models, memory);
    out_back(h, num_inliers, a.inliers, num_models, memory);
    out_back(h, error_max, a.error_max, num_models, memory);
    out_back(h, order, a.order, num_models * n, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    return GBBA_SUCCESS;
  });
}
