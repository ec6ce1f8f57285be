// Dense Cholesky solve of the reduced camera system S z = rhs.
//
// Replaces DenseSchurComplementSolver::SolveReducedLinearSystem (Eigen LLT,
// 3rdparty/ceres/internal/ceres/schur_complement_solver.cc:180-222) and the
// CXSparse factorisation the reference configures (:316-340): S is dense for
// the workloads here (every camera pair is covisible), so a blocked dense
// factorisation on the GPU is the right tool.
//
// Layout: S is n_pad x n_pad row-major (n_pad = round_up(n, 64)); only the
// lower triangle is read.  Padding rows/columns carry the identity, so every
// 64x64 tile is full and no kernel needs bounds checks.
//
// Algorithm (right-looking, block size 64, one launch sequence per panel k):
//   potrf_diag : factor S_kk = L_kk L_kk^T in shared memory, form L_kk^-1,
//                and finish the forward substitution of block k: y_k = L_kk^-1 b_k
//   trsm_panel : L_ik = S_ik L_kk^-T for every i > k, and b_i -= L_ik y_k
//                (forward substitution fused into the panel solve)
//   syrk       : S_ij -= L_ik L_jk^T for k < j <= i (trailing update)
// then the backward substitution L^T x = y, right-looking by block rows:
//   trsv_bwd(k): x_k = L_kk^-T y_k; y_j -= L_kj^T x_k for j < k.
// A non-positive pivot sets *flag (LINEAR_SOLVER_FAILURE in ceres terms).
#include "gbba_internal.h"

namespace gbba {

constexpr int NB = 64;

// Two padded 64x64 tiles (plus a few vectors) live in dynamic shared memory:
// 66.5 KB in FP64, above the 48 KB static limit.
template <typename T>
__device__ __forceinline__ T (*tile_at(int i))[NB + 1] {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  return reinterpret_cast<T(*)[NB + 1]>(smem_raw + (size_t)i * NB * (NB + 1) * sizeof(T));
}
template <typename T>
__device__ __forceinline__ T* vec_at(int i) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  return reinterpret_cast<T*>(smem_raw + (size_t)2 * NB * (NB + 1) * sizeof(T) + (size_t)i * NB * sizeof(T));
}
template <typename T>
constexpr size_t dense_smem_bytes() { return (size_t)2 * NB * (NB + 1) * sizeof(T) + 2 * NB * sizeof(T); }

template <typename T>
__global__ void __launch_bounds__(256) k_potrf_diag(T* __restrict__ S, int64_t ld, int kb, T* __restrict__ Linv_all,
                                                    T* __restrict__ b, int* __restrict__ flag) {
  T(*A)[NB + 1] = tile_at<T>(0);
  T(*Li)[NB + 1] = tile_at<T>(1);
  T* yb = vec_at<T>(0);
  T* sq = vec_at<T>(1);
  const int tid = threadIdx.x;
  const int64_t off = (int64_t)kb * NB;
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int r = idx / NB, c = idx % NB;
    A[r][c] = (c <= r) ? S[(off + r) * ld + off + c] : T(0);
  }
  if (tid < NB) yb[tid] = b[off + tid];
  __syncthreads();
  // Outer-product elimination on the lower triangle: after step j, column j
  // holds the unscaled multipliers and A[j][j] the pivot; one barrier per step.
  for (int j = 0; j < NB; ++j) {
    T d = A[j][j];
    if (!(d > T(0)) || !isfinite((double)d)) {
      if (tid == 0) atomicExch(flag, 1);
      d = T(1);
      if (tid == 0) A[j][j] = d;
    }
    const T invd = T(1) / d;
    const int m = NB - 1 - j;
    for (int idx = tid; idx < m * m; idx += 256) {
      const int ii = j + 1 + idx / m, ll = j + 1 + idx % m;
      if (ll <= ii) A[ii][ll] -= A[ii][j] * A[ll][j] * invd;
    }
    __syncthreads();
  }
  if (tid < NB) sq[tid] = sqrt(A[tid][tid]);
  __syncthreads();
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int r = idx / NB, c = idx % NB;
    if (c < r) A[r][c] /= sq[c];
    else if (c == r) A[r][c] = sq[c];
  }
  __syncthreads();
  // L^-1 row by row: Li[i][c] = (delta_ic - sum_{c<=j<i} L[i][j] Li[j][c]) / L[i][i],
  // four threads per column c, one barrier per row.
  {
    const int c = tid >> 2, q = tid & 3;
    for (int i = 0; i < NB; ++i) {
      T s = T(0);
      for (int j = c + q; j < i; j += 4) s += A[i][j] * Li[j][c];
      s += __shfl_xor_sync(0xffffffffu, s, 1);
      s += __shfl_xor_sync(0xffffffffu, s, 2);
      if (q == 0) Li[i][c] = (c > i) ? T(0) : (((i == c) ? T(1) : T(0)) - s) / A[i][i];
      __syncthreads();
    }
  }
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int r = idx / NB, c = idx % NB;
    if (c <= r) S[(off + r) * ld + off + c] = A[r][c];
    Linv_all[(int64_t)kb * NB * NB + idx] = Li[r][c];
  }
  if (tid < NB) {
    T y = T(0);
    for (int c = 0; c <= tid; ++c) y += Li[tid][c] * yb[c];
    b[off + tid] = y;
  }
}

// 64x64 tile product helper: acc(4x4 per thread) += X[rows] . Y[cols]^T over l.
template <typename T>
__device__ __forceinline__ void tile_xyt(const T (*X)[NB + 1], const T (*Y)[NB + 1], int ty, int tx, T acc[4][4]) {
#pragma unroll 8
  for (int l = 0; l < NB; ++l) {
    T xr[4], yc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      xr[i] = X[ty * 4 + i][l];
      yc[i] = Y[tx * 4 + i][l];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += xr[i] * yc[j];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_trsm_panel(T* __restrict__ S, int64_t ld, int kb, const T* __restrict__ Linv_all,
                                                    T* __restrict__ b) {
  T(*A)[NB + 1] = tile_at<T>(0);
  T(*Li)[NB + 1] = tile_at<T>(1);
  T* y = vec_at<T>(0);
  const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
  const int64_t ib = kb + 1 + blockIdx.x;
  const int64_t r0 = ib * NB, c0 = (int64_t)kb * NB;
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int r = idx / NB, c = idx % NB;
    A[r][c] = S[(r0 + r) * ld + c0 + c];
    Li[r][c] = Linv_all[(int64_t)kb * NB * NB + idx];
  }
  if (tid < NB) y[tid] = b[c0 + tid];
  __syncthreads();
  T acc[4][4] = {};
  tile_xyt<T>(A, Li, ty, tx, acc);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) A[ty * 4 + i][tx * 4 + j] = acc[i][j];
  __syncthreads();
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int r = idx / NB, c = idx % NB;
    S[(r0 + r) * ld + c0 + c] = A[r][c];
  }
  if (tid < NB) {
    T s = T(0);
    for (int c = 0; c < NB; ++c) s += A[tid][c] * y[c];
    b[r0 + tid] -= s;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_syrk(T* __restrict__ S, int64_t ld, int kb) {
  T(*Xi)[NB + 1] = tile_at<T>(0);
  T(*Xj)[NB + 1] = tile_at<T>(1);
  const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
  // triangular decode of blockIdx.x -> (row >= col)
  const int64_t t = blockIdx.x;
  int64_t row = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((row + 1) * (row + 2) / 2 <= t) ++row;
  while (row * (row + 1) / 2 > t) --row;
  const int64_t col = t - row * (row + 1) / 2;
  const int64_t ib = kb + 1 + row, jb = kb + 1 + col;
  const int64_t c0 = (int64_t)kb * NB;
  for (int idx = tid; idx < NB * NB; idx += 256) {
    const int r = idx / NB, c = idx % NB;
    Xi[r][c] = S[(ib * NB + r) * ld + c0 + c];
    Xj[r][c] = S[(jb * NB + r) * ld + c0 + c];
  }
  __syncthreads();
  T acc[4][4] = {};
  tile_xyt<T>(Xi, Xj, ty, tx, acc);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T* p = &S[(ib * NB + ty * 4 + i) * ld + jb * NB + tx * 4 + j];
      *p -= acc[i][j];
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_trsv_bwd(const T* __restrict__ S, int64_t ld, int kb, const T* __restrict__ Linv_all,
                                                  T* __restrict__ b, T* __restrict__ x) {
  T(*Li)[NB + 1] = tile_at<T>(0);
  T* yk = vec_at<T>(0);
  T* xk = vec_at<T>(1);
  const int tid = threadIdx.x;
  const int64_t k0 = (int64_t)kb * NB;
  for (int idx = tid; idx < NB * NB; idx += 256) Li[idx / NB][idx % NB] = Linv_all[(int64_t)kb * NB * NB + idx];
  if (tid < NB) yk[tid] = b[k0 + tid];
  __syncthreads();
  if (tid < NB) {
    T s = T(0);
    for (int r = tid; r < NB; ++r) s += Li[r][tid] * yk[r];
    xk[tid] = s;
  }
  __syncthreads();
  const int jb = blockIdx.x;
  if (jb == kb) {
    if (tid < NB) x[k0 + tid] = xk[tid];
    return;
  }
  // y_j -= L_kj^T x_k : column c of the tile, 4 threads per column
  const int c = tid / 4, q = tid % 4;
  T s = T(0);
  for (int r = q; r < NB; r += 4) s += S[(k0 + r) * ld + (int64_t)jb * NB + c] * xk[r];
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  if (q == 0) b[(int64_t)jb * NB + c] -= s;
}

// Opt the kernels into their dynamic shared memory (once per process and
// type; called before any stream capture).
template <typename T>
void dense_cholesky_prepare() {
  static bool configured = false;
  if (configured) return;
  const int sm = (int)dense_smem_bytes<T>();
  GBBA_CUDA(cudaFuncSetAttribute(k_potrf_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  GBBA_CUDA(cudaFuncSetAttribute(k_trsm_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  GBBA_CUDA(cudaFuncSetAttribute(k_syrk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  GBBA_CUDA(cudaFuncSetAttribute(k_trsv_bwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  configured = true;
}

// Solve S x = b in place of (S -> L, b -> y); x receives the solution.
template <typename T>
void dense_cholesky_solve(gbba_handle* h, T* S, int64_t n_pad, T* b, T* x, T* Linv_all, int* flag, cudaStream_t st) {
  const int nb = (int)(n_pad / NB);
  const size_t sm = dense_smem_bytes<T>();
  dense_cholesky_prepare<T>();
  for (int kb = 0; kb < nb; ++kb) {
    k_potrf_diag<T><<<1, 256, sm, st>>>(S, n_pad, kb, Linv_all, b, flag);
    check_launch(h);
    const int rem = nb - kb - 1;
    if (rem > 0) {
      k_trsm_panel<T><<<rem, 256, sm, st>>>(S, n_pad, kb, Linv_all, b);
      check_launch(h);
      const int64_t tiles = (int64_t)rem * (rem + 1) / 2;
      k_syrk<T><<<(unsigned)tiles, 256, sm, st>>>(S, n_pad, kb);
      check_launch(h);
    }
  }
  for (int kb = nb - 1; kb >= 0; --kb) {
    k_trsv_bwd<T><<<kb + 1, 256, sm, st>>>(S, n_pad, kb, Linv_all, b, x);
    check_launch(h);
  }
}

template void dense_cholesky_prepare<double>();
template void dense_cholesky_prepare<float>();
template void dense_cholesky_solve<double>(gbba_handle*, double*, int64_t, double*, double*, double*, int*, cudaStream_t);
template void dense_cholesky_solve<float>(gbba_handle*, float*, int64_t, float*, float*, float*, int*, cudaStream_t);

}  // namespace gbba
