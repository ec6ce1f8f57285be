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

// Copy the 64x64 tile at src (row stride ld) into a padded shared tile.  All
// of a thread's global loads are issued before its shared stores so that
// their latencies overlap.
template <typename T>
__device__ __forceinline__ void load_tile(T (*dst)[NB + 1], const T* __restrict__ src, int64_t ld, int tid) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n, PER_ROW = NB / W, ITER = NB * PER_ROW / 256;
  V v[ITER];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = tid + it * 256, r = idx / PER_ROW, c = (idx % PER_ROW) * W;
    v[it] = *reinterpret_cast<const V*>(src + r * ld + c);
  }
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = tid + it * 256, r = idx / PER_ROW, c = (idx % PER_ROW) * W;
    const T* e = reinterpret_cast<const T*>(&v[it]);
#pragma unroll
    for (int w = 0; w < W; ++w) dst[r][c + w] = e[w];
  }
}

// Factor the diagonal tile: S_kk = L L^T (written back into S's lower
// triangle, zeros above), L^-1 (into Linv_all), and y_k = L^-1 b_k.
//
// Outer-product LDL^T elimination with the same row operations applied to an
// identity block E, so that at the end A = L_u D L_u^T and E = L_u^-1 (one
// pass of 64 pivot steps yields both the factor and its inverse).  Thread
// (ty, tx) holds rows 4ty..4ty+3 x columns 4tx..4tx+3 of A and of E in
// registers.  At pivot j the owners of column j publish it with zeros at and
// above the pivot, the owners of row j of E publish that row (exactly zero
// right of the diagonal), and the diagonal owner publishes 1/d_j; every
// thread then applies a_il -= (c_i/d_j) c_l and e_il -= (c_i/d_j) E_jl to its
// whole block, with no predicates: the zeros leave finished columns, rows
// above the pivot and the zero part of E unchanged.
template <typename T>
__global__ void __launch_bounds__(256) k_potrf_diag(T* __restrict__ S, int64_t ld, int kb, T* __restrict__ Linv_all,
                                                    T* __restrict__ b, int* __restrict__ flag) {
  constexpr int BS = NB + 4;  // 16-byte aligned broadcast rows
  T* colbuf = &tile_at<T>(1)[0][0];  // [2][BS]: column j of A (double-buffered)
  T* rowbuf = colbuf + 2 * BS;       // [2][BS]: row j of E
  T* rpiv = rowbuf + 2 * BS;         // [2]: 1 / d_j
  T* part = &tile_at<T>(0)[0][0];    // 64 x 16 partial sums of L^-1 b
  T* yb = vec_at<T>(0);
  T* dv = vec_at<T>(1);
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int64_t off = (int64_t)kb * NB;
  T a[4][4], e[4][4];
#pragma unroll
  for (int ii = 0; ii < 4; ++ii) {
    ld4<T>(S + (off + ty * 4 + ii) * ld + off + tx * 4, a[ii]);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) e[ii][jj] = (ty * 4 + ii == tx * 4 + jj) ? T(1) : T(0);
  }
  if (tid < NB) yb[tid] = b[off + tid];
  for (int j4 = 0; j4 < NB; j4 += 4) {
    const bool col_owner = tx == (j4 >> 2), row_owner = ty == (j4 >> 2);
#pragma unroll
    for (int jc = 0; jc < 4; ++jc) {
      const int j = j4 + jc;
      T* cb = colbuf + (j & 1) * BS;
      T* rb = rowbuf + (j & 1) * BS;
      if (col_owner) {
        T c[4];
#pragma unroll
        for (int ii = 0; ii < 4; ++ii) c[ii] = (ty * 4 + ii > j) ? a[ii][jc] : T(0);
        st4<T>(cb + ty * 4, c);
        if (row_owner) {
          T d = a[jc][jc];
          if (!(d > T(0)) || !isfinite(d)) {
            d = T(1);
            atomicExch(flag, 1);
          }
          dv[j] = d;
          rpiv[j & 1] = T(1) / d;
        }
      }
      if (row_owner) st4<T>(rb + tx * 4, e[jc]);
      __syncthreads();
      const T r = rpiv[j & 1];
      T ci[4], cl[4], rl[4];
      ld4<T>(cb + ty * 4, ci);
      ld4<T>(cb + tx * 4, cl);
      ld4<T>(rb + tx * 4, rl);
#pragma unroll
      for (int ii = 0; ii < 4; ++ii) {
        const T m = ci[ii] * r;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          a[ii][jj] -= m * cl[jj];
          e[ii][jj] -= m * rl[jj];
        }
      }
    }
  }
  __syncthreads();
  if (tid < NB) dv[tid] = sqrt(dv[tid]);
  __syncthreads();
  // L_il = a_il / sqrt(d_l) (l < i), L_ii = sqrt(d_i); L^-1 = D^-1/2 E.
  T sl[4];
  ld4<T>(dv + tx * 4, sl);
  T yp[4] = {T(0), T(0), T(0), T(0)};
  T yv[4];
  ld4<T>(yb + tx * 4, yv);
#pragma unroll
  for (int ii = 0; ii < 4; ++ii) {
    const int i = ty * 4 + ii;
    const T si = dv[i];
    T lv[4], iv[4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int l = tx * 4 + jj;
      lv[jj] = (l < i) ? a[ii][jj] / sl[jj] : (l == i ? si : T(0));
      iv[jj] = (l <= i) ? e[ii][jj] / si : T(0);
      yp[ii] += iv[jj] * yv[jj];
    }
    st4<T>(S + (off + i) * ld + off + tx * 4, lv);
    st4<T>(Linv_all + (int64_t)kb * NB * NB + i * NB + tx * 4, iv);
  }
  // y = L^-1 b: thread (ty, tx) holds the partial sums of its 4x4 block
#pragma unroll
  for (int ii = 0; ii < 4; ++ii) part[(ty * 4 + ii) * 16 + tx] = yp[ii];
  __syncthreads();
  if (tid < NB) {
    T y = T(0);
#pragma unroll
    for (int t = 0; t < 16; ++t) y += part[tid * 16 + t];
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
  load_tile<T>(A, S + r0 * ld + c0, ld, tid);
  load_tile<T>(Li, Linv_all + (int64_t)kb * NB * NB, NB, tid);
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

// Trailing update by panel kb: S_ij -= L_ik L_jk^T.  With one_col the tiles
// are (first + blockIdx.x, first) (one block column); otherwise blockIdx.x
// enumerates the lower triangle of tiles first <= jb <= ib.
template <typename T>
__global__ void __launch_bounds__(256) k_syrk(T* __restrict__ S, int64_t ld, int kb, int first, int one_col) {
  T(*Xi)[NB + 1] = tile_at<T>(0);
  T(*Xj)[NB + 1] = tile_at<T>(1);
  const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
  int64_t ib, jb;
  if (one_col) {
    ib = first + (int64_t)blockIdx.x;
    jb = first;
  } else {
    // triangular decode of blockIdx.x -> (row >= col)
    const int64_t t = blockIdx.x;
    int64_t row = (int64_t)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while ((row + 1) * (row + 2) / 2 <= t) ++row;
    while (row * (row + 1) / 2 > t) --row;
    const int64_t col = t - row * (row + 1) / 2;
    ib = first + row;
    jb = first + col;
  }
  const int64_t c0 = (int64_t)kb * NB;
  load_tile<T>(Xi, S + ib * NB * ld + c0, ld, tid);
  load_tile<T>(Xj, S + jb * NB * ld + c0, ld, tid);
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
  load_tile<T>(Li, Linv_all + (int64_t)kb * NB * NB, NB, tid);
  if (tid < NB) yk[tid] = b[k0 + tid];
  __syncthreads();
  if (tid < NB) {
    T s = T(0);
#pragma unroll 16
    for (int r = 0; r < NB; ++r) s += Li[r][tid] * yk[r];  // L^-1 is lower: zeros for r < tid
    xk[tid] = s;
  }
  __syncthreads();
  const int jb = blockIdx.x;
  if (jb == kb) {
    if (tid < NB) x[k0 + tid] = xk[tid];
    return;
  }
  // y_j -= L_kj^T x_k : thread (q, c) sums rows q, q+4, ... of column c;
  // consecutive threads read consecutive columns of a row (coalesced)
  const int c = tid & (NB - 1), q = tid >> 6;
  const T* col = S + (k0 + q) * ld + (int64_t)jb * NB + c;
  T v[NB / 4];
#pragma unroll
  for (int t = 0; t < NB / 4; ++t) v[t] = col[(int64_t)(4 * t) * ld];
  T s = T(0);
#pragma unroll
  for (int t = 0; t < NB / 4; ++t) s += v[t] * xk[q + 4 * t];
  T* part = &Li[0][0];  // L_kk^-1 is no longer needed
  __syncthreads();
  part[q * NB + c] = s;
  __syncthreads();
  if (tid < NB) b[(int64_t)jb * NB + tid] -= part[tid] + part[NB + tid] + part[2 * NB + tid] + part[3 * NB + tid];
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

// Launch on the panel chain at the device's greatest stream priority (the
// attribute is kept when the launch is captured into a graph), so that the
// one-CTA diagonal factor is scheduled ahead of the trailing update's CTAs.
template <typename... Exp, typename... Act>
void launch_hi(gbba_handle* h, void (*k)(Exp...), unsigned grid, size_t smem, cudaStream_t st, Act... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = h->prio_hi;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GBBA_CUDA(cudaLaunchKernelEx(&cfg, k, args...));
  count_launch(h);
}

// Solve S x = b in place of (S -> L, b -> y); x receives the solution.
//
// Look-ahead by one panel: after panel k is solved, the update of block
// column k+1 (the next panel) runs on the call's stream followed by that
// panel's diagonal factor and panel solve, while the update of the remaining
// columns k+2.. runs on the side stream.  The two touch disjoint tiles; the
// call's stream waits for the side stream's update of step k-1 before it
// updates column k+1 (both write that column), and the side stream starts
// step k only after panel k is solved.  The side stream is joined back
// before the backward substitution, so the sequence can be captured.
template <typename T>
void dense_cholesky_solve(gbba_handle* h, T* S, int64_t n_pad, T* b, T* x, T* Linv_all, int* flag, cudaStream_t st) {
  const int nb = (int)(n_pad / NB);
  const size_t sm = dense_smem_bytes<T>();
  dense_cholesky_prepare<T>();
  launch_hi(h, k_potrf_diag<T>, 1, sm, st, S, n_pad, 0, Linv_all, b, flag);
  if (nb > 1) launch_hi(h, k_trsm_panel<T>, (unsigned)(nb - 1), sm, st, S, n_pad, 0, (const T*)Linv_all, b);
  bool side_pending = false;
  for (int k = 0; k + 1 < nb; ++k) {
    const int rem = nb - k - 1;  // tiles below the diagonal in column k
    if (side_pending) {
      GBBA_CUDA(cudaStreamWaitEvent(st, h->ev_side, 0));
      side_pending = false;
    }
    if (rem > 1) {
      GBBA_CUDA(cudaEventRecord(h->ev_main, st));
      GBBA_CUDA(cudaStreamWaitEvent(h->side, h->ev_main, 0));
      const int64_t tiles = (int64_t)(rem - 1) * rem / 2;
      k_syrk<T><<<(unsigned)tiles, 256, sm, h->side>>>(S, n_pad, k, k + 2, 0);
      check_launch(h);
      GBBA_CUDA(cudaEventRecord(h->ev_side, h->side));
      side_pending = true;
    }
    launch_hi(h, k_syrk<T>, (unsigned)rem, sm, st, S, n_pad, k, k + 1, 1);
    launch_hi(h, k_potrf_diag<T>, 1, sm, st, S, n_pad, k + 1, Linv_all, b, flag);
    if (rem > 1) launch_hi(h, k_trsm_panel<T>, (unsigned)(rem - 1), sm, st, S, n_pad, k + 1, (const T*)Linv_all, b);
  }
  if (side_pending) GBBA_CUDA(cudaStreamWaitEvent(st, h->ev_side, 0));
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
