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
#include <type_traits>

#include "gbba_internal.h"
#include "gbba_umma.cuh"

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

// Copy the contiguous 64x64 tile at src (row stride 64) with L2-only loads
// (ld.global.cg): for data written by a kernel that may still have been
// running when this kernel started (programmatic dependent launch), so that
// no line cached in L1 before that kernel finished can be read.
template <typename T>
__device__ __forceinline__ void load_tile_cg(T (*dst)[NB + 1], const T* src, int tid) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n, PER_ROW = NB / W, ITER = NB * PER_ROW / 256;
  V v[ITER];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = tid + it * 256, r = idx / PER_ROW, c = (idx % PER_ROW) * W;
    v[it] = __ldcg(reinterpret_cast<const V*>(src + r * NB + c));
  }
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = tid + it * 256, r = idx / PER_ROW, c = (idx % PER_ROW) * W;
    const T* e = reinterpret_cast<const T*>(&v[it]);
#pragma unroll
    for (int w = 0; w < W; ++w) dst[r][c + w] = e[w];
  }
}

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

// Reciprocal of a pivot.  Single precision uses the fast hardware reciprocal
// (__fdividef, within 2 ulp for normal pivots): it sits on the elimination's
// critical path, and the FP32 factor only feeds LM steps whose acceptance is
// decided on the FP64 cost.  Double precision divides exactly.
__device__ __forceinline__ float pivot_rcp(float d) { return __fdividef(1.0f, d); }
__device__ __forceinline__ double pivot_rcp(double d) { return 1.0 / d; }

// Factor the diagonal tile: S_kk = L L^T (written back into S's lower
// triangle, zeros above), L^-1 (into Linv_all), and y_k = L^-1 b_k.
//
// Blocked right-looking factorisation of the 64 x 64 tile in shared memory
// over four 16-column panels p (offset o = 16p):
//   1. warp 0 factors the 16 x 16 diagonal block: outer-product LDL^T with
//      the same row operations applied to an identity block E (so that
//      E = L_u^-1 at the end); lane (r, h) holds row r, columns 8h..8h+7 of
//      both in registers, pivots are broadcast through shared memory with
//      only __syncwarp between steps;
//   2. panel solve  L_ip = A_ip L_pp^-T  for the rows below (all threads);
//   3. trailing update  A_il -= L_ip L_lp^T  inside the tile (all threads);
// then the off-diagonal 16 x 16 blocks of L^-1 by increasing distance from
// the diagonal,  Li_IJ = -Li_II sum_{K=J..I-1} L_IK Li_KJ,  and y = L^-1 b.
// A non-positive (or non-finite) pivot is replaced by 1 and sets *flag.
constexpr int kPotrfThreads = 256;
constexpr int kTileLd = NB + 4;  // 16-byte aligned rows
template <typename T>
constexpr size_t potrf_smem_bytes() {
  return sizeof(T) * ((size_t)2 * NB * kTileLd   // A / L, L^-1
                      + 3 * 16 * 16              // scratch of the inverse blocks
                      + 4 * 16 + 4               // warp-0 broadcast buffers
                      + 2 * NB);                 // b, pivots
}

template <typename T>
__global__ void __launch_bounds__(kPotrfThreads) k_potrf_diag(T* __restrict__ S, int64_t ld, int kb,
                                                              T* __restrict__ Linv_all, T* __restrict__ b,
                                                              int* __restrict__ flag, int upd) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* A = reinterpret_cast<T*>(smem_raw);  // [64][kTileLd]: A, overwritten by L
  T* Li = A + NB * kTileLd;               // [64][kTileLd]: L^-1
  T* scr = Li + NB * kTileLd;             // [3][16][16]
  T* bc = scr + 3 * 256;                  // [2][16] pivot column
  T* br = bc + 32;                        // [2][16] row of E
  T* rp = br + 32;                        // [2] 1/d (+2 padding)
  T* yb = rp + 4;                         // [64]
  T* dv = yb + NB;                        // [64] pivots of the current panel
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t off = (int64_t)kb * NB;
  // the panel solve of this block column may start now: it reads L^-1 and y
  // only after griddepcontrol.wait, i.e. after this kernel has completed
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // load the tile (lower part is what is used) and b; with upd, also the
  // previous panel's block P = L_{kb,kb-1} (staged in the L^-1 buffer)
#pragma unroll
  for (int it = 0; it < NB * NB / 4 / kPotrfThreads; ++it) {
    const int idx = tid + it * kPotrfThreads, r = idx >> 4, c = (idx & 15) * 4;
    T v[4];
    ld4<T>(S + (off + r) * ld + off + c, v);
    st4<T>(A + r * kTileLd + c, v);
    if (upd) {
      ld4<T>(S + (off + r) * ld + off - NB + c, v);
      st4<T>(Li + r * kTileLd + c, v);
    }
  }
  if (tid < NB) yb[tid] = b[off + tid];
  __syncthreads();
  if (upd) {
    // A -= P P^T (thread: rows 4(tid>>4).., columns 4(tid&15)..)
    const int r0 = 4 * (tid >> 4), l0 = 4 * (tid & 15);
    T acc[4][4] = {};
#pragma unroll 4
    for (int k4 = 0; k4 < NB; k4 += 4) {
      T xi[4][4], xl[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ld4<T>(Li + (r0 + q) * kTileLd + k4, xi[q]);
        ld4<T>(Li + (l0 + q) * kTileLd + k4, xl[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int w = 0; w < 4; ++w)
#pragma unroll
          for (int k = 0; k < 4; ++k) acc[q][w] += xi[q][k] * xl[w][k];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T v[4];
      ld4<T>(A + (r0 + q) * kTileLd + l0, v);
#pragma unroll
      for (int w = 0; w < 4; ++w) v[w] -= acc[q][w];
      st4<T>(A + (r0 + q) * kTileLd + l0, v);
    }
    __syncthreads();
  }
  // clear L^-1
#pragma unroll
  for (int it = 0; it < NB * NB / 4 / kPotrfThreads; ++it) {
    const int idx = tid + it * kPotrfThreads, r = idx >> 4, c = (idx & 15) * 4;
    const T z[4] = {T(0), T(0), T(0), T(0)};
    st4<T>(Li + r * kTileLd + c, z);
  }
  __syncthreads();

  for (int p = 0; p < 4; ++p) {
    const int o = 16 * p;
    // ---- 1. diagonal 16 x 16 block, warp 0
    if (warp == 0) {
      const int r = lane & 15, h = lane >> 4;
      T a[8], e[8];
      ld4<T>(A + (o + r) * kTileLd + o + 8 * h, a);
      ld4<T>(A + (o + r) * kTileLd + o + 8 * h + 4, a + 4);
#pragma unroll
      for (int q = 0; q < 8; ++q) e[q] = (r == 8 * h + q) ? T(1) : T(0);
      // pivot j: lane (i, h') holds a_ij in a[j & 7] when h' = j >> 3, and
      // row j of E lives in lanes (j, 0) and (j, 1); everything a lane needs
      // is fetched with independent shuffles (no shared-memory round trip)
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int hs = 16 * (j >> 3);  // lane offset of the owners of column j
        T d = __shfl_sync(0xffffffffu, a[j & 7], j + hs);
        const T cr = __shfl_sync(0xffffffffu, a[j & 7], r + hs);
        T cl[8], rl[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          cl[q] = __shfl_sync(0xffffffffu, a[j & 7], 8 * h + q + hs);
          rl[q] = __shfl_sync(0xffffffffu, e[q], j + 16 * h);
        }
        if (!(d > T(0) && d - d == T(0))) {  // non-positive, NaN or infinite pivot
          d = T(1);
          if (lane == 0) atomicExch(flag, 1);
        }
        if (lane == 0) dv[o + j] = d;
        const T m = (r > j) ? cr * pivot_rcp(d) : T(0);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const T c = (8 * h + q > j) ? cl[q] : T(0);
          a[q] -= m * c;
          e[q] -= m * rl[q];
        }
      }
      __syncwarp();
      // L_pp = L_u D^1/2, L_pp^-1 = D^-1/2 E: sqrt(d) and 1/sqrt(d) once per
      // pivot (lanes 0..15 in parallel), then products only
      T* sqd = bc;       // [16] sqrt(d), reusing the broadcast buffers
      T* rsd = bc + 16;  // [16] 1/sqrt(d)
      if (lane < 16) {
        const T sd = sqrt(dv[o + lane]);
        sqd[lane] = sd;
        rsd[lane] = T(1) / sd;
      }
      __syncwarp();
      const T rr = rsd[r];
      T rl8[8];
      ld4<T>(rsd + 8 * h, rl8);
      ld4<T>(rsd + 8 * h + 4, rl8 + 4);
      T lv[8], iv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int l = 8 * h + q;
        lv[q] = (l < r) ? a[q] * rl8[q] : (l == r ? sqd[r] : T(0));
        iv[q] = (l <= r) ? e[q] * rr : T(0);
      }
      st4<T>(A + (o + r) * kTileLd + o + 8 * h, lv);
      st4<T>(A + (o + r) * kTileLd + o + 8 * h + 4, lv + 4);
      st4<T>(Li + (o + r) * kTileLd + o + 8 * h, iv);
      st4<T>(Li + (o + r) * kTileLd + o + 8 * h + 4, iv + 4);
    }
    __syncthreads();
    if (p == 3) break;
    // ---- 2. panel solve: rows o+16..63, L_ic = sum_k A_ik Li_pp[c][k]
    const int rows = NB - o - 16;
    T pv[3];
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int idx = tid + u * kPotrfThreads;
      pv[u] = T(0);
      if (idx < rows * 16) {
        const int i = o + 16 + (idx >> 4), c = idx & 15;
        T s4[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int k4 = 0; k4 < 16; k4 += 4) {
          T av[4], lv[4];
          ld4<T>(A + i * kTileLd + o + k4, av);
          ld4<T>(Li + (o + c) * kTileLd + o + k4, lv);
#pragma unroll
          for (int k = 0; k < 4; ++k) s4[k] += av[k] * lv[k];
        }
        pv[u] = (s4[0] + s4[1]) + (s4[2] + s4[3]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int idx = tid + u * kPotrfThreads;
      if (idx < rows * 16) A[(o + 16 + (idx >> 4)) * kTileLd + o + (idx & 15)] = pv[u];
    }
    __syncthreads();
    // ---- 3. trailing update inside the tile: 4 x 4 output blocks, lower blocks only
    {
      const int nbk = rows / 4;  // 4-row blocks of the trailing part
      for (int t = tid; t < nbk * nbk; t += kPotrfThreads) {
        const int bi = t / nbk, bl = t % nbk;
        if (bl > bi) continue;
        const int i0 = o + 16 + 4 * bi, l0 = o + 16 + 4 * bl;
        T acc[4][4] = {};
#pragma unroll
        for (int k4 = 0; k4 < 16; k4 += 4) {
          T xi[4][4], xl[4][4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            ld4<T>(A + (i0 + q) * kTileLd + o + k4, xi[q]);
            ld4<T>(A + (l0 + q) * kTileLd + o + k4, xl[q]);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int w = 0; w < 4; ++w)
#pragma unroll
              for (int k = 0; k < 4; ++k) acc[q][w] += xi[q][k] * xl[w][k];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          T v[4];
          ld4<T>(A + (i0 + q) * kTileLd + l0, v);
#pragma unroll
          for (int w = 0; w < 4; ++w) v[w] -= acc[q][w];
          st4<T>(A + (i0 + q) * kTileLd + l0, v);
        }
      }
    }
    __syncthreads();
  }

  // ---- off-diagonal blocks of L^-1, by distance from the diagonal
  for (int dist = 1; dist < 4; ++dist) {
    const int nblk = 4 - dist;  // blocks (J + dist, J), J = 0..nblk-1
    // T_IJ = sum_{K=J}^{I-1} L_IK Li_KJ
    for (int idx = tid; idx < nblk * 256; idx += kPotrfThreads) {
      const int J = idx >> 8, I = J + dist, r = (idx >> 4) & 15, c = idx & 15;
      T s4[4] = {T(0), T(0), T(0), T(0)};
      for (int K = J; K < I; ++K) {
        const T* ar = A + (16 * I + r) * kTileLd + 16 * K;
#pragma unroll
        for (int k4 = 0; k4 < 16; k4 += 4) {
          T av[4];
          ld4<T>(ar + k4, av);
#pragma unroll
          for (int k = 0; k < 4; ++k) s4[k] += av[k] * Li[(16 * K + k4 + k) * kTileLd + 16 * J + c];
        }
      }
      scr[idx] = (s4[0] + s4[1]) + (s4[2] + s4[3]);
    }
    __syncthreads();
    // Li_IJ = -Li_II T_IJ
    for (int idx = tid; idx < nblk * 256; idx += kPotrfThreads) {
      const int J = idx >> 8, I = J + dist, r = (idx >> 4) & 15, c = idx & 15;
      T s4[4] = {T(0), T(0), T(0), T(0)};
      const T* lr = Li + (16 * I + r) * kTileLd + 16 * I;
#pragma unroll
      for (int k4 = 0; k4 < 16; k4 += 4) {
        T lv[4];
        ld4<T>(lr + k4, lv);
#pragma unroll
        for (int k = 0; k < 4; ++k) s4[k] += lv[k] * scr[(J << 8) + (k4 + k) * 16 + c];
      }
      Li[(16 * I + r) * kTileLd + 16 * J + c] = -((s4[0] + s4[1]) + (s4[2] + s4[3]));
    }
    __syncthreads();
  }

  // ---- y = L^-1 b (4 threads per row), then write L and L^-1
  {
    const int r = tid >> 2, q = tid & 3;
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 16; ++c) s += Li[r * kTileLd + 16 * q + c] * yb[16 * q + c];
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (q == 0) b[off + r] = s;
  }
#pragma unroll
  for (int it = 0; it < NB * NB / 4 / kPotrfThreads; ++it) {
    const int idx = tid + it * kPotrfThreads, r = idx >> 4, c = (idx & 15) * 4;
    T v[4], w[4];
    ld4<T>(A + r * kTileLd + c, v);
    ld4<T>(Li + r * kTileLd + c, w);
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (c + e > r) v[e] = T(0);
    st4<T>(S + (off + r) * ld + off + c, v);
    st4<T>(Linv_all + (int64_t)kb * NB * NB + r * NB + c, w);
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

// Panel solve of block column kb: for tile ib = kb + 1 + blockIdx.x,
//   (with upd) S_ib,kb -= L_ib,kb-1 L_kb,kb-1^T   (the previous panel's
//                                                  update of this tile)
//   L_ib,kb = S_ib,kb L_kb,kb^-T,   b_ib -= L_ib,kb y_kb
// (the forward substitution is fused into the panel solve).
template <typename T>
__global__ void __launch_bounds__(256) k_trsm_panel(T* __restrict__ S, int64_t ld, int kb, const T* Linv_all, T* b,
                                                    int upd) {
  T(*A)[NB + 1] = tile_at<T>(0);
  T(*Li)[NB + 1] = tile_at<T>(1);
  T* y = vec_at<T>(0);
  const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
  const int64_t ib = kb + 1 + blockIdx.x;
  const int64_t r0 = ib * NB, c0 = (int64_t)kb * NB;
  T a[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) ld4<T>(S + (r0 + ty * 4 + i) * ld + c0 + tx * 4, a[i]);
  if (upd) {
    load_tile<T>(A, S + r0 * ld + c0 - NB, ld, tid);
    load_tile<T>(Li, S + c0 * ld + c0 - NB, ld, tid);
    __syncthreads();
    T acc[4][4] = {};
    tile_xyt<T>(A, Li, ty, tx, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) a[i][j] -= acc[i][j];
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) A[ty * 4 + i][tx * 4 + j] = a[i][j];
  // L^-1 and y_kb come from the diagonal factor launched just before this
  // kernel (programmatic dependent launch): wait for its completion
  asm volatile("griddepcontrol.wait;" ::: "memory");
  load_tile_cg<T>(Li, Linv_all + (int64_t)kb * NB * NB, tid);
  if (tid < NB) y[tid] = __ldcg(b + c0 + tid);
  __syncthreads();
  T acc[4][4] = {};
  tile_xyt<T>(A, Li, ty, tx, acc);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    st4<T>(S + (r0 + ty * 4 + i) * ld + c0 + tx * 4, acc[i]);
#pragma unroll
    for (int j = 0; j < 4; ++j) A[ty * 4 + i][tx * 4 + j] = acc[i][j];
  }
  __syncthreads();
  // b_ib -= L y: 4 threads per row, 16 columns each
  {
    const int r = tid >> 2, q = tid & 3;
    T s4 = T(0);
#pragma unroll
    for (int c = 0; c < 16; ++c) s4 += A[r][16 * q + c] * y[16 * q + c];
    s4 += __shfl_xor_sync(0xffffffffu, s4, 1);
    s4 += __shfl_xor_sync(0xffffffffu, s4, 2);
    if (q == 0) b[r0 + r] = __ldcg(b + r0 + r) - s4;
  }
}

// Trailing update over 128 x 128 output tiles (2 x 2 tiles of 64):
// S_IJ -= L_Ik L_Jk^T, K = 64 (panel kb).  blockIdx.x enumerates the lower
// triangle of 128-tiles over the 64-tiles first..nb-1; at the matrix edge a
// 128-tile holds one 64-tile row or column (the missing half is zero-filled
// and not stored), and the quarter of a diagonal 128-tile above the diagonal
// is not stored.  Operands are staged k-major (X^T, row stride 132) so that a
// thread's 8 rows and 8 columns at one k are 16-byte shared loads; thread
// (ty, tx) owns rows 8ty..8ty+7 x columns 8tx..8tx+7 of the output tile.
constexpr int kWideLd = 2 * NB + 4;
template <typename T>
constexpr size_t wide_smem_bytes() { return (size_t)2 * NB * kWideLd * sizeof(T); }

template <typename T>
__device__ __forceinline__ void load_panel_t(T* __restrict__ dst, const T* __restrict__ S, int64_t ld, int64_t row0,
                                             int64_t col0, int valid_rows, int tid) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n, ITER = 2 * NB * NB / W / 256;
  V v[ITER];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = tid + it * 256, kv = idx / (2 * NB), r = idx % (2 * NB);
    if (r < valid_rows) v[it] = *reinterpret_cast<const V*>(S + (row0 + r) * ld + col0 + kv * W);
    else {
      T* z = reinterpret_cast<T*>(&v[it]);
#pragma unroll
      for (int w = 0; w < W; ++w) z[w] = T(0);
    }
  }
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = tid + it * 256, kv = idx / (2 * NB), r = idx % (2 * NB);
    const T* e = reinterpret_cast<const T*>(&v[it]);
#pragma unroll
    for (int w = 0; w < W; ++w) dst[(kv * W + w) * kWideLd + r] = e[w];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_syrk_wide(T* __restrict__ S, int64_t ld, int kb, int first, int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* XiT = reinterpret_cast<T*>(smem_raw);
  T* XjT = XiT + NB * kWideLd;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int64_t t = blockIdx.x;
  int64_t R = (int64_t)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((R + 1) * (R + 2) / 2 <= t) ++R;
  while (R * (R + 1) / 2 > t) --R;
  const int64_t C = t - R * (R + 1) / 2;
  const int64_t ib0 = first + 2 * R, jb0 = first + 2 * C;
  const int rows_i = ib0 + 1 < nb ? 2 * NB : NB, rows_j = jb0 + 1 < nb ? 2 * NB : NB;
  const int64_t c0 = (int64_t)kb * NB;
  load_panel_t<T>(XiT, S, ld, ib0 * NB, c0, rows_i, tid);
  load_panel_t<T>(XjT, S, ld, jb0 * NB, c0, rows_j, tid);
  __syncthreads();
  // rows {4ty+i, 64+4ty+i} x columns {4tx+j, 64+4tx+j}: the 16-byte shared
  // loads of a quarter warp cover 128 contiguous bytes (no bank conflicts)
  T acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = T(0);
#pragma unroll 4
  for (int k = 0; k < NB; ++k) {
    T xa[8], xb[8];
    ld4<T>(XiT + k * kWideLd + ty * 4, xa);
    ld4<T>(XiT + k * kWideLd + NB + ty * 4, xa + 4);
    ld4<T>(XjT + k * kWideLd + tx * 4, xb);
    ld4<T>(XjT + k * kWideLd + NB + tx * 4, xb + 4);
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] += xa[i] * xb[j];
  }
#pragma unroll
  for (int qi = 0; qi < 2; ++qi)
#pragma unroll
    for (int qj = 0; qj < 2; ++qj) {
      const int64_t rb = ib0 + qi, cb = jb0 + qj;
      if (rb >= nb || cb >= nb || rb < cb) continue;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        T* p = S + (rb * NB + ty * 4 + i) * ld + cb * NB + tx * 4;
        T v[4];
        ld4<T>(p, v);
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] -= acc[4 * qi + i][4 * qj + j];
        st4<T>(p, v);
      }
    }
}

// The same trailing update on the tensor cores (FP32 path): one CTA per
// 128 x 128 output tile of the same enumeration as k_syrk_wide, acc = X_i X_j^T
// over the panel's 64 columns by tcgen05 kind::tf32 MMAs in 3xTF32 (FP32
// accuracy), accumulated in tensor memory; the epilogue subtracts it from S.
// Rows of a tile beyond the matrix edge are staged as zeros and not stored;
// quarters above the diagonal are not stored.  A bounded wait that runs out
// sets *flag = 6 (the step is then rejected) and the tile is left alone.
constexpr int kSyrkTcThreads = 256;
__global__ void __launch_bounds__(kSyrkTcThreads) k_syrk_tc(float* __restrict__ S, int64_t ld, int kb, int first,
                                                            int nb, int* __restrict__ flag) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  umma::GemmSmem& g = *reinterpret_cast<umma::GemmSmem*>(smem_raw);
  const int64_t t = blockIdx.x;
  int64_t R = (int64_t)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((R + 1) * (R + 2) / 2 <= t) ++R;
  while (R * (R + 1) / 2 > t) --R;
  const int64_t C = t - R * (R + 1) / 2;
  const int64_t ib0 = first + 2 * R, jb0 = first + 2 * C;
  const int rows_i = ib0 + 1 < nb ? 2 * NB : NB, rows_j = jb0 + 1 < nb ? 2 * NB : NB;
  const int64_t c0 = (int64_t)kb * NB;
  umma::gemm_setup(g, 128);
  const bool ok = umma::gemm_tile<kSyrkTcThreads>(g, 0, S + ib0 * NB * ld + c0, ld, S + jb0 * NB * ld + c0, ld, NB / umma::kChunk,
                                  rows_i, rows_j);
  if (ok) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = 32 * (w & 3) + lane;       // tile row = tensor-memory lane
    const int qj = w >> 2;                   // column half: 64-tile jb0 + qj
    const int64_t rb = ib0 + (r >> 6), cb = jb0 + qj;
    if (rb < nb && cb < nb && rb >= cb) {
      float* row = S + (rb * NB + (r & 63)) * ld + cb * NB;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v[32];
        umma::tmem_ld32(g.tmem_base + ((uint32_t)(32 * (w & 3)) << 16) + 64 * qj + 32 * h, v);
#pragma unroll
        for (int e = 0; e < 32; e += 4) {
          float4 c = *reinterpret_cast<float4*>(row + 32 * h + e);
          c.x -= v[e];
          c.y -= v[e + 1];
          c.z -= v[e + 2];
          c.w -= v[e + 3];
          *reinterpret_cast<float4*>(row + 32 * h + e) = c;
        }
      }
    }  // (the condition is uniform over a warp, as the warp-collective tcgen05.ld requires)
  } else if (threadIdx.x == 0) {
    atomicExch(flag, 6);
  }
  umma::gemm_teardown(g, 128);
}

template <typename T>
__global__ void __launch_bounds__(256) k_trsv_bwd(const T* __restrict__ S, int64_t ld, int kb, const T* __restrict__ Linv_all,
                                                  T* __restrict__ b, T* __restrict__ x) {
  T(*Li)[NB + 1] = tile_at<T>(0);
  T* yk = vec_at<T>(0);
  T* xk = vec_at<T>(1);
  const int tid = threadIdx.x;
  const int64_t k0 = (int64_t)kb * NB;
  // the next block row's kernel may start now (programmatic dependent
  // launch): it touches b only after its griddepcontrol.wait
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  load_tile<T>(Li, Linv_all + (int64_t)kb * NB * NB, NB, tid);
  const int jb = blockIdx.x;
  const int c = tid & (NB - 1), q = tid >> 6;
  // this block's column of L_kj^T (written by the factorisation, complete
  // before the backward substitution began) is loaded before the wait
  T v[NB / 4];
  if (jb != kb) {
    const T* col = S + (k0 + q) * ld + (int64_t)jb * NB + c;
#pragma unroll
    for (int t = 0; t < NB / 4; ++t) v[t] = col[(int64_t)(4 * t) * ld];
  }
  // y_k and the b entries this kernel updates were written by the previous
  // block row's kernel: wait for it, and read b through L2
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (tid < NB) yk[tid] = __ldcg(b + k0 + tid);
  __syncthreads();
  if (tid < NB) {
    T s = T(0);
#pragma unroll 16
    for (int r = 0; r < NB; ++r) s += Li[r][tid] * yk[r];  // L^-1 is lower: zeros for r < tid
    xk[tid] = s;
  }
  __syncthreads();
  if (jb == kb) {
    if (tid < NB) x[k0 + tid] = xk[tid];
    return;
  }
  // y_j -= L_kj^T x_k : thread (q, c) sums rows q, q+4, ... of column c;
  // consecutive threads read consecutive columns of a row (coalesced)
  T s = T(0);
#pragma unroll
  for (int t = 0; t < NB / 4; ++t) s += v[t] * xk[q + 4 * t];
  T* part = &Li[0][0];  // L_kk^-1 is no longer needed
  __syncthreads();
  part[q * NB + c] = s;
  __syncthreads();
  if (tid < NB)
    b[(int64_t)jb * NB + tid] = __ldcg(b + (int64_t)jb * NB + tid) -
                                (part[tid] + part[NB + tid] + part[2 * NB + tid] + part[3 * NB + tid]);
}

// Opt the kernels into their dynamic shared memory (once per device and type;
// called before any stream capture).
template <typename T>
void dense_cholesky_prepare() {
  static PerDeviceOnce once;
  once.run([] {
    const int sm = (int)dense_smem_bytes<T>();
    GBBA_CUDA(cudaFuncSetAttribute(k_potrf_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)potrf_smem_bytes<T>()));
    GBBA_CUDA(cudaFuncSetAttribute(k_trsm_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    GBBA_CUDA(cudaFuncSetAttribute(k_trsv_bwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    GBBA_CUDA(cudaFuncSetAttribute(k_syrk_wide<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)wide_smem_bytes<T>()));
    if (std::is_same<T, float>::value)
      GBBA_CUDA(cudaFuncSetAttribute(k_syrk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(umma::GemmSmem)));
  });
}

// Launch on the panel chain at the device's greatest stream priority (the
// attribute is kept when the launch is captured into a graph), so that the
// one-CTA diagonal factor is scheduled ahead of the trailing update's CTAs.
//
// With pdl the launch may begin while the previous kernel on the stream is
// still running (programmatic dependent launch): the kernel must execute
// griddepcontrol.wait before it touches anything the previous kernel writes.
template <typename... Exp, typename... Act>
void launch_hi(gbba_handle* h, bool pdl, void (*k)(Exp...), unsigned grid, unsigned block, size_t smem,
               cudaStream_t st, Act... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = h->prio_hi;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 2 : 1;
  GBBA_CUDA(cudaLaunchKernelEx(&cfg, k, args...));
  count_launch(h);
}

// Solve S x = b in place of (S -> L, b -> y); x receives the solution.
//
// Right-looking, 64-wide panels, look-ahead by one panel.  Per step k the
// call's stream runs two kernels:
//   potrf(k+1): applies panel k's update to diagonal tile k+1, factors it
//               (L, L^-1, y_{k+1});
//   trsm(k+1):  applies panel k's update to the tiles below it in block
//               column k+1, then solves them (and updates b);
// while the side stream applies panel k's update to block columns k+2..
// (128-wide tiles).  The two streams touch disjoint tiles; the call's stream
// waits for the side stream's step k-1 before step k (that step wrote block
// column k+1), and the side stream starts step k once panel k is solved.
// The side stream is joined back before the backward substitution, so the
// sequence can be captured.
// kTensor: the trailing update on the tensor cores (k_syrk_tc, FP32 only) or
// on the FP32/FP64 pipes (k_syrk_wide).
template <typename T, bool kTensor>
void dense_cholesky_solve_impl(gbba_handle* h, T* S, int64_t n_pad, T* b, T* x, T* Linv_all, int* flag,
                               cudaStream_t st) {
  const int nb = (int)(n_pad / NB);
  const size_t sm = dense_smem_bytes<T>(), psm = potrf_smem_bytes<T>();
  dense_cholesky_prepare<T>();
  launch_hi(h, false, k_potrf_diag<T>, 1, kPotrfThreads, psm, st, S, n_pad, 0, Linv_all, b, flag, 0);
  if (nb > 1)
    launch_hi(h, true, k_trsm_panel<T>, (unsigned)(nb - 1), 256, sm, st, S, n_pad, 0, (const T*)Linv_all, b, 0);
  bool side_pending = false;
  for (int k = 0; k + 1 < nb; ++k) {
    const int rem = nb - k - 1;  // tiles in block column k+1, diagonal included
    if (side_pending) {
      GBBA_CUDA(cudaStreamWaitEvent(st, h->ev_side, 0));
      side_pending = false;
    }
    if (rem > 1) {
      GBBA_CUDA(cudaEventRecord(h->ev_main, st));
      GBBA_CUDA(cudaStreamWaitEvent(h->side, h->ev_main, 0));
      const int64_t tw = rem / 2;  // 128-tiles per side over the 64-tiles k+2..nb-1
      if constexpr (kTensor)
        k_syrk_tc<<<(unsigned)(tw * (tw + 1) / 2), kSyrkTcThreads, sizeof(umma::GemmSmem), h->side>>>(
            S, n_pad, k, k + 2, nb, flag);
      else
        k_syrk_wide<T><<<(unsigned)(tw * (tw + 1) / 2), 256, wide_smem_bytes<T>(), h->side>>>(S, n_pad, k, k + 2, nb);
      check_launch(h);
      GBBA_CUDA(cudaEventRecord(h->ev_side, h->side));
      side_pending = true;
    }
    launch_hi(h, false, k_potrf_diag<T>, 1, kPotrfThreads, psm, st, S, n_pad, k + 1, Linv_all, b, flag, 1);
    if (rem > 1)
      launch_hi(h, true, k_trsm_panel<T>, (unsigned)(rem - 1), 256, sm, st, S, n_pad, k + 1, (const T*)Linv_all,
                b, 1);
  }
  if (side_pending) GBBA_CUDA(cudaStreamWaitEvent(st, h->ev_side, 0));
  // backward substitution: each block row's kernel starts while the previous
  // one finishes (programmatic dependent launch; the first one waits fully)
  for (int kb = nb - 1; kb >= 0; --kb)
    launch_hi(h, kb != nb - 1, k_trsv_bwd<T>, (unsigned)(kb + 1), 256, sm, st, S, n_pad, kb,
              (const T*)Linv_all, b, x);
}

template <typename T>
void dense_cholesky_solve(gbba_handle* h, T* S, int64_t n_pad, T* b, T* x, T* Linv_all, int* flag, cudaStream_t st) {
  if (std::is_same<T, float>::value && h->factor_tensor)
    dense_cholesky_solve_impl<T, std::is_same<T, float>::value>(h, S, n_pad, b, x, Linv_all, flag, st);
  else
    dense_cholesky_solve_impl<T, false>(h, S, n_pad, b, x, Linv_all, flag, st);
}

template void dense_cholesky_solve_impl<float, false>(gbba_handle*, float*, int64_t, float*, float*, float*, int*,
                                                      cudaStream_t);
template void dense_cholesky_solve_impl<float, true>(gbba_handle*, float*, int64_t, float*, float*, float*, int*,
                                                     cudaStream_t);
template void dense_cholesky_prepare<double>();
template void dense_cholesky_prepare<float>();
template void dense_cholesky_solve<double>(gbba_handle*, double*, int64_t, double*, double*, double*, int*, cudaStream_t);
template void dense_cholesky_solve<float>(gbba_handle*, float*, int64_t, float*, float*, float*, int*, cudaStream_t);

}  // namespace gbba
