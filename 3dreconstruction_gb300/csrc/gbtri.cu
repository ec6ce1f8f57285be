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
// The N-view and algebraic nullspaces are computed without forming the
// 3n x (4+n) design: see nview_track below.  The same templated code runs in
// FP64 (parity path) and in FP32 (production path, followed by Gauss-Newton
// steps on the reprojection error; the block's observations are staged in
// shared memory with coalesced loads and the camera table lives in shared
// memory).
#include <cstring>

#include "gbba_internal.h"
#include "gbtri_track.cuh"

namespace gbba {

// ---------------------------------------------------------------- FP64 DLT (4x4)
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

// ------------------------------------------------------- Gauss-Newton (templated)
template <typename T>
__device__ __forceinline__ void gn_accumulate(const T* Pi, const T X[3], T px, T py, T H[6], T g[3],
                                              T* cost = nullptr) {
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
  if (cost) *cost += ru * ru + rv * rv;
}

// Squared reprojection error of X over a track's views.
template <typename T, typename Views>
__device__ __forceinline__ T reprojection_cost(const Views& view, int n, const T X[3]) {
  T e = T(0);
  for (int j = 0; j < n; ++j) {
    const T* Pi;
    T px, py;
    view(j, &Pi, &px, &py);
    T h[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) h[r] = Pi[4 * r] * X[0] + Pi[4 * r + 1] * X[1] + Pi[4 * r + 2] * X[2] + Pi[4 * r + 3];
    const T ru = h[0] / h[2] - px, rv = h[1] / h[2] - py;
    e += ru * ru + rv * rv;
  }
  return e;
}

template <typename T>
__device__ __forceinline__ void gn_apply(const T Hi[6], const T g[3], T X[3]) {
  X[0] -= Hi[0] * g[0] + Hi[1] * g[1] + Hi[2] * g[2];
  X[1] -= Hi[1] * g[0] + Hi[3] * g[1] + Hi[4] * g[2];
  X[2] -= Hi[2] * g[0] + Hi[4] * g[1] + Hi[5] * g[2];
}

__global__ void k_refine_gn64(const double* P, const int64_t* offs, const uint32_t* cam, const double* xy, int64_t nt,
                              int steps, double* X, const unsigned int* __restrict__ bad) {
  if (*bad) return;
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

// Views of one track read straight from global memory (FP64 parity path).
struct GlobalViews64 {
  const double* P;
  const uint32_t* cam;
  const double* xy;
  int64_t b;
  __device__ void operator()(int j, const double** Pj, double* x, double* y) const {
    *Pj = P + 12 * (int64_t)cam[b + j];
    *x = xy[2 * (b + j)];
    *y = xy[2 * (b + j) + 1];
  }
};

// FP64 parity path, one thread per track: X [nt][4] (NVIEW / ALGEBRAIC) or
// [nt][3] and Triangulation::error (ITERATIVE).
__global__ void __launch_bounds__(128) k_nview64(int method, const double* __restrict__ P, const int64_t* __restrict__ offs,
                                                 const uint32_t* __restrict__ cam, const double* __restrict__ xy,
                                                 int64_t nt, double* __restrict__ X, double* __restrict__ err,
                                                 const unsigned int* __restrict__ bad) {
  if (*bad) return;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = offs[t];
    const int n = (int)(offs[t + 1] - b);
    const GlobalViews64 views{P, cam, xy, b};
    if (method == 2) {
      double Xc[3];
      iterative_track<double>(views, n, Xc);
#pragma unroll
      for (int r = 0; r < 3; ++r) X[3 * t + r] = Xc[r];
      if (err) {
        // Triangulation::error: sum of the reprojection distances
        double e = 0.0;
        for (int i = 0; i < n; ++i) {
          const double* Pi;
          double px, py;
          views(i, &Pi, &px, &py);
          double hp[3];
#pragma unroll
          for (int r = 0; r < 3; ++r) hp[r] = Pi[4 * r] * Xc[0] + Pi[4 * r + 1] * Xc[1] + Pi[4 * r + 2] * Xc[2] + Pi[4 * r + 3];
          const double dx = px - hp[0] / hp[2], dy = py - hp[1] / hp[2];
          e += sqrt(dx * dx + dy * dy);
        }
        err[t] = e;
      }
      continue;
    }
    double Xh[4];
    if (method == 0) nview_track<double>(views, n, Xh);
    else algebraic_track<double>(views, n, Xh);
#pragma unroll
    for (int r = 0; r < 4; ++r) X[4 * t + r] = Xh[r];
  }
}

// FP32 production kernel: 128 tracks per block, a thread per track, the
// block's observations staged in shared memory with coalesced loads and the
// camera table in shared memory.  method: GBTRI_NVIEW (the reference's
// TriangulateNView estimator, dehomogenised), GBTRI_NVIEW_ALGEBRAIC, or
// GBTRI_ITERATIVE (Triangulation::compute(3)); then gn_steps Gauss-Newton
// steps on the reprojection error.
constexpr int kTriThreads = 128;
constexpr int kTriStage = 4096;  // observations staged per block (12 B each)
constexpr int kTriCams = 1024;   // camera table kept in shared memory up to this size

struct StagedViews32 {
  const float* sP;     // camera table in shared memory, or null
  const float* gP;     // camera table in global memory
  const uint32_t* scam;
  const float2* sxy;
  const uint32_t* gcam;
  const float2* gxy;
  uint32_t ob, b;
  bool staged;
  __device__ void operator()(int j, const float** Pj, float* x, float* y) const {
    const uint32_t o = b + (uint32_t)j;
    const uint32_t c = staged ? scam[o - ob] : gcam[o];
    *Pj = sP ? sP + 12 * c : gP + 12 * (int64_t)c;
    const float2 p = staged ? sxy[o - ob] : gxy[o];
    *x = p.x;
    *y = p.y;
  }
};

__global__ void __launch_bounds__(kTriThreads) k_tri_f32(int method, const float* __restrict__ P, int64_t ncam,
                                                         const uint32_t* __restrict__ offs, const uint32_t* __restrict__ cam,
                                                         const float2* __restrict__ xy, int64_t nt, int gn_steps,
                                                         float* __restrict__ X, uint8_t* __restrict__ status,
                                                         float* __restrict__ min_depth,
                                                         const unsigned int* __restrict__ bad) {
  if (*bad) return;
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
  const StagedViews32 views{ncam_s ? sP : nullptr, P, scam, sxy, cam, xy, ob, b, staged};
  float Xc[3] = {0.f, 0.f, 0.f};
  uint8_t st = n >= 2 ? 0 : 1;
  if (st == 0) {
    if (method == 2) {
      if (!iterative_track<float>(views, n, Xc)) st = 1;
    } else {
      float Xh[4];
      if (method == 0) nview_track<float, false>(views, n, Xh);
      else algebraic_track<float>(views, n, Xh);
      const float nrm = fabsf(Xh[0]) + fabsf(Xh[1]) + fabsf(Xh[2]);
      if (!(fabsf(Xh[3]) > 1e-6f * nrm)) {
        st = 1;
      } else {
        const float iw = 1.f / Xh[3];
        Xc[0] = Xh[0] * iw;
        Xc[1] = Xh[1] * iw;
        Xc[2] = Xh[2] * iw;
      }
    }
  }
  // Gauss-Newton steps on the reprojection error, each kept only when it
  // lowers that error (a step from a poorly conditioned linear estimate can
  // overshoot); a singular normal matrix ends the refinement and keeps X.
  for (int s = 0; s < gn_steps && st == 0; ++s) {
    float H[6] = {0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0}, Hi[6], e0 = 0.f;
    for (int j = 0; j < n; ++j) {
      const float* Pj;
      float px, py;
      views(j, &Pj, &px, &py);
      gn_accumulate<float>(Pj, Xc, px, py, H, g, &e0);
    }
    if (!inv3t<float>(H, Hi)) break;
    float Xn[3] = {Xc[0], Xc[1], Xc[2]};
    gn_apply<float>(Hi, g, Xn);
    const float e1 = reprojection_cost<float>(views, n, Xn);
    if (!(e1 <= e0)) break;
    Xc[0] = Xn[0];
    Xc[1] = Xn[1];
    Xc[2] = Xn[2];
  }
  float md = 3.402823466e38f;
  for (int j = 0; j < n; ++j) {
    const float* Pj;
    float px, py;
    views(j, &Pj, &px, &py);
    md = fminf(md, Pj[8] * Xc[0] + Pj[9] * Xc[1] + Pj[10] * Xc[2] + Pj[11]);
  }
  if (st == 0 && !(isfinite(Xc[0]) && isfinite(Xc[1]) && isfinite(Xc[2]))) st = 1;
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

// One pass over a batch's CSR offsets and camera indices: offs[0] == 0,
// non-decreasing offsets, every camera index below ncam (the camera index
// array holds offs[nt] entries).  Sets bit 0 (offsets) or bit 1 (camera
// index) of *err.  The triangulation kernels that follow on the stream read
// *err first and do nothing when it is set, so a bad batch is never indexed;
// the host reads *err once, after them.
template <typename Off>
__global__ void k_check_tracks(const Off* __restrict__ offs, int64_t nt, const uint32_t* __restrict__ cam,
                               int64_t ncam, unsigned int* __restrict__ err) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool bad_off = false, bad_cam = false;
  for (int64_t t = i0; t < nt; t += stride) {
    const int64_t a = (int64_t)offs[t], b = (int64_t)offs[t + 1];
    if (b < a || (t == 0 && a != 0)) bad_off = true;
  }
  const int64_t no = (int64_t)offs[nt];
  for (int64_t o = i0; o < no; o += stride)
    if (cam[o] >= ncam) bad_cam = true;
  if (bad_off) atomicOr(err, 1u);
  if (bad_cam) atomicOr(err, 2u);
}

// Observation count of a batch (offs[nt]): read on the host for host memory
// (the copies need it), not needed for device memory.
template <typename Off>
int64_t host_total(const Off* offs, int64_t nt, int memory) {
  if (memory == GBBA_MEMORY_DEVICE) return 0;
  GBBA_REQUIRE(offs[0] == 0 && (int64_t)offs[nt] >= 0, GBBA_ERROR_INVALID_ARGUMENT,
               "track_offsets must start at 0 and be non-decreasing");
  return (int64_t)offs[nt];
}

template <typename Off>
unsigned int* launch_check(gbba_handle* h, const Off* doff, int64_t nt, const uint32_t* dcam, int64_t ncam) {
  unsigned int* err = h->arena.take<unsigned int>(1);
  GBBA_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned int), h->active));
  k_check_tracks<Off><<<std::max(1, std::min<int>((int)ceil_div(nt, 256), h->sm_count * 8)), 256, 0, h->active>>>(
      doff, nt, dcam, ncam, err);
  check_launch(h);
  return err;
}

// Waits for the call's work and turns the check bits into a status.
void finish_check(gbba_handle* h, const unsigned int* err) {
  unsigned int* hp = reinterpret_cast<unsigned int*>(h->pinned + 128);
  GBBA_CUDA(cudaMemcpyAsync(hp, err, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->active));
  GBBA_CUDA(cudaStreamSynchronize(h->active));
  GBBA_REQUIRE((*hp & 1u) == 0, GBBA_ERROR_INVALID_ARGUMENT, "track_offsets must start at 0 and be non-decreasing");
  GBBA_REQUIRE((*hp & 2u) == 0, GBBA_ERROR_INVALID_ARGUMENT, "camera_index out of range");
}

// Device time of the call's main kernel, kept in the handle (gbba_last_kernel_time).
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
    const int64_t no = host_total(track_offsets, num_tracks, memory);
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
    const unsigned int* bad = launch_check(h, doff, num_tracks, dcam, num_cameras);
    KernelTimer timer(h);
    k_nview64<<<std::max(1, std::min<int>((int)ceil_div(num_tracks, 128), h->sm_count * 16)), 128, 0, h->active>>>(
        method, dP, doff, dcam, dxy, num_tracks, dX, method == GBTRI_ITERATIVE ? derr : nullptr, bad);
    timer.stop();
    check_launch(h);
    out_back(h, X, dX, xo * num_tracks, memory);
    if (method == GBTRI_ITERATIVE) out_back(h, error, derr, num_tracks, memory);
    finish_check(h, bad);
    return GBBA_SUCCESS;
  });
}

gbba_status gbtri_nview_batched_f32(gbba_handle* h, int32_t method, const float* P, int64_t num_cameras,
                                    const uint32_t* track_offsets, const uint32_t* camera_index, const float* xy,
                                    int64_t num_tracks, int32_t gn_steps, float* X, uint8_t* status, float* min_depth,
                                    int32_t memory) {
  if (method < 0 || method > 2 || num_tracks < 0 || num_cameras < 0 || gn_steps < 0 || !P || !track_offsets || !X)
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (num_tracks >= 0xFFFFFFFFLL) return GBBA_ERROR_TOO_LARGE;
  return tri_guard(h, [&]() {
    if (num_tracks == 0) return GBBA_SUCCESS;
    const int64_t no = host_total(track_offsets, num_tracks, memory);
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
    const unsigned int* bad = launch_check(h, doff, num_tracks, dcam, num_cameras);
    const size_t smem = tri_f32_smem(num_cameras);
    static PerDeviceOnce once;
    once.run([] {
      GBBA_CUDA(cudaFuncSetAttribute(k_tri_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tri_f32_smem(kTriCams)));
    });
    KernelTimer timer(h);
    k_tri_f32<<<(unsigned)ceil_div(num_tracks, kTriThreads), kTriThreads, smem, h->active>>>(
        method, dP, num_cameras, doff, dcam, reinterpret_cast<const float2*>(dxy), num_tracks, gn_steps, dX, dst, dmd,
        bad);
    timer.stop();
    check_launch(h);
    out_back(h, X, dX, 3 * num_tracks, memory);
    out_back(h, status, dst, num_tracks, memory);
    out_back(h, min_depth, dmd, num_tracks, memory);
    finish_check(h, bad);
    return GBBA_SUCCESS;
  });
}

gbba_status gbtri_refine_gn(gbba_handle* h, const double* P, int64_t num_cameras, const int64_t* track_offsets,
                            const uint32_t* camera_index, const double* xy, int64_t num_tracks, int32_t steps, double* X,
                            int32_t memory) {
  if (num_tracks < 0 || steps < 0 || !P || !track_offsets || !X) return GBBA_ERROR_INVALID_ARGUMENT;
  return tri_guard(h, [&]() {
    if (num_tracks == 0) return GBBA_SUCCESS;
    const int64_t no = host_total(track_offsets, num_tracks, memory);
    h->arena.reset();
    h->arena.reserve(sizeof(double) * (12 * num_cameras + 2 * no + 3 * num_tracks) + sizeof(int64_t) * (num_tracks + 1) +
                     sizeof(uint32_t) * no + 16 * 256);
    const double* dP = in_view(h, P, 12 * (size_t)num_cameras, memory);
    const int64_t* doff = in_view(h, track_offsets, num_tracks + 1, memory);
    const uint32_t* dcam = in_view(h, camera_index, no, memory);
    const double* dxy = in_view(h, xy, 2 * no, memory);
    double* dX = const_cast<double*>(in_view(h, (const double*)X, 3 * num_tracks, memory));
    const unsigned int* bad = launch_check(h, doff, num_tracks, dcam, num_cameras);
    KernelTimer timer(h);
    k_refine_gn64<<<std::max(1, std::min<int>((int)ceil_div(num_tracks, 128), h->sm_count * 16)), 128, 0, h->active>>>(
        dP, doff, dcam, dxy, num_tracks, steps, dX, bad);
    timer.stop();
    check_launch(h);
    out_back(h, X, dX, 3 * num_tracks, memory);
    finish_check(h, bad);
    return GBBA_SUCCESS;
  });
}

}  // extern "C"
