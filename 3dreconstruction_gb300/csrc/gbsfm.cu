// Engine-side scans of the incremental reconstruction (include/gbsfm.h): the
// pair triangulation with its keep filter, the bad-track rejection and the
// residual statistics, one thread per match or per track.  They restate the
// element-wise loops of
//   triangulate2View_Vector   libs/sfm/include/mvg/sfm/sfm_robust.h:152-195
//   Resection / MakeInitialPair3D keep decisions
//                             libs/sfm/src/sfm_incremental_engine.cpp:977-1029, 492-533
//   badTrackRejector          :1047-1140
//   ComputeResidualsHistogram :1550-1616
// on the BrownPinholeCamera model (libs/camera/include/mvg/camera/
// brown_pinhole_camera.h:15-140) in FP64.  The scans are HBM-bound: a match
// reads 32 B and writes 33 B, an observation reads 20 B plus its camera
// (cached) and its track's point.
#include <cstdlib>
#include <cstring>

#include <cub/device/device_radix_sort.cuh>

#include "../../include/gbsfm.h"
#include "gbba_internal.h"
#include "gbba_device.cuh"
#include "gbtri_track.cuh"

namespace gbba {
namespace {

// BrownPinholeCamera::Project: R X + t, x/z, the radial K3 factor, f and the
// principal point; the depth is (R X + t)_z (mvg::camera::Depth).
__device__ __forceinline__ void brown_project(const gbsfm_camera& c, const double X[3], double* u, double* v,
                                              double* depth) {
  double p[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) p[r] = c.R[3 * r] * X[0] + c.R[3 * r + 1] * X[1] + c.R[3 * r + 2] * X[2] + c.t[r];
  const double xe = p[0] / p[2], ye = p[1] / p[2];
  const double r2 = xe * xe + ye * ye, r4 = r2 * r2, r6 = r4 * r2;
  const double rc = 1.0 + c.k1 * r2 + c.k2 * r4 + c.k3 * r6;
  *u = c.ppx + c.f * (xe * rc);
  *v = c.ppy + c.f * (ye * rc);
  *depth = p[2];
}

__device__ __forceinline__ double brown_residual(const gbsfm_camera& c, const double X[3], double x, double y,
                                                 double* depth) {
  double u, v;
  brown_project(c, X, &u, &v, depth);
  return sqrt((x - u) * (x - u) + (y - v) * (y - v));
}

// P = K [R | t] (P_From_KRt).
__device__ __forceinline__ void projection_matrix(const gbsfm_camera& c, double P[12]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const double r0 = j < 3 ? c.R[j] : c.t[0], r1 = j < 3 ? c.R[3 + j] : c.t[1], r2 = j < 3 ? c.R[6 + j] : c.t[2];
    P[j] = c.f * r0 + c.ppx * r2;
    P[4 + j] = c.f * r1 + c.ppy * r2;
    P[8 + j] = r2;
  }
}

// PinholeCamera::Residual(P, X, x): |x - Project(P, X)|.
__device__ __forceinline__ double pinhole_residual(const double P[12], const double X[3], double x, double y) {
  double h[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) h[r] = P[4 * r] * X[0] + P[4 * r + 1] * X[1] + P[4 * r + 2] * X[2] + P[4 * r + 3];
  const double u = h[0] / h[2], v = h[1] / h[2];
  return sqrt((x - u) * (x - u) + (y - v) * (y - v));
}

// Unit ray of pixel (x, y) in world axes: R^T K^-1 (x, y, 1), normalised.
__device__ __forceinline__ void pixel_ray(const gbsfm_camera& c, double x, double y, double ray[3]) {
  const double k[3] = {(x - c.ppx) / c.f, (y - c.ppy) / c.f, 1.0};
  double n2 = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    ray[i] = c.R[i] * k[0] + c.R[3 + i] * k[1] + c.R[6 + i] * k[2];
    n2 += ray[i] * ray[i];
  }
  const double in = 1.0 / sqrt(n2);
#pragma unroll
  for (int i = 0; i < 3; ++i) ray[i] *= in;
}

// R2D(acos(clamp(cosine, -1 + 1e-8, 1 - 1e-8))).
__device__ __forceinline__ double angle_deg(double cosine) {
  const double cl = fmin(fmax(cosine, -1.0 + 1.e-8), 1.0 - 1.e-8);
  return acos(cl) * (180.0 / 3.14159265358979323846);
}

__global__ void __launch_bounds__(256) k_triangulate_pair(gbsfm_camera c1, gbsfm_camera c2, int64_t n,
                                                          const double* __restrict__ x1, const double* __restrict__ x2,
                                                          const uint8_t* __restrict__ inlier, double th1, double th2,
                                                          double min_angle, double* __restrict__ Xout,
                                                          double* __restrict__ res, uint8_t* __restrict__ keep,
                                                          unsigned long long* __restrict__ kept) {
  double P1[12], P2[12];
  projection_matrix(c1, P1);
  projection_matrix(c2, P2);
  unsigned int count = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double a0 = x1[2 * i], a1 = x1[2 * i + 1], b0 = x2[2 * i], b1 = x2[2 * i + 1];
    // TriangulateDLT (triangulation.cpp:10-29), Euclidean
    double D[4][4], Xh[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      D[0][j] = a0 * P1[8 + j] - P1[j];
      D[1][j] = a1 * P1[8 + j] - P1[4 + j];
      D[2][j] = b0 * P2[8 + j] - P2[j];
      D[3][j] = b1 * P2[8 + j] - P2[4 + j];
    }
    jacobi_nullspace4(D, Xh);
    const double X[3] = {Xh[0] / Xh[3], Xh[1] / Xh[3], Xh[2] / Xh[3]};
    if (Xout) {
      Xout[3 * i] = X[0];
      Xout[3 * i + 1] = X[1];
      Xout[3 * i + 2] = X[2];
    }
    if (res) res[i] = (pinhole_residual(P1, X, a0, a1) + pinhole_residual(P2, X, b0, b1)) / 2.0;
    double d1, d2;
    const double r1 = brown_residual(c1, X, a0, a1, &d1), r2 = brown_residual(c2, X, b0, b1, &d2);
    bool k = (!inlier || inlier[i] != 0) && r1 < th1 && r2 < th2 && d1 > 0 && d2 > 0;
    if (k) {
      double ra[3], rb[3];
      pixel_ray(c1, a0, a1, ra);
      pixel_ray(c2, b0, b1, rb);
      const double mag = sqrt((ra[0] * ra[0] + ra[1] * ra[1] + ra[2] * ra[2]) * (rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]));
      k = angle_deg((ra[0] * rb[0] + ra[1] * rb[1] + ra[2] * rb[2]) / mag) > min_angle;
    }
    if (keep) keep[i] = k ? 1 : 0;
    count += k ? 1u : 0u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
  if ((threadIdx.x & 31) == 0 && count) atomicAdd(kept, (unsigned long long)count);
}

// One thread per track: the residual test per measurement, the largest angle
// between the first ray (the observation of the lowest camera index) and the
// others, and the removal of a track left with fewer than two measurements.
__global__ void __launch_bounds__(128) k_reject_tracks(const gbsfm_camera* __restrict__ cams, const double* __restrict__ pts,
                                                       int64_t nt, const int64_t* __restrict__ offs,
                                                       const uint32_t* __restrict__ cam, const double* __restrict__ xy,
                                                       double precision, double min_angle,
                                                       uint8_t* __restrict__ obs_keep, uint8_t* __restrict__ track_keep,
                                                       unsigned long long* __restrict__ counts) {
  unsigned int erased_total = 0, removed = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = offs[t], e = offs[t + 1];
    const double X[3] = {pts[3 * t], pts[3 * t + 1], pts[3 * t + 2]};
    // origin: the observation of the lowest camera index
    int64_t first = b;
    for (int64_t o = b + 1; o < e; ++o)
      if (cam[o] < cam[first]) first = o;
    double origin[3] = {0.0, 0.0, 0.0};
    if (e > b) {
      const gbsfm_camera& c = cams[cam[first]];
      double C[3], n2 = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        C[i] = -(c.R[i] * c.t[0] + c.R[3 + i] * c.t[1] + c.R[6 + i] * c.t[2]);  // camera_center_ = -R^T t
        origin[i] = X[i] - C[i];
        n2 += origin[i] * origin[i];
      }
      const double in = 1.0 / sqrt(n2);
#pragma unroll
      for (int i = 0; i < 3; ++i) origin[i] *= in;
    }
    double max_angle = 0.0;
    unsigned int erased = 0;
    for (int64_t o = b; o < e; ++o) {
      const gbsfm_camera& c = cams[cam[o]];
      double depth;
      const double r = brown_residual(c, X, xy[2 * o], xy[2 * o + 1], &depth);
      if (o != first) {
        double dir[3], n2 = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const double Ci = -(c.R[i] * c.t[0] + c.R[3 + i] * c.t[1] + c.R[6 + i] * c.t[2]);
          dir[i] = X[i] - Ci;
          n2 += dir[i] * dir[i];
        }
        const double in = 1.0 / sqrt(n2);
        const double dot = (origin[0] * dir[0] + origin[1] * dir[1] + origin[2] * dir[2]) * in;
        max_angle = fmax(max_angle, angle_deg(dot));
      }
      const bool bad = r > precision;
      erased += bad ? 1u : 0u;
      if (obs_keep) obs_keep[o] = bad ? 0 : 1;
    }
    const bool narrow = max_angle < min_angle;
    if (narrow) {
      erased = (unsigned int)(e - b);
      if (obs_keep)
        for (int64_t o = b; o < e; ++o) obs_keep[o] = 0;
    }
    const bool gone = erased > 0 && (e - b) - (int64_t)erased < 2;
    if (track_keep) track_keep[t] = gone ? 0 : 1;
    erased_total += erased;
    removed += gone ? 1u : 0u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    erased_total += __shfl_xor_sync(0xffffffffu, erased_total, o);
    removed += __shfl_xor_sync(0xffffffffu, removed, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (erased_total) atomicAdd(&counts[0], (unsigned long long)erased_total);
    if (removed) atomicAdd(&counts[1], (unsigned long long)removed);
  }
}

// Residual of every measurement, rounded to float as the reference stores it.
__global__ void __launch_bounds__(128) k_track_residuals(const gbsfm_camera* __restrict__ cams,
                                                         const double* __restrict__ pts, int64_t nt,
                                                         const int64_t* __restrict__ offs,
                                                         const uint32_t* __restrict__ cam,
                                                         const double* __restrict__ xy, float* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    const double X[3] = {pts[3 * t], pts[3 * t + 1], pts[3 * t + 2]};
    for (int64_t o = offs[t]; o < offs[t + 1]; ++o) {
      double depth;
      out[o] = (float)brown_residual(cams[cam[o]], X, xy[2 * o], xy[2 * o + 1], &depth);
    }
  }
}

// Over the sorted residuals: partial sums (in double) per block, and the
// histogram Histogram<double>(min, max, 10).Add: below min -> underflow, else
// bin (size_t)((x - min) * (10 / (max - min))), 10 or more -> overflow.
__global__ void __launch_bounds__(256) k_residual_stats(const float* __restrict__ sorted, int64_t n,
                                                        double* __restrict__ part,
                                                        unsigned long long* __restrict__ hist) {
  __shared__ unsigned int sh_hist[12];
  __shared__ double sh_sum[8];
  if (threadIdx.x < 12) sh_hist[threadIdx.x] = 0;
  __syncthreads();
  const double start = sorted[0], end = sorted[n - 1];
  const double per = 10.0 / (end - start);
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = sorted[i];
    s += x;
    if (x < start) {
      atomicAdd(&sh_hist[10], 1u);
    } else {
      const double f = (x - start) * per;
      const unsigned long long bin = (unsigned long long)f;
      atomicAdd(&sh_hist[bin < 10 ? bin : 11], 1u);
    }
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh_sum[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sh_sum[w];
    part[blockIdx.x] = t;
  }
  if (threadIdx.x < 12 && sh_hist[threadIdx.x]) atomicAdd(&hist[threadIdx.x], (unsigned long long)sh_hist[threadIdx.x]);
}

template <typename F>
gbba_status sfm_guard(gbba_handle* h, F&& f) {
  if (!h) return GBBA_ERROR_INVALID_ARGUMENT;
  try {
    GBBA_CUDA(cudaSetDevice(h->device));
    h->active = h->stream;
    return f();
  } catch (const Error& e) {
    if (std::getenv("GBBA_VERBOSE")) fprintf(stderr, "gbsfm: %s\n", e.what.c_str());
    cudaGetLastError();
    return e.status;
  }
}

// Device views of a batch of tracks.  Offsets and camera indices are checked
// on the host first, so a bad batch is never indexed.
struct TrackBatch {
  const gbsfm_camera* cams;
  const double *pts, *xy;
  const int64_t* offs;
  const uint32_t* cam;
  int64_t no;
};

// The batch's observation count, after the host has checked the offsets
// (offs[0] == 0, non-decreasing) and every camera index (below nc).
int64_t check_tracks(gbba_handle* h, const gbsfm_camera* cameras, int64_t nc, const double* points, int64_t nt,
                     const int64_t* offs, const uint32_t* cam, const double* xy, int memory) {
  GBBA_REQUIRE(cameras && offs && (nt == 0 || points), GBBA_ERROR_INVALID_ARGUMENT, "NULL array");
  std::vector<int64_t> ho(nt + 1);
  if (memory == GBBA_MEMORY_DEVICE) {
    GBBA_CUDA(cudaMemcpyAsync(ho.data(), offs, sizeof(int64_t) * (nt + 1), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
  } else {
    std::memcpy(ho.data(), offs, sizeof(int64_t) * (nt + 1));
  }
  GBBA_REQUIRE(ho[0] == 0, GBBA_ERROR_INVALID_ARGUMENT, "track_offsets[0] must be 0");
  for (int64_t t = 0; t < nt; ++t)
    GBBA_REQUIRE(ho[t + 1] >= ho[t], GBBA_ERROR_INVALID_ARGUMENT, "track_offsets must be non-decreasing");
  const int64_t no = ho[nt];
  GBBA_REQUIRE(no == 0 || (cam && xy), GBBA_ERROR_INVALID_ARGUMENT, "NULL array");
  if (no) {
    std::vector<uint32_t> hc(no);
    if (memory == GBBA_MEMORY_DEVICE) {
      GBBA_CUDA(cudaMemcpyAsync(hc.data(), cam, sizeof(uint32_t) * no, cudaMemcpyDeviceToHost, h->active));
      GBBA_CUDA(cudaStreamSynchronize(h->active));
    } else {
      std::memcpy(hc.data(), cam, sizeof(uint32_t) * no);
    }
    for (int64_t o = 0; o < no; ++o)
      GBBA_REQUIRE(hc[o] < (uint64_t)nc, GBBA_ERROR_INVALID_ARGUMENT, "camera_index out of range");
  }
  return no;
}

// Device views of a checked batch, with `extra` bytes of the arena left for
// the call's own outputs and scratch.
TrackBatch stage_tracks(gbba_handle* h, const gbsfm_camera* cameras, int64_t nc, const double* points, int64_t nt,
                        const int64_t* offs, const uint32_t* cam, const double* xy, int memory, int64_t no,
                        size_t extra) {
  h->arena.reset();
  h->arena.reserve(sizeof(gbsfm_camera) * nc + sizeof(double) * (3 * nt + 2 * no) + sizeof(int64_t) * (nt + 1) +
                   sizeof(uint32_t) * no + extra + 16 * 256);
  TrackBatch tb;
  tb.cams = in_view(h, cameras, nc, memory);
  tb.pts = in_view(h, points, 3 * nt, memory);
  tb.offs = in_view(h, offs, nt + 1, memory);
  tb.cam = in_view(h, cam, no, memory);
  tb.xy = in_view(h, xy, 2 * no, memory);
  tb.no = no;
  return tb;
}

unsigned grid_for(gbba_handle* h, int64_t n, int threads) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), (int64_t)h->sm_count * 16));
}

}  // namespace
}  // namespace gbba

using namespace gbba;

extern "C" {

gbba_status gbsfm_triangulate_pair(gbba_handle* h, const gbsfm_camera* cam1, const gbsfm_camera* cam2, int64_t n,
                                   const double* x1, const double* x2, const uint8_t* inlier, double max_residual1,
                                   double max_residual2, double min_angle_deg, double* X, double* residual,
                                   uint8_t* keep, int64_t* num_kept, int32_t memory) {
  if (!cam1 || !cam2 || n < 0 || (n > 0 && (!x1 || !x2))) return GBBA_ERROR_INVALID_ARGUMENT;
  return sfm_guard(h, [&]() {
    if (num_kept) *num_kept = 0;
    if (n == 0) return GBBA_SUCCESS;
    h->arena.reset();
    h->arena.reserve(sizeof(double) * 8 * n + 2 * n + 16 * 256);
    const double* d1 = in_view(h, x1, 2 * n, memory);
    const double* d2 = in_view(h, x2, 2 * n, memory);
    const uint8_t* din = in_view(h, inlier, n, memory);
    double* dX = out_view(h, X, 3 * n, memory);
    double* dr = out_view(h, residual, n, memory);
    uint8_t* dk = out_view(h, keep, n, memory);
    unsigned long long* kept = h->arena.take<unsigned long long>(1);
    GBBA_CUDA(cudaMemsetAsync(kept, 0, sizeof(unsigned long long), h->active));
    k_triangulate_pair<<<grid_for(h, n, 256), 256, 0, h->active>>>(*cam1, *cam2, n, d1, d2, din, max_residual1,
                                                                   max_residual2, min_angle_deg, dX, dr, dk, kept);
    check_launch(h);
    out_back(h, X, dX, 3 * n, memory);
    out_back(h, residual, dr, n, memory);
    out_back(h, keep, dk, n, memory);
    unsigned long long* hk = reinterpret_cast<unsigned long long*>(h->pinned + 176);
    GBBA_CUDA(cudaMemcpyAsync(hk, kept, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    if (num_kept) *num_kept = (int64_t)*hk;
    return GBBA_SUCCESS;
  });
}

gbba_status gbsfm_reject_tracks(gbba_handle* h, const gbsfm_camera* cameras, int64_t num_cameras, const double* points,
                                int64_t num_tracks, const int64_t* track_offsets, const uint32_t* camera_index,
                                const double* xy, double precision, double min_track_angle_deg, uint8_t* obs_keep,
                                uint8_t* track_keep, int64_t* rejected_measurements, int64_t* rejected_tracks,
                                int32_t memory) {
  if (num_cameras < 0 || num_tracks < 0) return GBBA_ERROR_INVALID_ARGUMENT;
  return sfm_guard(h, [&]() {
    if (rejected_measurements) *rejected_measurements = 0;
    if (rejected_tracks) *rejected_tracks = 0;
    if (num_tracks == 0) return GBBA_SUCCESS;
    const int64_t no = check_tracks(h, cameras, num_cameras, points, num_tracks, track_offsets, camera_index, xy,
                                    memory);
    const TrackBatch tb = stage_tracks(h, cameras, num_cameras, points, num_tracks, track_offsets, camera_index, xy,
                                       memory, no, no + num_tracks + 1024);
    uint8_t* dok = out_view(h, obs_keep, tb.no, memory);
    uint8_t* dtk = out_view(h, track_keep, num_tracks, memory);
    unsigned long long* counts = h->arena.take<unsigned long long>(2);
    GBBA_CUDA(cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), h->active));
    k_reject_tracks<<<grid_for(h, num_tracks, 128), 128, 0, h->active>>>(tb.cams, tb.pts, num_tracks, tb.offs, tb.cam,
                                                                         tb.xy, precision, min_track_angle_deg, dok,
                                                                         dtk, counts);
    check_launch(h);
    out_back(h, obs_keep, dok, tb.no, memory);
    out_back(h, track_keep, dtk, num_tracks, memory);
    unsigned long long* hc = reinterpret_cast<unsigned long long*>(h->pinned + 176);
    GBBA_CUDA(cudaMemcpyAsync(hc, counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    if (rejected_measurements) *rejected_measurements = (int64_t)hc[0];
    if (rejected_tracks) *rejected_tracks = (int64_t)hc[1];
    return GBBA_SUCCESS;
  });
}

gbba_status gbsfm_residual_histogram(gbba_handle* h, const gbsfm_camera* cameras, int64_t num_cameras,
                                     const double* points, int64_t num_tracks, const int64_t* track_offsets,
                                     const uint32_t* camera_index, const double* xy, gbsfm_residual_stats* stats,
                                     int32_t memory) {
  if (num_cameras < 0 || num_tracks < 0 || !stats) return GBBA_ERROR_INVALID_ARGUMENT;
  return sfm_guard(h, [&]() {
    std::memset(stats, 0, sizeof(*stats));
    if (num_tracks == 0) return GBBA_SUCCESS;
    const int64_t no = check_tracks(h, cameras, num_cameras, points, num_tracks, track_offsets, camera_index, xy,
                                    memory);
    GBBA_REQUIRE(no <= 0x7fffffffLL, GBBA_ERROR_TOO_LARGE, "too many observations for one sort");
    size_t sort_bytes = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, (const float*)nullptr, (float*)nullptr, (int)no);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(no, 256), 1024));
    const TrackBatch tb = stage_tracks(h, cameras, num_cameras, points, num_tracks, track_offsets, camera_index, xy,
                                       memory, no, 2 * sizeof(float) * no + sort_bytes + sizeof(double) * nb + 2048);
    stats->count = tb.no;
    if (tb.no <= 1) {
      GBBA_CUDA(cudaStreamSynchronize(h->active));
      return GBBA_SUCCESS;
    }
    float* res = h->arena.take<float>(tb.no);
    float* sorted = h->arena.take<float>(tb.no);
    void* tmp = h->arena.take<char>(sort_bytes);
    double* part = h->arena.take<double>(nb);
    unsigned long long* hist = h->arena.take<unsigned long long>(12);
    GBBA_CUDA(cudaMemsetAsync(hist, 0, 12 * sizeof(unsigned long long), h->active));
    k_track_residuals<<<grid_for(h, num_tracks, 128), 128, 0, h->active>>>(tb.cams, tb.pts, num_tracks, tb.offs,
                                                                           tb.cam, tb.xy, res);
    check_launch(h);
    size_t bytes = sort_bytes;
    GBBA_CUDA(cub::DeviceRadixSort::SortKeys(tmp, bytes, res, sorted, (int)tb.no, 0, 32, h->active));
    count_launch(h, 4);
    k_residual_stats<<<nb, 256, 0, h->active>>>(sorted, tb.no, part, hist);
    check_launch(h);
    std::vector<double> hp(nb);
    unsigned long long hh[12];
    float ends[3];
    GBBA_CUDA(cudaMemcpyAsync(hp.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaMemcpyAsync(hh, hist, sizeof(hh), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaMemcpyAsync(&ends[0], sorted, sizeof(float), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaMemcpyAsync(&ends[1], sorted + tb.no - 1, sizeof(float), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaMemcpyAsync(&ends[2], sorted + tb.no / 2, sizeof(float), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    double sum = 0.0;
    for (double v : hp) sum += v;
    stats->min = ends[0];
    stats->max = ends[1];
    stats->median = ends[2];
    stats->mean = (float)(sum / (double)tb.no);  // MinMaxMeanMedian<float> stores the mean as float
    for (int i = 0; i < 10; ++i) stats->hist[i] = (int64_t)hh[i];
    stats->underflow = (int64_t)hh[10];
    stats->overflow = (int64_t)hh[11];
    return GBBA_SUCCESS;
  });
}

}  // extern "C"
