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

// ---- Problem assembly ------------------------------------------------------

// ceres::RotationMatrixToQuaternion (Shoemake's branch on the trace, then on
// the largest diagonal entry; include/ceres/rotation.h:312-350) followed by
// QuaternionToAngleAxis (:266-306), which maps a rotation of more than pi
// back below pi through atan2 of the negated pair.  R is row-major:
// R(i, j) = R[3 i + j].
__device__ void rotation_to_angle_axis(const double* R, double aa[3]) {
  double q[4];
  const double trace = R[0] + R[4] + R[8];
  if (trace >= 0.0) {
    double s = sqrt(trace + 1.0);
    q[0] = 0.5 * s;
    s = 0.5 / s;
    q[1] = (R[7] - R[5]) * s;
    q[2] = (R[2] - R[6]) * s;
    q[3] = (R[3] - R[1]) * s;
  } else {
    int i = R[4] > R[0] ? 1 : 0;
    if (R[8] > R[4 * i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double s = sqrt(R[4 * i] - R[4 * j] - R[4 * k] + 1.0);
    q[i + 1] = 0.5 * s;
    s = 0.5 / s;
    q[0] = (R[3 * k + j] - R[3 * j + k]) * s;
    q[j + 1] = (R[3 * j + i] + R[3 * i + j]) * s;
    q[k + 1] = (R[3 * k + i] + R[3 * i + k]) * s;
  }
  const double sin2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  double scale = 2.0;  // zero rotation: the first term of the series
  if (sin2 > 0.0) {
    const double sn = sqrt(sin2), cs = q[0];
    scale = 2.0 * (cs < 0.0 ? atan2(-sn, -cs) : atan2(sn, cs)) / sn;
  }
  aa[0] = q[1] * scale;
  aa[1] = q[2] * scale;
  aa[2] = q[3] * scale;
}

// ceres::AngleAxisToRotationMatrix (include/ceres/rotation.h:377-414), row-major
// output: Rodrigues' formula with the unit axis, or its first-order form when
// theta^2 is not above the double epsilon.
__device__ void angle_axis_to_rotation(const double aa[3], double R[9]) {
  const double th2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
  if (th2 > 2.220446049250313e-16) {
    const double th = sqrt(th2);
    const double wx = aa[0] / th, wy = aa[1] / th, wz = aa[2] / th;
    double sn, cs;
    sincos(th, &sn, &cs);
    const double oc = 1.0 - cs;
    R[0] = cs + wx * wx * oc;
    R[1] = wx * wy * oc - wz * sn;
    R[2] = wy * sn + wx * wz * oc;
    R[3] = wz * sn + wx * wy * oc;
    R[4] = cs + wy * wy * oc;
    R[5] = -wx * sn + wy * wz * oc;
    R[6] = -wy * sn + wx * wz * oc;
    R[7] = wx * sn + wy * wz * oc;
    R[8] = cs + wz * wz * oc;
  } else {
    R[0] = 1.0;
    R[1] = -aa[2];
    R[2] = aa[1];
    R[3] = aa[2];
    R[4] = 1.0;
    R[5] = -aa[0];
    R[6] = -aa[1];
    R[7] = aa[0];
    R[8] = 1.0;
  }
}

constexpr uint32_t kNoCamera = 0xffffffffu;
constexpr int kPackThreads = 256;
constexpr int kPackPer = 8;  // entries per thread and tile: a tile is 2048 entries
constexpr int64_t kPackTile = (int64_t)kPackThreads * kPackPer;

// Error bits of the pack and the write-back.
enum : unsigned long long {
  kBadImage = 1,       // an entry names an image outside the state
  kBadFeature = 2,     // an entry names a feature outside its image
  kBadOffsets = 4,     // track_offsets is not a CSR of num_entries entries
  kBadGroup = 8,       // an intrinsic group outside the groups
  kLockPastEnd = 16,   // the reference's lock reads past its observations
  kBadCameraImage = 32 // a write-back ordinal names an image outside the state
};

// Exclusive block-wide count of `flag` over blockDim.x <= 1024 threads;
// returns the thread's offset and leaves the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive_count(bool flag, uint32_t* sh_warp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const unsigned mask = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) sh_warp[warp] = __popc(mask);
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (int w = 0; w < nw; ++w) {
    const uint32_t c = sh_warp[w];
    before += w < warp ? c : 0u;
    all += c;
  }
  __syncthreads();  // sh_warp is reused by the next call
  *total = all;
  return before + __popc(mask & ((1u << lane) - 1u));
}

// One block over the images: camera ordinals (ascending image id among the
// reconstructed, the key order of map_Camera), the extrinsic blocks
// [angle-axis, t] and the ordinal -> image table.
__global__ void __launch_bounds__(1024) k_pack_images(int64_t ni, const uint8_t* __restrict__ rec,
                                                      const gbsfm_camera* __restrict__ cams,
                                                      const uint32_t* __restrict__ group, int64_t num_groups,
                                                      uint32_t* __restrict__ ordinal, double* __restrict__ ext,
                                                      uint32_t* __restrict__ camera_image,
                                                      unsigned long long* __restrict__ counters) {
  __shared__ uint32_t sh_warp[32];
  uint32_t base = 0;
  unsigned long long err = 0;
  for (int64_t c0 = 0; c0 < ni; c0 += blockDim.x) {
    const int64_t i = c0 + threadIdx.x;
    const bool flag = i < ni && rec[i] != 0;
    uint32_t total;
    const uint32_t pos = base + block_exclusive_count(flag, sh_warp, &total);
    if (i < ni) ordinal[i] = flag ? pos : kNoCamera;
    if (flag) {
      const gbsfm_camera& c = cams[i];
      double aa[3];
      rotation_to_angle_axis(c.R, aa);
      double* e = ext + 6 * (int64_t)pos;
      e[0] = aa[0];
      e[1] = aa[1];
      e[2] = aa[2];
      e[3] = c.t[0];
      e[4] = c.t[1];
      e[5] = c.t[2];
      if (camera_image) camera_image[pos] = (uint32_t)i;
      if (group[i] >= (uint64_t)num_groups) err |= kBadGroup;
    }
    base += total;
  }
  if (err) atomicOr(&counters[2], err);
  if (threadIdx.x == 0) counters[0] = base;
}

__device__ __forceinline__ bool entry_kept(int64_t e, int64_t ne, int64_t ni, const uint32_t* __restrict__ img,
                                           const uint32_t* __restrict__ ordinal, uint32_t* im) {
  if (e >= ne) return false;
  *im = img[e];
  return *im < (uint64_t)ni && ordinal[*im] != kNoCamera;
}

// Pass 1 over the entries: kept entries per tile of 2048, and the checks of
// the image ids and of the track offsets.
__global__ void __launch_bounds__(kPackThreads) k_pack_count(int64_t ne, int64_t ni, int64_t nt,
                                                             const int64_t* __restrict__ offs,
                                                             const uint32_t* __restrict__ img,
                                                             const uint32_t* __restrict__ ordinal,
                                                             uint32_t* __restrict__ tile_count,
                                                             unsigned long long* __restrict__ counters) {
  __shared__ uint32_t sh_warp[32];
  unsigned long long err = 0;
  uint32_t kept = 0;
  const int64_t tile = blockIdx.x * kPackTile;
#pragma unroll
  for (int j = 0; j < kPackPer; ++j) {
    const int64_t e = tile + j * kPackThreads + threadIdx.x;
    uint32_t im = 0;
    kept += entry_kept(e, ne, ni, img, ordinal, &im) ? 1u : 0u;
    if (e < ne && im >= (uint64_t)ni) err |= kBadImage;
  }
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t <= nt; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = offs[t];
    const bool bad = (t == 0 && o != 0) || (t == nt && o != ne) || (t < nt && offs[t + 1] < o);
    if (bad) err |= kBadOffsets;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
  if ((threadIdx.x & 31) == 0) sh_warp[threadIdx.x >> 5] = kept;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < kPackThreads / 32; ++w) s += sh_warp[w];
    tile_count[blockIdx.x] = s;
  }
  if (err) atomicOr(&counters[2], err);
}

// Exclusive scan of the tile counts in place (one block); the total is the
// observation count.
__global__ void __launch_bounds__(1024) k_pack_scan(uint32_t* __restrict__ tile_count, int64_t nb,
                                                    unsigned long long* __restrict__ counters) {
  __shared__ uint32_t sh[1024];
  __shared__ unsigned long long sh_base;
  if (threadIdx.x == 0) sh_base = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < nb; c0 += 1024) {
    const int64_t i = c0 + threadIdx.x;
    const uint32_t v = i < nb ? tile_count[i] : 0u;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {  // Hillis-Steele inclusive scan
      const uint32_t add = threadIdx.x >= d ? sh[threadIdx.x - d] : 0u;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    const unsigned long long base = sh_base;
    if (i < nb) tile_count[i] = (uint32_t)(base + sh[threadIdx.x] - v);
    __syncthreads();
    if (threadIdx.x == 1023) sh_base = base + sh[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) counters[1] = sh_base;
}

// Pass 2: the same tiles in entry order; each kept entry gets its place from
// the tile base and the block-wide count, and gathers its feature (float ->
// double), camera ordinal, intrinsic group and track (binary search of the
// offsets: the last track that starts at or before the entry).
__global__ void __launch_bounds__(kPackThreads) k_pack_gather(
    int64_t ne, int64_t ni, int64_t nt, int64_t nf, const int64_t* __restrict__ offs,
    const uint32_t* __restrict__ img, const uint32_t* __restrict__ feat, const uint32_t* __restrict__ ordinal,
    const uint32_t* __restrict__ group, const int64_t* __restrict__ feature_offsets,
    const float* __restrict__ features, const uint32_t* __restrict__ tile_base, double* __restrict__ obs,
    uint32_t* __restrict__ camera_index, uint32_t* __restrict__ intrinsic_index, uint32_t* __restrict__ point_index,
    unsigned long long* __restrict__ counters) {
  __shared__ uint32_t sh_warp[32];
  unsigned long long err = 0;
  uint32_t running = tile_base[blockIdx.x];
  const int64_t tile = blockIdx.x * kPackTile;
  for (int j = 0; j < kPackPer; ++j) {
    const int64_t e = tile + j * kPackThreads + threadIdx.x;
    uint32_t im = 0, total;
    const bool flag = entry_kept(e, ne, ni, img, ordinal, &im);
    const uint32_t pos = running + block_exclusive_count(flag, sh_warp, &total);
    if (flag) {
      const uint32_t f = feat[e];
      const int64_t a = feature_offsets[im], b = feature_offsets[im + 1];
      const bool ok = a >= 0 && b <= nf && (int64_t)f < b - a;
      float x = 0.0f, y = 0.0f;
      if (ok) {
        x = features[2 * (a + f)];
        y = features[2 * (a + f) + 1];
      } else {
        err |= kBadFeature;
      }
      int64_t lo = 0, hi = nt;  // offs[lo] <= e < offs[hi] on a valid CSR
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (offs[mid] <= e) lo = mid; else hi = mid;
      }
      obs[2 * (int64_t)pos] = (double)x;
      obs[2 * (int64_t)pos + 1] = (double)y;
      camera_index[pos] = ordinal[im];
      intrinsic_index[pos] = group[im];
      point_index[pos] = (uint32_t)lo;
    }
    running += total;
  }
  if (err) atomicOr(&counters[2], err);
}

// The locked block: the reference's mutable_camera_extrinsic_for_observation
// (ordinal of the first-added image) is the block of observation number
// `ordinal`; std::map::operator[] gives ordinal 0 to an image without a camera.
__global__ void k_pack_lock(int32_t lock, int64_t first, const uint32_t* __restrict__ ordinal,
                            const uint32_t* __restrict__ camera_index, uint8_t* __restrict__ camera_constant,
                            unsigned long long* __restrict__ counters) {
  const unsigned long long nc = counters[0], nobs = counters[1];
  long long locked = -1;
  if (lock != GBSFM_LOCK_NONE && first >= 0 && nc > 0) {
    const uint32_t o = ordinal[first];
    if (lock == GBSFM_LOCK_FIRST_ADDED) {
      locked = o == kNoCamera ? -1 : (long long)o;
    } else {
      const unsigned long long k = o == kNoCamera ? 0ull : o;
      if (k < nobs) locked = camera_index[k];
      else atomicOr(&counters[2], kLockPastEnd);
    }
  }
  if (locked >= 0 && camera_constant) camera_constant[locked] = 1;
  counters[3] = (unsigned long long)(locked + 1);
}

// Write-back checks: every ordinal's image inside the state, every such
// image's group inside the groups.
__global__ void __launch_bounds__(128) k_unpack_check(int64_t nc, const uint32_t* __restrict__ camera_image,
                                                      int64_t ni, const uint32_t* __restrict__ group, int64_t ng,
                                                      unsigned long long* __restrict__ err) {
  unsigned long long e = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t im = camera_image[c];
    if (im >= (uint64_t)ni) e |= kBadCameraImage;
    else if (group[im] >= (uint64_t)ng) e |= kBadGroup;
  }
  if (e) atomicOr(err, e);
}

// Write-back: camera_image[c] becomes the BrownPinholeCamera of the refined
// block c and its group's intrinsics.  Runs only after k_unpack_check found
// nothing, so nothing is written for a bad call.
__global__ void __launch_bounds__(128) k_unpack(int64_t nc, const double* __restrict__ ext,
                                                const uint32_t* __restrict__ camera_image,
                                                const double* __restrict__ intr, const uint32_t* __restrict__ group,
                                                const unsigned long long* __restrict__ err,
                                                gbsfm_camera* __restrict__ cams) {
  if (*err) return;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t im = camera_image[c];
    const double* e = ext + 6 * c;
    const double* k = intr + 6 * (int64_t)group[im];
    gbsfm_camera out;
    const double aa[3] = {e[0], e[1], e[2]};
    angle_axis_to_rotation(aa, out.R);
    out.t[0] = e[3];
    out.t[1] = e[4];
    out.t[2] = e[5];
    out.f = k[0];
    out.ppx = k[1];
    out.ppy = k[2];
    out.k1 = k[3];
    out.k2 = k[4];
    out.k3 = k[5];
    cams[im] = out;
  }
}

const char* pack_error(unsigned long long bits) {
  if (bits & kBadOffsets) return "track_offsets is not a CSR of num_entries entries";
  if (bits & kBadImage) return "a track entry names an image outside the state";
  if (bits & kBadFeature) return "a track entry names a feature outside its image";
  if (bits & kBadGroup) return "an intrinsic group out of range";
  if (bits & kLockPastEnd) return "the first-added camera's ordinal is past the observations";
  return "a camera ordinal names an image outside the state";
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

gbba_status gbsfm_pack_ba(gbba_handle* h, const gbsfm_engine_state* st, int64_t first_added_image, int32_t lock,
                          gbsfm_ba_arrays* out, int32_t memory) {
  if (!st || !out || lock < GBSFM_LOCK_AS_REFERENCE || lock > GBSFM_LOCK_NONE) return GBBA_ERROR_INVALID_ARGUMENT;
  const int64_t ni = st->num_images, ng = st->num_intrinsic_groups, nf = st->num_features, nt = st->num_points,
                ne = st->num_entries;
  if (ni < 0 || ng < 0 || nf < 0 || nt < 0 || ne < 0 || first_added_image >= ni || first_added_image < -1)
    return GBBA_ERROR_INVALID_ARGUMENT;
  if ((ni > 0 && (!st->cameras || !st->reconstructed || !st->intrinsic_group || !out->extrinsics)) ||
      !st->feature_offsets || (nf > 0 && !st->features) || !st->track_offsets ||
      (ne > 0 && (!st->track_image || !st->track_feature || !out->observations || !out->camera_index ||
                  !out->intrinsic_index || !out->point_index)) ||
      (ng > 0 && (!st->group_intrinsics || !out->intrinsics)) || (nt > 0 && (!st->points || !out->points)))
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (ni > 0xfffffffeLL || ne > 0xffffffffLL || nt > 0xffffffffLL) return GBBA_ERROR_TOO_LARGE;
  return sfm_guard(h, [&]() {
    out->num_cameras = out->num_observations = 0;
    out->measurements = ne;
    out->locked_camera = -1;
    const int64_t nb = std::max<int64_t>(1, ceil_div(ne, kPackTile));
    h->arena.reset();
    h->arena.reserve(sizeof(gbsfm_camera) * ni + 16 * ni + sizeof(int64_t) * (ni + nt + 2) + sizeof(float) * 2 * nf +
                     sizeof(uint32_t) * 2 * ne + sizeof(double) * 6 * ni + sizeof(double) * 2 * ne +
                     sizeof(uint32_t) * 3 * ne + 4 * nb + 256 * 24);
    const gbsfm_camera* dcam = in_view(h, st->cameras, ni, memory);
    const uint8_t* drec = in_view(h, st->reconstructed, ni, memory);
    const uint32_t* dgrp = in_view(h, st->intrinsic_group, ni, memory);
    const int64_t* dfo = in_view(h, st->feature_offsets, ni + 1, memory);
    const float* dft = in_view(h, st->features, 2 * nf, memory);
    const int64_t* doff = in_view(h, st->track_offsets, nt + 1, memory);
    const uint32_t* dimg = in_view(h, st->track_image, ne, memory);
    const uint32_t* dfeat = in_view(h, st->track_feature, ne, memory);
    double* dext = out_view(h, out->extrinsics, 6 * ni, memory);
    double* dobs = out_view(h, out->observations, 2 * ne, memory);
    uint32_t* dci = out_view(h, out->camera_index, ne, memory);
    uint32_t* dii = out_view(h, out->intrinsic_index, ne, memory);
    uint32_t* dpi = out_view(h, out->point_index, ne, memory);
    uint8_t* dcc = out_view(h, out->camera_constant, ni, memory);
    uint32_t* dcimg = out_view(h, out->camera_image, ni, memory);
    uint32_t* ordinal = h->arena.take<uint32_t>(std::max<int64_t>(1, ni));
    uint32_t* tiles = h->arena.take<uint32_t>(nb);
    unsigned long long* counters = h->arena.take<unsigned long long>(4);
    // intrinsic groups and points enter the problem as they are
    if (ng > 0 && out->intrinsics != st->group_intrinsics)
      GBBA_CUDA(cudaMemcpyAsync(out->intrinsics, st->group_intrinsics, sizeof(double) * 6 * ng, cudaMemcpyDefault,
                                h->active));
    if (nt > 0 && out->points != st->points)
      GBBA_CUDA(cudaMemcpyAsync(out->points, st->points, sizeof(double) * 3 * nt, cudaMemcpyDefault, h->active));
    GBBA_CUDA(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), h->active));
    if (dcc && ni > 0) GBBA_CUDA(cudaMemsetAsync(dcc, 0, ni, h->active));
    KernelTimer timer(h);
    if (ni > 0) {
      k_pack_images<<<1, 1024, 0, h->active>>>(ni, drec, dcam, dgrp, ng, ordinal, dext, dcimg, counters);
      check_launch(h);
    }
    k_pack_count<<<(unsigned)nb, kPackThreads, 0, h->active>>>(ne, ni, nt, doff, dimg, ordinal, tiles, counters);
    check_launch(h);
    k_pack_scan<<<1, 1024, 0, h->active>>>(tiles, nb, counters);
    check_launch(h);
    if (ne > 0) {
      k_pack_gather<<<(unsigned)nb, kPackThreads, 0, h->active>>>(ne, ni, nt, nf, doff, dimg, dfeat, ordinal, dgrp,
                                                                  dfo, dft, tiles, dobs, dci, dii, dpi, counters);
      check_launch(h);
    }
    if (ni > 0) {
      k_pack_lock<<<1, 1, 0, h->active>>>(lock, first_added_image, ordinal, dci, dcc, counters);
      check_launch(h);
    }
    timer.stop();
    unsigned long long* hc = reinterpret_cast<unsigned long long*>(h->pinned + 176);
    GBBA_CUDA(cudaMemcpyAsync(hc, counters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    const unsigned long long nc = hc[0], nobs = hc[1], err = hc[2], locked = hc[3];
    GBBA_REQUIRE(err == 0, GBBA_ERROR_INVALID_ARGUMENT, pack_error(err));
    out_back(h, out->extrinsics, dext, 6 * nc, memory);
    out_back(h, out->observations, dobs, 2 * nobs, memory);
    out_back(h, out->camera_index, dci, nobs, memory);
    out_back(h, out->intrinsic_index, dii, nobs, memory);
    out_back(h, out->point_index, dpi, nobs, memory);
    out_back(h, out->camera_constant, dcc, nc, memory);
    out_back(h, out->camera_image, dcimg, nc, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    out->num_cameras = (int64_t)nc;
    out->num_observations = (int64_t)nobs;
    out->locked_camera = (int64_t)locked - 1;
    return GBBA_SUCCESS;
  });
}

gbba_status gbsfm_unpack_ba(gbba_handle* h, int64_t num_cameras, const double* extrinsics,
                            const uint32_t* camera_image, const double* intrinsics, int64_t num_intrinsic_groups,
                            const uint32_t* intrinsic_group, int64_t num_images, gbsfm_camera* cameras,
                            int32_t memory) {
  if (num_cameras < 0 || num_images < 0 || num_intrinsic_groups < 0 || num_cameras > num_images)
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (num_cameras > 0 && (!extrinsics || !camera_image || !intrinsics || !intrinsic_group || !cameras))
    return GBBA_ERROR_INVALID_ARGUMENT;
  return sfm_guard(h, [&]() {
    if (num_cameras == 0) return GBBA_SUCCESS;
    h->arena.reset();
    h->arena.reserve(sizeof(double) * 6 * (num_cameras + num_intrinsic_groups) +
                     sizeof(uint32_t) * (num_cameras + num_images) + sizeof(gbsfm_camera) * num_images + 256 * 8);
    const double* dext = in_view(h, extrinsics, 6 * num_cameras, memory);
    const uint32_t* dcimg = in_view(h, camera_image, num_cameras, memory);
    const double* dintr = in_view(h, intrinsics, 6 * num_intrinsic_groups, memory);
    const uint32_t* dgrp = in_view(h, intrinsic_group, num_images, memory);
    gbsfm_camera* dcam = const_cast<gbsfm_camera*>(in_view(h, (const gbsfm_camera*)cameras, num_images, memory));
    unsigned long long* err = h->arena.take<unsigned long long>(1);
    GBBA_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned long long), h->active));
    const unsigned grid = grid_for(h, num_cameras, 128);
    KernelTimer timer(h);
    k_unpack_check<<<grid, 128, 0, h->active>>>(num_cameras, dcimg, num_images, dgrp, num_intrinsic_groups, err);
    check_launch(h);
    k_unpack<<<grid, 128, 0, h->active>>>(num_cameras, dext, dcimg, dintr, dgrp, err, dcam);
    check_launch(h);
    timer.stop();
    unsigned long long* he = reinterpret_cast<unsigned long long*>(h->pinned + 176);
    GBBA_CUDA(cudaMemcpyAsync(he, err, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->active));
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    GBBA_REQUIRE(*he == 0, GBBA_ERROR_INVALID_ARGUMENT, pack_error(*he));
    out_back(h, cameras, (const gbsfm_camera*)dcam, num_images, memory);
    GBBA_CUDA(cudaStreamSynchronize(h->active));
    return GBBA_SUCCESS;
  });
}

}  // extern "C"
