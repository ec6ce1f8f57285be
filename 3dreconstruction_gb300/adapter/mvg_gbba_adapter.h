// C++ adapter between the reference's libs/sfm / libs/multiview types and the
// GB300 engine's C ABI (include/gbba.h, include/gbtri.h).
//
// Header-only; include it from libs/sfm or libs/multiview (after the
// reference's own headers) and link 3dreconstruction_gb300/libgbba.so.
//
//   mvg::sfm::gpu::SolveBundleAdjustment     replaces the ceres::Problem +
//       ceres::Solve blocks of libs/sfm/src/sfm_incremental_engine.cpp:
//       1395-1473 and libs/sfm/src/sfm_global_engine.cpp:1142-1174,
//       1546-1594, 1756-1802; the containers are
//       libs/sfm/include/mvg/sfm/problem_data_container.h:16-121.
//   mvg::multiview::gpu::TriangulateDLT / TriangulateNView  keep the exact
//       signatures of libs/multiview/include/mvg/multiview/triangulation.h:
//       12-20 and triangulation_nview.h:12-15 and route to the batched entry.
#ifndef MVG_GBBA_ADAPTER_H_
#define MVG_GBBA_ADAPTER_H_

#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/gbba.h"
#include "../../include/gbtri.h"

namespace mvg {
namespace gbba_detail {
// One handle per host thread (the C ABI's handles are not thread safe).
inline gbba_handle* ThreadHandle() {
  static thread_local gbba_handle* h = nullptr;
  if (!h && gbba_create(0, &h) != GBBA_SUCCESS) h = nullptr;
  return h;
}
inline std::vector<uint32_t> Narrow(const std::vector<size_t>& v) { return std::vector<uint32_t>(v.begin(), v.end()); }
// The reference's triangulation functions return nothing; when the GPU call
// fails the adapter leaves the caller's output untouched and says why here.
inline bool Report(gbba_status st, const char* what) {
  if (st == GBBA_SUCCESS) return true;
  std::fprintf(stderr, "mvg gpu %s: %s (output left unchanged)\n", what, gbba_status_string(st));
  return false;
}
}  // namespace gbba_detail

namespace sfm {
namespace gpu {

// The solver options the reference call sites set, with ceres's defaults.
struct BundleAdjustmentOptions {
  int loss = GBBA_LOSS_SQUARED;
  double loss_scale = 1.0;            // ceres::HuberLoss(a): a is the residual-norm threshold
  uint32_t intrinsic_fixed_mask = 0;  // SubsetParameterization of the intrinsic block
  uint32_t extrinsic_fixed_mask = 0;  // held extrinsic coordinates (rotation for the t-only BA)
  int max_num_iterations = 50;
  int precision = GBBA_PRECISION_FP64;
};

// BA_Problem_data_camMotionAndIntrinsic<6,K>: [angle-axis,t] per camera, one
// intrinsic block per group.  camera_constant: one byte per camera (the
// reference holds the first-added camera, sfm_incremental_engine.cpp:1439-1445).
template <class Problem>
bool SolveBundleAdjustment(Problem& ba, int camera_model, const BundleAdjustmentOptions& opt,
                           const std::vector<uint8_t>& camera_constant, gbba_summary* summary,
                           const std::vector<uint8_t>* intrinsic_constant = nullptr) {
  gbba_handle* h = gbba_detail::ThreadHandle();
  if (!h) return false;
  const std::vector<uint32_t> cam = gbba_detail::Narrow(ba.camera_index_extrinsic);
  const std::vector<uint32_t> intr = gbba_detail::Narrow(ba.camera_index_intrinsic);
  const std::vector<uint32_t> pt = gbba_detail::Narrow(ba.point_index_);
  gbba_problem p = {};
  p.camera_model = camera_model;
  p.memory = GBBA_MEMORY_HOST;
  p.num_cameras = (int64_t)ba.num_cameras_;
  p.num_intrinsics = (int64_t)ba.num_intrinsic_;
  p.num_points = (int64_t)ba.num_points_;
  p.num_observations = (int64_t)ba.num_observations_;
  p.extrinsics = ba.mutable_cameras_extrinsic();
  p.intrinsics = ba.mutable_cameras_intrinsic();
  p.points = ba.mutable_points();
  p.observations = ba.observations();
  p.camera_index = cam.data();
  p.intrinsic_index = intr.data();
  p.point_index = pt.data();
  p.camera_constant = camera_constant.empty() ? nullptr : camera_constant.data();
  p.intrinsic_constant = intrinsic_constant ? intrinsic_constant->data() : nullptr;
  p.extrinsic_fixed_mask = opt.extrinsic_fixed_mask;
  p.intrinsic_fixed_mask = opt.intrinsic_fixed_mask;
  gbba_options o;
  gbba_default_options(&o);
  o.loss_type = opt.loss;
  o.loss_scale = opt.loss_scale;
  o.max_num_iterations = opt.max_num_iterations;
  o.precision = opt.precision;
  gbba_summary local;
  gbba_summary* s = summary ? summary : &local;
  return gbba_solve(h, &p, &o, s) == GBBA_SUCCESS && s->usable;
}

// BAProblemData<7>: one [angle-axis, t, f] block per camera (the reference's
// unit-test container, ErrorFuncRefineCamera3DPointsPinhole).  The 7-vectors
// are split into the ABI's extrinsic / intrinsic arrays and merged back.
template <class Problem>
bool SolveBundleAdjustmentRtf(Problem& ba, const BundleAdjustmentOptions& opt, gbba_summary* summary) {
  gbba_handle* h = gbba_detail::ThreadHandle();
  if (!h) return false;
  const size_t nc = ba.num_cameras_;
  std::vector<double> ext(6 * nc), f(nc);
  double* cams = ba.mutable_cameras();
  for (size_t c = 0; c < nc; ++c) {
    for (int j = 0; j < 6; ++j) ext[6 * c + j] = cams[7 * c + j];
    f[c] = cams[7 * c + 6];
  }
  const std::vector<uint32_t> cam = gbba_detail::Narrow(ba.camera_index_);
  const std::vector<uint32_t> pt = gbba_detail::Narrow(ba.point_index_);
  gbba_problem p = {};
  p.camera_model = GBBA_PINHOLE_F;
  p.memory = GBBA_MEMORY_HOST;
  p.num_cameras = (int64_t)nc;
  p.num_intrinsics = (int64_t)nc;
  p.num_points = (int64_t)ba.num_points_;
  p.num_observations = (int64_t)ba.num_observations_;
  p.extrinsics = ext.data();
  p.intrinsics = f.data();
  p.points = ba.mutable_points();
  p.observations = ba.observations();
  p.camera_index = cam.data();
  p.intrinsic_index = cam.data();
  p.point_index = pt.data();
  gbba_options o;
  gbba_default_options(&o);
  o.loss_type = opt.loss;
  o.loss_scale = opt.loss_scale;
  o.max_num_iterations = opt.max_num_iterations;
  o.precision = opt.precision;
  gbba_summary local;
  gbba_summary* s = summary ? summary : &local;
  const bool ok = gbba_solve(h, &p, &o, s) == GBBA_SUCCESS && s->usable;
  if (ok)
    for (size_t c = 0; c < nc; ++c) {
      for (int j = 0; j < 6; ++j) cams[7 * c + j] = ext[6 * c + j];
      cams[7 * c + 6] = f[c];
    }
  return ok;
}

}  // namespace gpu
}  // namespace sfm

namespace multiview {
namespace gpu {

// Same signature as mvg::multiview::TriangulateDLT (triangulation.h:12-20).
// Eigen matrices are column-major; the ABI takes row-major 3x4.
template <class Mat34, class Vec2, class Vec4>
void TriangulateDLT(const Mat34& P1, const Vec2& x1, const Mat34& P2, const Vec2& x2, Vec4* X_homogeneous) {
  double a[12], b[12], u[2] = {x1(0), x1(1)}, v[2] = {x2(0), x2(1)}, X[4];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) {
      a[4 * r + c] = P1(r, c);
      b[4 * r + c] = P2(r, c);
    }
  gbba_handle* h = mvg::gbba_detail::ThreadHandle();
  const gbba_status st = h ? gbtri_dlt2_batched(h, 1, a, b, 12, u, v, X, nullptr, GBBA_MEMORY_HOST) : GBBA_ERROR_NO_DEVICE;
  if (!mvg::gbba_detail::Report(st, "TriangulateDLT")) return;
  for (int i = 0; i < 4; ++i) (*X_homogeneous)(i) = X[i];
}

// Same signature as mvg::multiview::TriangulateNView (triangulation_nview.h:12-15).
template <class Mat2X, class Mat34, class Vec4>
void TriangulateNView(const Mat2X& x, const std::vector<Mat34>& Ps, Vec4* X) {
  const int64_t n = (int64_t)x.cols();
  std::vector<double> P(12 * n), xy(2 * n);
  std::vector<uint32_t> cam(n);
  for (int64_t i = 0; i < n; ++i) {
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) P[12 * i + 4 * r + c] = Ps[i](r, c);
    xy[2 * i] = x(0, i);
    xy[2 * i + 1] = x(1, i);
    cam[i] = (uint32_t)i;
  }
  const int64_t off[2] = {0, n};
  double out[4];
  gbba_handle* h = mvg::gbba_detail::ThreadHandle();
  const gbba_status st = h ? gbtri_nview_batched(h, GBTRI_NVIEW, P.data(), n, off, cam.data(), xy.data(), 1, out,
                                                 nullptr, GBBA_MEMORY_HOST)
                           : GBBA_ERROR_NO_DEVICE;
  if (!mvg::gbba_detail::Report(st, "TriangulateNView")) return;
  for (int i = 0; i < 4; ++i) (*X)(i) = out[i];
}

}  // namespace gpu
}  // namespace multiview
}  // namespace mvg

#endif  // MVG_GBBA_ADAPTER_H_
