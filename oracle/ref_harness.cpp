// Reference harness: drives the reference project's own code (its ceres
// functors, vendored ceres-solver 1.10 / CXSparse 2.3.0 / Eigen 3.2.2, and its
// libs/multiview triangulation) on problems read from a text file, and writes
// the results as text.  It is TEST INFRASTRUCTURE: it is compiled from the
// reference sources by oracle/Makefile into oracle/_ref/ (never committed) and
// is only run by tests/golden/make_golden.py to produce golden fixtures and to
// pin the CPU restatement in oracle/gbba_oracle.cpp.
//
// Modes
//   ref_harness tri-ring <nviews> <npoints> <out>   reference unit-test scene
//       (NRealisticCamerasRing, libs/multiview/src/nview_data_sets.cpp:23) and
//       the outputs of TriangulateDLT / TriangulateNView /
//       TriangulateNViewAlgebraic / Triangulation::compute on it.
//   ref_harness tri <in> <out>     same functions on caller-given tracks.
//   ref_harness ba <in> <out>      ceres::Solve with the reference functors and
//       the call-site options of libs/sfm/src/sfm_incremental_engine.cpp:1395-1473.
//   ref_harness eval <in> <out>    ceres::Problem::Evaluate (cost, residuals,
//       gradient, dense Jacobian) at the given parameters.
//   ref_harness two-view <in> <out>   triangulate2View_Vector's per-match DLT
//       and residual (libs/sfm/include/mvg/sfm/sfm_robust.h:152-195) and the
//       keep decision of its callers (sfm_incremental_engine.cpp:977-1029 with
//       residual thresholds, :492-533 without), on the reference's
//       BrownPinholeCamera / PinholeCamera functions.
//   ref_harness reject <in> <out>  badTrackRejector's decisions
//       (sfm_incremental_engine.cpp:1047-1140) per measurement and track.
//   ref_harness histogram <in> <out>  ComputeResidualsHistogram
//       (sfm_incremental_engine.cpp:1550-1616): float residuals, MinMaxMeanMedian
//       and Histogram<double>(min, max, 10).
//   ref_harness pack <in> <out>    BundleAdjustment's assembly of its std::map
//       state into the BA problem and its write-back of refined parameters
//       (sfm_incremental_engine.cpp:1250-1393, 1475-1546) with ceres's
//       RotationMatrixToAngleAxis / AngleAxisToRotationMatrix.
//   ref_harness acransac <in> <out>  robustResection's ACRANSAC with the
//       reference's resection kernels (six-point DLT, or P3P with K), every
//       model it draws recorded and scored by the reference's bestNFA.
// The pair, reject, histogram and pack modes restate the engines' loops (whose classes need the whole
// engine) around the reference's own camera, triangulation and histogram code.
//
// File format ("kv text"): a sequence of records `name count` followed by
// `count` whitespace-separated numbers (%.17g).

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "ceres/ceres.h"
#include "ceres/rotation.h"
#include "mvg/camera/brown_pinhole_camera.h"
#include "mvg/camera/pinhole_camera.h"
#include "mvg/camera/projection.h"
#include "mvg/utils/histogram.h"
#include "mvg/multiview/nview_data_sets.h"
#include "mvg/multiview/triangulation.h"
#include "mvg/multiview/triangulation_nview.h"
using namespace mvg::camera;  // pinhole_brown_rt_ceres_functor.h expects it
#include "mvg/sfm/pinhole_brown_rt_ceres_functor.h"
#include "mvg/sfm/pinhole_ceres_functor.h"
#include "mvg/sfm/sfm_bundle_adjustment_helper_tonly.h"
// sfm_robust.h logs through MVG_INFO without including its definition; the
// harness discards that log.
#ifndef MVG_INFO
#define MVG_INFO if (false) std::cerr
#endif
#include "mvg/sfm/sfm_robust.h"

using namespace mvg::multiview;
using namespace mvg::sfm;

typedef std::map<std::string, std::vector<double> > KV;

static KV ReadKV(const char* path) {
  KV kv;
  std::ifstream in(path);
  if (!in) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  std::string name;
  long long n;
  while (in >> name >> n) {
    std::vector<double>& v = kv[name];
    v.resize((size_t)n);
    for (long long i = 0; i < n; ++i) in >> v[(size_t)i];
  }
  return kv;
}

struct KVWriter {
  FILE* f;
  explicit KVWriter(const char* path) { f = fopen(path, "w"); if (!f) exit(2); }
  ~KVWriter() { fclose(f); }
  void put(const char* name, const double* v, size_t n) {
    fprintf(f, "%s %zu\n", name, n);
    for (size_t i = 0; i < n; ++i) fprintf(f, "%.17g%c", v[i], (i + 1) % 8 == 0 ? '\n' : ' ');
    fprintf(f, "\n");
  }
  void put(const char* name, const std::vector<double>& v) { put(name, v.data(), v.size()); }
  void put1(const char* name, double x) { put(name, &x, 1); }
};

static double Get1(const KV& kv, const char* name, double dflt) {
  KV::const_iterator it = kv.find(name);
  return (it == kv.end() || it->second.empty()) ? dflt : it->second[0];
}
static const std::vector<double>& Get(const KV& kv, const char* name) {
  KV::const_iterator it = kv.find(name);
  if (it == kv.end()) { fprintf(stderr, "missing %s\n", name); exit(2); }
  return it->second;
}

// Brown radial-K3 + tangential-T2 functor.  The reference has the tangential
// terms only as a commented-out formula (libs/camera/include/mvg/camera/
// brown_pinhole_camera.h:35-36, OFFSET_P1/P2 at pinhole_brown_rt_ceres_functor.h:
// 25-26); this harness functor enables them exactly as written there.
struct HarnessBrownT2 {
  explicit HarnessBrownT2(const double* xy) { m[0] = xy[0]; m[1] = xy[1]; }
  template <typename T>
  bool operator()(const T* const K, const T* const Rt, const T* const X, T* r) const {
    T p[3];
    ceres::AngleAxisRotatePoint(Rt, X, p);
    p[0] += Rt[3]; p[1] += Rt[4]; p[2] += Rt[5];
    T x = p[0] / p[2], y = p[1] / p[2];
    T r2 = x * x + y * y, r4 = r2 * r2, r6 = r4 * r2;
    T rc = T(1) + K[3] * r2 + K[4] * r4 + K[5] * r6;
    T xd = x * rc + T(2) * K[6] * x * y + K[7] * (r2 + T(2) * x * x);
    T yd = y * rc + T(2) * K[7] * x * y + K[6] * (r2 + T(2) * y * y);
    r[0] = K[1] + K[0] * xd - T(m[0]);
    r[1] = K[2] + K[0] * yd - T(m[1]);
    return true;
  }
  double m[2];
};

enum { MODEL_PINHOLE_F = 0, MODEL_RADIAL_K3 = 1, MODEL_BROWN_T2 = 2 };
enum { LAYOUT_SPLIT = 0, LAYOUT_RTF7 = 1, LAYOUT_T_ONLY = 2, LAYOUT_RT_ONLY = 3 };
static int ModelK(int model) { return model == MODEL_PINHOLE_F ? 1 : model == MODEL_RADIAL_K3 ? 6 : 8; }

struct BAInput {
  int model, layout, loss;
  double loss_scale;
  size_t nc, ni, np, no;
  std::vector<double> ext, intr, pts, obs;
  std::vector<size_t> cam, in, pt;
  std::vector<int> cam_const, intr_const;
  int intr_fixed_mask, ext_fixed_mask;
  std::vector<double> rtf;  // LAYOUT_RTF7 parameter storage [R t f] per camera
};

static BAInput LoadBA(const KV& kv) {
  BAInput b;
  b.model = (int)Get1(kv, "model", 1);
  b.layout = (int)Get1(kv, "layout", 0);
  b.loss = (int)Get1(kv, "loss", 0);
  b.loss_scale = Get1(kv, "loss_scale", 1.0);
  b.ext = Get(kv, "extrinsics");
  b.intr = Get(kv, "intrinsics");
  b.pts = Get(kv, "points");
  b.obs = Get(kv, "observations");
  const int k = ModelK(b.model);
  b.nc = b.ext.size() / 6; b.ni = b.intr.size() / k; b.np = b.pts.size() / 3; b.no = b.obs.size() / 2;
  const std::vector<double>& c = Get(kv, "camera_index");
  const std::vector<double>& i = Get(kv, "intrinsic_index");
  const std::vector<double>& p = Get(kv, "point_index");
  for (size_t o = 0; o < b.no; ++o) { b.cam.push_back((size_t)c[o]); b.in.push_back((size_t)i[o]); b.pt.push_back((size_t)p[o]); }
  b.cam_const.assign(b.nc, 0); b.intr_const.assign(b.ni, 0);
  if (kv.count("camera_constant")) { const std::vector<double>& v = Get(kv, "camera_constant"); for (size_t j = 0; j < b.nc; ++j) b.cam_const[j] = (int)v[j]; }
  if (kv.count("intrinsic_constant")) { const std::vector<double>& v = Get(kv, "intrinsic_constant"); for (size_t j = 0; j < b.ni; ++j) b.intr_const[j] = (int)v[j]; }
  b.intr_fixed_mask = (int)Get1(kv, "intrinsic_fixed_mask", 0);
  b.ext_fixed_mask = (int)Get1(kv, "extrinsic_fixed_mask", 0);
  return b;
}

// Builds the ceres problem exactly as the reference call sites do: one
// AutoDiffCostFunction per observation with the reference functor for the
// chosen layout, the same loss object for all, constant blocks and a
// SubsetParameterization for held intrinsic coordinates.
static void BuildProblem(BAInput& b, ceres::Problem* problem, bool with_constants) {
  const int k = ModelK(b.model);
  ceres::LossFunction* loss = NULL;
  if (b.loss == 1) loss = new ceres::HuberLoss(b.loss_scale);
  ceres::SubsetParameterization* subset = NULL;
  std::vector<int> fixed;
  for (int j = 0; j < k; ++j) if (b.intr_fixed_mask & (1 << j)) fixed.push_back(j);
  if (with_constants && !fixed.empty() && (int)fixed.size() < k) subset = new ceres::SubsetParameterization(k, fixed);
  if (b.layout == LAYOUT_RTF7) {
    b.rtf.resize(7 * b.nc);
    for (size_t c = 0; c < b.nc; ++c) {
      for (int j = 0; j < 6; ++j) b.rtf[7 * c + j] = b.ext[6 * c + j];
      b.rtf[7 * c + 6] = b.intr[c];
    }
  }
  for (size_t o = 0; o < b.no; ++o) {
    const double* xy = &b.obs[2 * o];
    double* E = &b.ext[6 * b.cam[o]];
    double* I = &b.intr[k * b.in[o]];
    double* X = &b.pts[3 * b.pt[o]];
    if (b.layout == LAYOUT_RTF7) {
      problem->AddResidualBlock(new ceres::AutoDiffCostFunction<ErrorFuncRefineCamera3DPointsPinhole, 2, 7, 3>(
          new ErrorFuncRefineCamera3DPointsPinhole(xy)), loss, &b.rtf[7 * b.cam[o]], X);
    } else if (b.layout == LAYOUT_T_ONLY) {
      problem->AddResidualBlock(new ceres::AutoDiffCostFunction<PinholeReprojectionError_t, 2, 3, 3>(
          new PinholeReprojectionError_t(xy, I[0], E)), loss, E + 3, X);
    } else if (b.layout == LAYOUT_RT_ONLY) {
      problem->AddResidualBlock(new ceres::AutoDiffCostFunction<PinholeReprojectionError_Rt, 2, 6, 3>(
          new PinholeReprojectionError_Rt(xy, I[0])), loss, E, X);
    } else if (b.model == MODEL_PINHOLE_F) {
      problem->AddResidualBlock(new ceres::AutoDiffCostFunction<ErrorFuncRefineCamera3DPointsFocal, 2, 1, 6, 3>(
          new ErrorFuncRefineCamera3DPointsFocal(xy)), loss, I, E, X);
    } else if (b.model == MODEL_RADIAL_K3) {
      problem->AddResidualBlock(new ceres::AutoDiffCostFunction<ErrorFunc_Refine_Camera_3DPoints, 2, 6, 6, 3>(
          new ErrorFunc_Refine_Camera_3DPoints(xy)), loss, I, E, X);
      if (subset) problem->SetParameterization(I, subset);
    } else {
      problem->AddResidualBlock(new ceres::AutoDiffCostFunction<HarnessBrownT2, 2, 8, 6, 3>(
          new HarnessBrownT2(xy)), loss, I, E, X);
      if (subset) problem->SetParameterization(I, subset);
    }
  }
  if (!with_constants) return;
  for (size_t c = 0; c < b.nc; ++c) {
    if (!b.cam_const[c]) continue;
    if (b.layout == LAYOUT_RTF7) problem->SetParameterBlockConstant(&b.rtf[7 * c]);
    else if (b.layout == LAYOUT_T_ONLY) problem->SetParameterBlockConstant(&b.ext[6 * c + 3]);
    else problem->SetParameterBlockConstant(&b.ext[6 * c]);
  }
  if (b.layout == LAYOUT_SPLIT) {
    for (size_t i = 0; i < b.ni; ++i) {
      bool all_fixed = ((int)fixed.size() == k);
      if (b.intr_const[i] || all_fixed) problem->SetParameterBlockConstant(&b.intr[k * i]);
    }
  }
}

static int RunBA(const KV& kv, const char* out) {
  BAInput b = LoadBA(kv);
  ceres::Problem problem;
  BuildProblem(b, &problem, true);
  ceres::Solver::Options options;
  const int solver = (int)Get1(kv, "linear_solver", 0);
  // preconditioner: 0 = JACOBI (ceres's default), 1 = SCHUR_JACOBI (the block
  // diagonal of the reduced camera system, which the GPU PCG implements)
  options.preconditioner_type = (int)Get1(kv, "preconditioner", 0) == 1 ? ceres::SCHUR_JACOBI : ceres::JACOBI;
  options.max_linear_solver_iterations = (int)Get1(kv, "max_linear_solver_iterations", 500);
  options.eta = Get1(kv, "eta", 1e-1);
  if (solver == 0) {
    options.linear_solver_type = ceres::SPARSE_SCHUR;
    options.sparse_linear_algebra_library_type = ceres::CX_SPARSE;
  } else if (solver == 1) {
    options.linear_solver_type = ceres::DENSE_SCHUR;
  } else {
    options.linear_solver_type = ceres::ITERATIVE_SCHUR;
  }
  options.max_num_iterations = (int)Get1(kv, "max_num_iterations", 50);
  options.function_tolerance = Get1(kv, "function_tolerance", 1e-6);
  options.gradient_tolerance = Get1(kv, "gradient_tolerance", 1e-10);
  options.parameter_tolerance = Get1(kv, "parameter_tolerance", 1e-8);
  options.num_threads = (int)Get1(kv, "num_threads", 1);
  options.num_linear_solver_threads = options.num_threads;
  options.minimizer_progress_to_stdout = false;
  options.logging_type = ceres::SILENT;
  ceres::Solver::Summary summary;
  ceres::Solve(options, &problem, &summary);
  if (b.layout == LAYOUT_RTF7) {
    for (size_t c = 0; c < b.nc; ++c) {
      for (int j = 0; j < 6; ++j) b.ext[6 * c + j] = b.rtf[7 * c + j];
      b.intr[c] = b.rtf[7 * c + 6];
    }
  }
  KVWriter w(out);
  w.put1("initial_cost", summary.initial_cost);
  w.put1("final_cost", summary.final_cost);
  w.put1("num_successful_steps", summary.num_successful_steps);
  w.put1("num_unsuccessful_steps", summary.num_unsuccessful_steps);
  w.put1("termination_type", (double)summary.termination_type);
  w.put1("usable", summary.IsSolutionUsable() ? 1 : 0);
  w.put1("total_time_s", summary.total_time_in_seconds);
  {
    std::vector<double> lin;
    for (size_t i = 0; i < summary.iterations.size(); ++i) lin.push_back(summary.iterations[i].linear_solver_iterations);
    w.put("iteration_linear_solver_iterations", lin);
  }
  w.put1("minimizer_time_s", summary.minimizer_time_in_seconds);
  std::vector<double> costs, radii, succ;
  for (size_t i = 0; i < summary.iterations.size(); ++i) {
    costs.push_back(summary.iterations[i].cost);
    radii.push_back(summary.iterations[i].trust_region_radius);
    succ.push_back(summary.iterations[i].step_is_successful ? 1 : 0);
  }
  w.put("iteration_cost", costs);
  w.put("iteration_radius", radii);
  w.put("iteration_success", succ);
  w.put("extrinsics", b.ext);
  w.put("intrinsics", b.intr);
  w.put("points", b.pts);
  return summary.IsSolutionUsable() ? 0 : 1;
}

static int RunEval(const KV& kv, const char* out) {
  BAInput b = LoadBA(kv);
  ceres::Problem problem;
  BuildProblem(b, &problem, false);
  const int k = ModelK(b.model);
  ceres::Problem::EvaluateOptions eo;
  for (size_t c = 0; c < b.nc; ++c) eo.parameter_blocks.push_back(&b.ext[6 * c]);
  for (size_t i = 0; i < b.ni; ++i) eo.parameter_blocks.push_back(&b.intr[k * i]);
  for (size_t p = 0; p < b.np; ++p) eo.parameter_blocks.push_back(&b.pts[3 * p]);
  double cost = 0;
  std::vector<double> res, grad;
  ceres::CRSMatrix J;
  problem.Evaluate(eo, &cost, &res, &grad, &J);
  std::vector<double> dense((size_t)J.num_rows * J.num_cols, 0.0);
  for (int r = 0; r < J.num_rows; ++r)
    for (int q = J.rows[r]; q < J.rows[r + 1]; ++q) dense[(size_t)r * J.num_cols + J.cols[q]] = J.values[q];
  KVWriter w(out);
  w.put1("cost", cost);
  w.put("residuals", res);
  w.put("gradient", grad);
  w.put1("jac_rows", J.num_rows);
  w.put1("jac_cols", J.num_cols);
  w.put("jacobian", dense);
  return 0;
}

// Triangulation on caller-given tracks: P (row-major 3x4 per camera), CSR
// track offsets, per-observation camera index and pixel coordinates.
static void Triangulate(const std::vector<Mat34>& Ps, const std::vector<double>& offs,
                        const std::vector<double>& cam, const std::vector<double>& xy, KVWriter& w) {
  const size_t nt = offs.size() - 1;
  std::vector<double> dlt4, dlt3, nv4, alg4, it3, iterr;
  for (size_t t = 0; t < nt; ++t) {
    const size_t b = (size_t)offs[t], e = (size_t)offs[t + 1], n = e - b;
    Mat2X x(2, n);
    std::vector<Mat34> P;
    for (size_t j = 0; j < n; ++j) { x(0, j) = xy[2 * (b + j)]; x(1, j) = xy[2 * (b + j) + 1]; P.push_back(Ps[(size_t)cam[b + j]]); }
    Vec4 X4; Vec3 X3;
    TriangulateDLT(P[0], x.col(0), P[1], x.col(1), &X4);
    TriangulateDLT(P[0], x.col(0), P[1], x.col(1), &X3);
    for (int i = 0; i < 4; ++i) dlt4.push_back(X4(i));
    for (int i = 0; i < 3; ++i) dlt3.push_back(X3(i));
    TriangulateNView(x, P, &X4);
    for (int i = 0; i < 4; ++i) nv4.push_back(X4(i));
    TriangulateNViewAlgebraic(x, P, &X4);
    for (int i = 0; i < 4; ++i) alg4.push_back(X4(i));
    Triangulation tri;
    for (size_t j = 0; j < n; ++j) tri.add(P[j], x.col(j));
    X3 = tri.compute();
    for (int i = 0; i < 3; ++i) it3.push_back(X3(i));
    iterr.push_back(tri.error(X3));
  }
  w.put("dlt_h", dlt4);
  w.put("dlt_e", dlt3);
  w.put("nview_h", nv4);
  w.put("algebraic_h", alg4);
  w.put("iterative_e", it3);
  w.put("iterative_error", iterr);
}

static int RunTriRing(int nviews, int npoints, const char* out) {
  NViewDataSet d = NRealisticCamerasRing(nviews, npoints);
  std::vector<Mat34> Ps;
  std::vector<double> P, offs, cam, xy, Xgt;
  for (int j = 0; j < nviews; ++j) {
    Ps.push_back(d.P(j));
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 4; ++c) P.push_back(Ps.back()(r, c));
  }
  offs.push_back(0);
  for (int i = 0; i < npoints; ++i) {
    for (int j = 0; j < nviews; ++j) {
      cam.push_back(j);
      xy.push_back(d.projected_points_[j](0, i));
      xy.push_back(d.projected_points_[j](1, i));
    }
    offs.push_back(offs.back() + nviews);
    for (int r = 0; r < 3; ++r) Xgt.push_back(d.point_3d_(r, i));
  }
  KVWriter w(out);
  w.put("P", P);
  w.put("track_offsets", offs);
  w.put("camera_index", cam);
  w.put("xy", xy);
  w.put("X_gt", Xgt);
  std::vector<double> K, R, t;
  for (int j = 0; j < nviews; ++j) {
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) { K.push_back(d.camera_matrix_[j](r, c)); R.push_back(d.rotation_matrix_[j](r, c)); }
    for (int r = 0; r < 3; ++r) t.push_back(d.translation_vector_[j](r));
  }
  w.put("K", K);
  w.put("R", R);
  w.put("t", t);
  Triangulate(Ps, offs, cam, xy, w);
  return 0;
}

static int RunTri(const KV& kv, const char* out) {
  const std::vector<double>& P = Get(kv, "P");
  std::vector<Mat34> Ps(P.size() / 12);
  for (size_t j = 0; j < Ps.size(); ++j)
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 4; ++c) Ps[j](r, c) = P[12 * j + 4 * r + c];
  KVWriter w(out);
  Triangulate(Ps, Get(kv, "track_offsets"), Get(kv, "camera_index"), Get(kv, "xy"), w);
  return 0;
}

// Cameras as [R (row-major 9), t (3), f, ppx, ppy, k1, k2, k3] per camera.
static std::vector<BrownPinholeCamera> LoadCameras(const std::vector<double>& v) {
  std::vector<BrownPinholeCamera> cams;
  for (size_t c = 0; c + 18 <= v.size(); c += 18) {
    Mat3 R;
    for (int r = 0; r < 3; ++r) for (int k = 0; k < 3; ++k) R(r, k) = v[c + 3 * r + k];
    const Vec3 t(v[c + 9], v[c + 10], v[c + 11]);
    cams.push_back(BrownPinholeCamera(v[c + 12], v[c + 13], v[c + 14], R, t, v[c + 15], v[c + 16], v[c + 17]));
  }
  return cams;
}

static int RunTwoView(const KV& kv, const char* out) {
  const std::vector<BrownPinholeCamera> cams = LoadCameras(Get(kv, "cameras"));
  const BrownPinholeCamera& cam1 = cams[0];
  const BrownPinholeCamera& cam2 = cams[1];
  const std::vector<double>& x1 = Get(kv, "x1");
  const std::vector<double>& x2 = Get(kv, "x2");
  const std::vector<double>& inlier = Get(kv, "inlier");
  const double th1 = Get1(kv, "max_residual1", 1e300), th2 = Get1(kv, "max_residual2", 1e300);
  const double min_angle = Get1(kv, "min_angle", 2.0);
  const size_t n = x1.size() / 2;
  std::vector<double> X, res, keep;
  for (size_t i = 0; i < n; ++i) {
    const Vec2 a(x1[2 * i], x1[2 * i + 1]), b(x2[2 * i], x2[2 * i + 1]);
    Vec3 Xe = Vec3::Zero();
    TriangulateDLT(cam1.projection_matrix_, a, cam2.projection_matrix_, b, &Xe);
    const double r = (PinholeCamera::Residual(cam1.projection_matrix_, Xe, a) +
                      PinholeCamera::Residual(cam2.projection_matrix_, Xe, b)) / 2.0;
    bool k = inlier[i] != 0;
    k = k && cam1.Residual(Xe, a) < th1 && cam2.Residual(Xe, b) < th2;
    k = k && cam1.Depth(Xe) > 0 && cam2.Depth(Xe) > 0;
    k = k && BrownPinholeCamera::AngleBetweenRay(cam1, cam2, a, b) > min_angle;
    for (int j = 0; j < 3; ++j) X.push_back(Xe(j));
    res.push_back(r);
    keep.push_back(k ? 1 : 0);
  }
  KVWriter w(out);
  w.put("X", X);
  w.put("residual", res);
  w.put("keep", keep);
  return 0;
}

// Tracks as CSR (track_offsets, camera_index, xy) over the cameras, with one
// 3D point per track; observations of a track in increasing camera order (the
// order of the reference's SubmapTrack map).
static int RunReject(const KV& kv, const char* out) {
  const std::vector<BrownPinholeCamera> cams = LoadCameras(Get(kv, "cameras"));
  const std::vector<double>& pts = Get(kv, "points");
  const std::vector<double>& offs = Get(kv, "track_offsets");
  const std::vector<double>& cam = Get(kv, "camera_index");
  const std::vector<double>& xy = Get(kv, "xy");
  const double precision = Get1(kv, "precision", 4.0);
  const size_t nt = offs.size() - 1;
  std::vector<double> obs_keep(cam.size(), 1.0), track_keep(nt, 1.0);
  double rejected_tracks = 0, rejected_measurements = 0;
  for (size_t t = 0; t < nt; ++t) {
    const Vec3 X(pts[3 * t], pts[3 * t + 1], pts[3 * t + 2]);
    double maxAngle = 0.0;
    Vec3 originRay;
    std::vector<size_t> erase;
    for (size_t o = (size_t)offs[t]; o < (size_t)offs[t + 1]; ++o) {
      const BrownPinholeCamera& c = cams[(size_t)cam[o]];
      const double r = c.Residual(X, Vec2(xy[2 * o], xy[2 * o + 1]));
      const Vec3 dir = (X - c.camera_center_).normalized();
      if (o == (size_t)offs[t]) {
        originRay = dir;
      } else {
        const double angle = R2D(acos(clamp(originRay.dot(dir), -1.0 + 1.e-8, 1.0 - 1.e-8)));
        maxAngle = std::max(angle, maxAngle);
      }
      if (r > precision) erase.push_back(o);
    }
    if (maxAngle < 3) {
      erase.clear();
      for (size_t o = (size_t)offs[t]; o < (size_t)offs[t + 1]; ++o) erase.push_back(o);
    }
    for (size_t e = 0; e < erase.size(); ++e) obs_keep[erase[e]] = 0.0;
    rejected_measurements += (double)erase.size();
    const size_t remaining = (size_t)(offs[t + 1] - offs[t]) - erase.size();
    if (!erase.empty() && remaining < 2) {
      track_keep[t] = 0.0;
      rejected_tracks += 1;
    }
  }
  KVWriter w(out);
  w.put("obs_keep", obs_keep);
  w.put("track_keep", track_keep);
  w.put1("rejected_measurements", rejected_measurements);
  w.put1("rejected_tracks", rejected_tracks);
  return 0;
}

static int RunHistogram(const KV& kv, const char* out) {
  const std::vector<BrownPinholeCamera> cams = LoadCameras(Get(kv, "cameras"));
  const std::vector<double>& pts = Get(kv, "points");
  const std::vector<double>& offs = Get(kv, "track_offsets");
  const std::vector<double>& cam = Get(kv, "camera_index");
  const std::vector<double>& xy = Get(kv, "xy");
  std::vector<float> vec_residuals;
  for (size_t t = 0; t + 1 < offs.size(); ++t) {
    const Vec3 X(pts[3 * t], pts[3 * t + 1], pts[3 * t + 2]);
    for (size_t o = (size_t)offs[t]; o < (size_t)offs[t + 1]; ++o)
      vec_residuals.push_back(cams[(size_t)cam[o]].Residual(X, Vec2(xy[2 * o], xy[2 * o + 1])));
  }
  KVWriter w(out);
  if (vec_residuals.size() > 1) {
    float mn, mx, mean, median;
    MinMaxMeanMedian<float>(vec_residuals.begin(), vec_residuals.end(), mn, mx, mean, median);
    mvg::utils::Histogram<double> histo(mn, mx, 10);
    histo.Add(vec_residuals.begin(), vec_residuals.end());
    std::vector<double> freq(histo.GetHist().begin(), histo.GetHist().end());
    w.put1("min", mn);
    w.put1("max", mx);
    w.put1("mean", mean);
    w.put1("median", median);
    w.put("hist", freq);
    w.put1("underflow", (double)histo.GetUnderflow());
    w.put1("overflow", (double)histo.GetOverflow());
  }
  w.put1("count", (double)vec_residuals.size());
  return 0;
}

// The incremental engine's BA assembly and write-back
// (libs/sfm/src/sfm_incremental_engine.cpp:1250-1393, 1475-1546) over the
// engine's own std::map containers, built here from dense arrays; the
// rotation conversions are ceres's (rotation.h).  Outputs the packed
// parameters_ / observations_ / index vectors, the locked extrinsic block and
// the cameras written back from a given refined parameter set.
static int RunPack(const KV& kv, const char* out) {
  const std::vector<double>& cams = Get(kv, "cameras");
  const std::vector<double>& rec = Get(kv, "reconstructed");
  const std::vector<double>& image_group_key = Get(kv, "image_group_key");
  const std::vector<double>& group_keys = Get(kv, "group_keys");
  const std::vector<double>& group_intr = Get(kv, "group_intrinsics");
  const std::vector<double>& foff = Get(kv, "feature_offsets");
  const std::vector<double>& feats = Get(kv, "features");
  const std::vector<double>& track_keys = Get(kv, "track_keys");
  const std::vector<double>& pts = Get(kv, "points");
  const std::vector<double>& toff = Get(kv, "track_offsets");
  const std::vector<double>& timg = Get(kv, "track_image");
  const std::vector<double>& tfeat = Get(kv, "track_feature");
  const double first_added = Get1(kv, "first_added", -1);
  const size_t ni = rec.size();

  // engine state as the reference holds it
  std::map<size_t, BrownPinholeCamera> map_Camera;
  std::map<size_t, std::vector<std::pair<float, float> > > map_features;
  std::map<size_t, std::vector<size_t> > map_images_id_per_intrinsic_group;
  std::map<size_t, Vec6> map_intrinsics_per_group;
  std::map<size_t, Vec3> map_3d_points;
  std::map<size_t, std::map<size_t, size_t> > map_reconstructed;
  for (size_t g = 0; g < group_keys.size(); ++g) {
    Vec6 v;
    for (int j = 0; j < 6; ++j) v(j) = group_intr[6 * g + j];
    map_intrinsics_per_group[(size_t)group_keys[g]] = v;
  }
  for (size_t i = 0; i < ni; ++i) {
    map_images_id_per_intrinsic_group[(size_t)image_group_key[i]].push_back(i);
    std::vector<std::pair<float, float> >& f = map_features[i];
    for (size_t k = (size_t)foff[i]; k < (size_t)foff[i + 1]; ++k)
      f.push_back(std::make_pair((float)feats[2 * k], (float)feats[2 * k + 1]));
    if (rec[i] == 0) continue;
    const double* c = &cams[18 * i];
    Mat3 R;
    for (int r = 0; r < 3; ++r) for (int k = 0; k < 3; ++k) R(r, k) = c[3 * r + k];
    map_Camera[i] = BrownPinholeCamera(c[12], c[13], c[14], R, Vec3(c[9], c[10], c[11]), c[15], c[16], c[17]);
  }
  for (size_t t = 0; t < track_keys.size(); ++t) {
    const size_t id = (size_t)track_keys[t];
    map_3d_points[id] = Vec3(pts[3 * t], pts[3 * t + 1], pts[3 * t + 2]);
    std::map<size_t, size_t>& tr = map_reconstructed[id];
    for (size_t e = (size_t)toff[t]; e < (size_t)toff[t + 1]; ++e) tr[(size_t)timg[e]] = (size_t)tfeat[e];
  }

  // the pack (:1250-1393)
  size_t measurements = 0;
  for (std::map<size_t, Vec3>::const_iterator it = map_3d_points.begin(); it != map_3d_points.end(); ++it)
    measurements += map_reconstructed[it->first].size();
  std::vector<double> parameters, observations, point_index, cam_ext, cam_intr;
  std::set<size_t> set_camIndex;
  std::map<size_t, size_t> ext_number, intr_number;
  size_t cpt = 0;
  for (std::map<size_t, BrownPinholeCamera>::const_iterator it = map_Camera.begin(); it != map_Camera.end();
       ++it, ++cpt) {
    set_camIndex.insert(it->first);
    ext_number.insert(std::make_pair(it->first, cpt));
    const Mat3 R = it->second.rotation_matrix_;
    double aa[3];
    ceres::RotationMatrixToAngleAxis((const double*)R.data(), aa);
    const Vec3 t = it->second.translation_vector_;
    parameters.push_back(aa[0]);
    parameters.push_back(aa[1]);
    parameters.push_back(aa[2]);
    parameters.push_back(t[0]);
    parameters.push_back(t[1]);
    parameters.push_back(t[2]);
  }
  for (std::map<size_t, Vec6>::const_iterator it = map_intrinsics_per_group.begin();
       it != map_intrinsics_per_group.end(); ++it)
    for (int j = 0; j < 6; ++j) parameters.push_back(it->second(j));
  cpt = 0;
  for (std::map<size_t, std::vector<size_t> >::const_iterator it = map_images_id_per_intrinsic_group.begin();
       it != map_images_id_per_intrinsic_group.end(); ++it, ++cpt)
    for (size_t k = 0; k < it->second.size(); ++k) intr_number.insert(std::make_pair(it->second[k], cpt));
  for (std::map<size_t, Vec3>::const_iterator it = map_3d_points.begin(); it != map_3d_points.end(); ++it)
    for (int j = 0; j < 3; ++j) parameters.push_back(it->second[j]);
  cpt = 0;
  for (std::map<size_t, Vec3>::const_iterator it = map_3d_points.begin(); it != map_3d_points.end(); ++it, ++cpt) {
    const std::map<size_t, size_t>& tr = map_reconstructed[it->first];
    for (std::map<size_t, size_t>::const_iterator e = tr.begin(); e != tr.end(); ++e) {
      if (set_camIndex.find(e->first) == set_camIndex.end()) continue;
      const std::pair<float, float>& f = map_features[e->first][e->second];
      observations.push_back(f.first);
      observations.push_back(f.second);
      point_index.push_back((double)cpt);
      cam_ext.push_back((double)ext_number[e->first]);
      cam_intr.push_back((double)intr_number[e->first]);
    }
  }
  // the locked block (:1437-1443): mutable_camera_extrinsic_for_observation
  // indexes camera_index_extrinsic with the camera ordinal
  double locked = -1;
  if (first_added >= 0 && !ext_number.empty()) {
    const size_t k = ext_number[(size_t)first_added];
    locked = k < cam_ext.size() ? cam_ext[k] : -2;  // -2: the reference reads past its vector
  }

  // the write-back (:1491-1516) of a refined parameter set
  const std::vector<double>& ref_ext = Get(kv, "refined_extrinsics");
  const std::vector<double>& ref_intr = Get(kv, "refined_intrinsics");
  std::vector<double> unpacked;
  for (std::map<size_t, BrownPinholeCamera>::const_iterator it = map_Camera.begin(); it != map_Camera.end(); ++it) {
    const size_t e = ext_number[it->first];
    const double* camE = &ref_ext[6 * e];
    Mat3 R;
    ceres::AngleAxisToRotationMatrix(camE, R.data());
    const double* ci = &ref_intr[6 * intr_number[it->first]];
    const BrownPinholeCamera c(ci[0], ci[1], ci[2], R, Vec3(camE[3], camE[4], camE[5]), ci[3], ci[4], ci[5]);
    for (int r = 0; r < 3; ++r) for (int k = 0; k < 3; ++k) unpacked.push_back(c.rotation_matrix_(r, k));
    for (int r = 0; r < 3; ++r) unpacked.push_back(c.translation_vector_[r]);
    unpacked.push_back(c._f);
    unpacked.push_back(c._ppx);
    unpacked.push_back(c._ppy);
    unpacked.push_back(c._k1);
    unpacked.push_back(c._k2);
    unpacked.push_back(c._k3);
  }
  KVWriter w(out);
  w.put("parameters", parameters);
  w.put("observations", observations);
  w.put("point_index", point_index);
  w.put("camera_index_extrinsic", cam_ext);
  w.put("camera_index_intrinsic", cam_intr);
  w.put1("num_cameras", (double)map_Camera.size());
  w.put1("measurements", (double)measurements);
  w.put1("locked", locked);
  w.put("unpacked", unpacked);
  return 0;
}

// robustResection's AC-RANSAC (libs/sfm/include/mvg/sfm/sfm_robust.h:207-254)
// with the reference's kernels, solvers and ACRANSAC, the kernel wrapped so
// that every model its Fit returns is recorded.  Then, for each recorded
// model, the reference's per-model scoring: ResectionSquaredResidualError
// on the normalised points, std::sort of (error, index) and bestNFA with the
// logcombi tables.  Outputs the normalised points, the models, their
// (nfa, k, e[k-1]), the models per iteration, and ACRANSAC's own result.
template <class Base>
struct RecordingKernel : public Base {
  RecordingKernel(const Mat& a, int w, int h, const Mat& b) : Base(a, w, h, b) {}
  RecordingKernel(const Mat& a, const Mat& b, const Mat3& K) : Base(a, b, K) {}
  mutable std::vector<Mat34> models;
  mutable std::vector<double> per_fit;
  void Fit(const std::vector<size_t>& samples, std::vector<Mat34>* m) const {
    Base::Fit(samples, m);
    models.insert(models.end(), m->begin(), m->end());
    per_fit.push_back((double)m->size());
  }
};

template <class Kernel>
static void RecordAcransac(const Kernel& kernel, const Mat& xn, const Mat& x3d, size_t iters, KVWriter& w) {
  std::vector<size_t> inliers;
  Mat34 P;
  const std::pair<double, double> res =
      mvg::feature::ACRANSAC(kernel, inliers, iters, &P, std::numeric_limits<double>::infinity(), false);
  const size_t n = (size_t)xn.cols(), s = Kernel::MINIMUM_SAMPLES;
  std::vector<float> logc_n, logc_k;
  mvg::feature::makelogcombi_n(n, logc_n);
  mvg::feature::makelogcombi_k(s, n, logc_k);
  const double loge0 = log10((double)Kernel::MAX_MODELS * (n - s));
  std::vector<double> models, nfa, k, emax;
  std::vector<mvg::feature::ErrorIndex> e(n);
  for (size_t m = 0; m < kernel.models.size(); ++m) {
    const Mat34& M = kernel.models[m];
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 4; ++c) models.push_back(M(r, c));
    for (size_t i = 0; i < n; ++i)
      e[i] = mvg::feature::ErrorIndex(mvg::sfm::ResectionSquaredResidualError::Error(M, xn.col(i), x3d.col(i)), i);
    std::sort(e.begin(), e.end());
    const mvg::feature::ErrorIndex best = mvg::feature::bestNFA(
        (int)s, kernel.logalpha0(), e, loge0, std::numeric_limits<double>::infinity(), logc_n, logc_k,
        kernel.multError());
    nfa.push_back(best.first);
    k.push_back((double)best.second);
    emax.push_back(best.second > s ? e[best.second - 1].first : std::numeric_limits<double>::infinity());
  }
  std::vector<double> xnv, inl(inliers.begin(), inliers.end()), Pv;
  for (size_t i = 0; i < n; ++i) { xnv.push_back(xn(0, i)); xnv.push_back(xn(1, i)); }
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 4; ++c) Pv.push_back(P(r, c));
  w.put("x2d_normalized", xnv);
  w.put("models", models);
  w.put("models_per_fit", kernel.per_fit);
  w.put("nfa", nfa);
  w.put("k", k);
  w.put("error_max", emax);
  w.put1("sample_size", (double)s);
  w.put1("max_models", (double)Kernel::MAX_MODELS);
  w.put1("logalpha0", kernel.logalpha0());
  w.put1("normalizer", kernel.normalizer1()(0, 0));
  w.put1("result_error_max", res.first);
  w.put1("result_min_nfa", res.second);
  w.put("result_inliers", inl);
  w.put("result_P", Pv);
}

static int RunAcransac(const KV& kv, const char* out) {
  const std::vector<double>& x2 = Get(kv, "x2d");
  const std::vector<double>& x3 = Get(kv, "x3d");
  const size_t n = x2.size() / 2;
  Mat x2d(2, n), x3d(3, n);
  for (size_t i = 0; i < n; ++i) {
    x2d(0, i) = x2[2 * i];
    x2d(1, i) = x2[2 * i + 1];
    for (int r = 0; r < 3; ++r) x3d(r, i) = x3[3 * i + r];
  }
  srand((unsigned)Get1(kv, "seed", 1));
  const size_t iters = (size_t)Get1(kv, "iterations", 4096);
  KVWriter w(out);
  if (kv.count("K")) {
    const std::vector<double>& kk = Get(kv, "K");
    Mat3 K;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) K(r, c) = kk[3 * r + c];
    typedef mvg::feature::ACKernelAdaptorResection_K<mvg::multiview::P3PSolver,
        mvg::sfm::ResectionSquaredResidualError, mvg::feature::UnnormalizerResection, Mat34> Base;
    RecordingKernel<Base> kernel(x2d, x3d, K);
    Mat xn;
    mvg::multiview::applyTransformationToPoints(x2d, K.inverse(), &xn);
    RecordAcransac(kernel, xn, x3d, iters, w);
  } else {
    const int width = (int)Get1(kv, "width", 1920), height = (int)Get1(kv, "height", 1080);
    typedef mvg::feature::ACKernelAdaptorResection<mvg::multiview::resection::SixPointResectionSolver,
        mvg::sfm::ResectionSquaredResidualError, mvg::feature::UnnormalizerResection, Mat34> Base;
    RecordingKernel<Base> kernel(x2d, width, height, x3d);
    Mat xn;
    Mat3 N1;
    mvg::multiview::NormalizePoints(x2d, &xn, &N1, width, height);
    RecordAcransac(kernel, xn, x3d, iters, w);
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3) { fprintf(stderr, "usage: ref_harness <mode> ...\n"); return 2; }
  const std::string mode = argv[1];
  if (mode == "tri-ring" && argc == 5) return RunTriRing(atoi(argv[2]), atoi(argv[3]), argv[4]);
  if (mode == "tri" && argc == 4) return RunTri(ReadKV(argv[2]), argv[3]);
  if (mode == "ba" && argc == 4) return RunBA(ReadKV(argv[2]), argv[3]);
  if (mode == "eval" && argc == 4) return RunEval(ReadKV(argv[2]), argv[3]);
  if (mode == "two-view" && argc == 4) return RunTwoView(ReadKV(argv[2]), argv[3]);
  if (mode == "reject" && argc == 4) return RunReject(ReadKV(argv[2]), argv[3]);
  if (mode == "histogram" && argc == 4) return RunHistogram(ReadKV(argv[2]), argv[3]);
  if (mode == "pack" && argc == 4) return RunPack(ReadKV(argv[2]), argv[3]);
  if (mode == "acransac" && argc == 4) return RunAcransac(ReadKV(argv[2]), argv[3]);
  fprintf(stderr, "bad arguments\n");
  return 2;
}
