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
// The last three restate the engines' loops (whose classes need the whole
// engine) around the reference's own camera, triangulation and histogram code.
//
// File format ("kv text"): a sequence of records `name count` followed by
// `count` whitespace-separated numbers (%.17g).

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
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
  fprintf(stderr, "bad arguments\n");
  return 2;
}
