// C-ABI entry points of libgbba (include/gbba.h): handle management, the
// solve entry, and the forward / backward projection contract that replaces
// ceres::Problem::Evaluate (3rdparty/ceres/include/ceres/problem.h:392-468)
// for the reference's reprojection functors.
#include <math_constants.h>
#include <cstring>

#include "gbba_device.cuh"
#include "gbba_internal.h"

namespace gbba {
gbba_status solve_impl(gbba_handle* h, const gbba_problem* P, const gbba_options* o, gbba_summary* sum);
gbba_status solve_batched_impl(gbba_handle* h, const gbba_problem* probs, int32_t n, const gbba_options* o,
                               gbba_summary* sums);

static int model_k(int m) { return m == kPinholeF ? 1 : m == kRadialK3 ? 6 : 8; }

static gbba_status check_problem(const gbba_problem* P) {
  if (!P) return GBBA_ERROR_INVALID_ARGUMENT;
  if (P->camera_model < 0 || P->camera_model > 2) return GBBA_ERROR_INVALID_ARGUMENT;
  if (P->memory != GBBA_MEMORY_HOST && P->memory != GBBA_MEMORY_DEVICE) return GBBA_ERROR_INVALID_ARGUMENT;
  if (P->num_cameras < 0 || P->num_intrinsics < 0 || P->num_points < 0 || P->num_observations < 0)
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (P->num_observations > 0xFFFFFFFFLL || P->num_points >= 0xFFFFFFFFLL || P->num_cameras >= 0x7FFFFFFFLL)
    return GBBA_ERROR_TOO_LARGE;
  if (P->num_observations > 0 &&
      (!P->observations || !P->camera_index || !P->intrinsic_index || !P->point_index || !P->extrinsics ||
       !P->intrinsics || !P->points))
    return GBBA_ERROR_INVALID_ARGUMENT;
  return GBBA_SUCCESS;
}

template <typename F>
static gbba_status guarded(gbba_handle* h, void* stream, F&& f) {
  if (!h) return GBBA_ERROR_INVALID_ARGUMENT;
  try {
    GBBA_CUDA(cudaSetDevice(h->device));
    h->active = stream ? (cudaStream_t)stream : h->stream;
    return f();
  } catch (const Error& e) {
    if (std::getenv("GBBA_VERBOSE")) fprintf(stderr, "gbba: %s\n", e.what.c_str());
    cudaGetLastError();
    return e.status;
  }
}

__global__ void k_check_indices(const uint32_t* cam, const uint32_t* icam, const uint32_t* pt, int64_t no, int64_t nc,
                                int64_t ni, int64_t np, int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < no; i += (int64_t)gridDim.x * blockDim.x)
    if (cam[i] >= nc || icam[i] >= ni || pt[i] >= np) atomicExch(err, 1);
}

template <int M>
__global__ void __launch_bounds__(256) k_forward(const double* ext, const double* intr, const double* pts,
                                                 const double* obs, const uint32_t* cam, const uint32_t* icam,
                                                 const uint32_t* pt, int64_t no, int loss_type, double a, double* res,
                                                 double* part) {
  constexpr int K = Model<M>::K;
  __shared__ double sh[8];
  double acc = 0.0;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < no; o += (int64_t)gridDim.x * blockDim.x) {
    double E[6], Kp[K], X[3], r[2], dJe[2][6], dJk[2][K], dJx[2][3];
    for (int i = 0; i < 6; ++i) E[i] = ext[6 * (int64_t)cam[o] + i];
    for (int i = 0; i < K; ++i) Kp[i] = intr[K * (int64_t)icam[o] + i];
    for (int i = 0; i < 3; ++i) X[i] = pts[3 * (int64_t)pt[o] + i];
    residual<M, double, false>(Kp, E, X, obs[2 * o], obs[2 * o + 1], r, dJe, dJk, dJx, (double*)nullptr);
    double sr1;
    acc += robust<double>(loss_type, a, r[0] * r[0] + r[1] * r[1], &sr1);
    if (res) {
      res[2 * o] = r[0];
      res[2 * o + 1] = r[1];
    }
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += sh[w];
    part[blockIdx.x] = s;
  }
}

// Jacobian blocks and gradient of the robustified residual.  T = double is
// the plain FP64 path.  T = float is the Jacobian the mixed solve uses inside
// its Schur build (obs_jacobian<M, float, ...> in gbba_solver.cu): the FP32
// instantiation of the same hand-written adjoint, evaluated at FP32 copies of
// the parameters and observation, with the residual and the Corrector scale
// sqrt(rho') taken in FP64; the blocks are written widened to FP64.
template <int M, typename T>
__global__ void __launch_bounds__(256) k_backward(const double* ext, const double* intr, const double* pts,
                                                  const double* obs, const uint32_t* cam, const uint32_t* icam,
                                                  const uint32_t* pt, int64_t no, int64_t nc, int64_t ni, int loss_type,
                                                  double a, double* je, double* jk, double* jx, double* grad,
                                                  const int* gexp, int pass) {
  constexpr int K = Model<M>::K;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < no; o += (int64_t)gridDim.x * blockDim.x) {
    double E[6], Kp[K], X[3], r[2];
    T Je[2][6], Jk[2][K], Jx[2][3];
    const uint32_t c = cam[o], g = icam[o], p = pt[o];
    for (int i = 0; i < 6; ++i) E[i] = ext[6 * (int64_t)c + i];
    for (int i = 0; i < K; ++i) Kp[i] = intr[K * (int64_t)g + i];
    for (int i = 0; i < 3; ++i) X[i] = pts[3 * (int64_t)p + i];
    if constexpr (sizeof(T) == 8) {
      residual<M, double, true>(Kp, E, X, obs[2 * o], obs[2 * o + 1], r, Je, Jk, Jx, (double*)nullptr);
    } else {
      double dJe[2][6], dJk[2][K], dJx[2][3];
      residual<M, double, false>(Kp, E, X, obs[2 * o], obs[2 * o + 1], r, dJe, dJk, dJx, (double*)nullptr);
      T Ef[6], Kf[K], Xf[3], rf[2];
      for (int i = 0; i < 6; ++i) Ef[i] = (T)E[i];
      for (int i = 0; i < K; ++i) Kf[i] = (T)Kp[i];
      for (int i = 0; i < 3; ++i) Xf[i] = (T)X[i];
      residual<M, T, true>(Kf, Ef, Xf, (T)obs[2 * o], (T)obs[2 * o + 1], rf, Je, Jk, Jx, (T*)nullptr);
    }
    double sr1;
    robust<double>(loss_type, a, r[0] * r[0] + r[1] * r[1], &sr1);
    const double rc0 = r[0] * sr1, rc1 = r[1] * sr1;
    const T s = (T)sr1;
    const bool out = pass == 1;  // the Jacobians are written by the accumulating pass
    for (int i = 0; i < 2; ++i) {
      for (int j = 0; j < 6; ++j) {
        Je[i][j] *= s;
        if (je && out) je[(o * 2 + i) * 6 + j] = (double)Je[i][j];
      }
      for (int j = 0; j < K; ++j) {
        Jk[i][j] *= s;
        if (jk && out) jk[(o * 2 + i) * K + j] = (double)Jk[i][j];
      }
      for (int j = 0; j < 3; ++j) {
        Jx[i][j] *= s;
        if (jx && out) jx[(o * 2 + i) * 3 + j] = (double)Jx[i][j];
      }
    }
    if (grad) {
      // deterministic sums (see lin_fx): pass 0 records each entry's
      // largest |term|, pass 1 adds the terms in fixed point
      auto put = [&](int64_t idx, double v) {
        unsigned long long* q = reinterpret_cast<unsigned long long*>(grad + idx);
        if (pass == 0) atomicMax(q, isfinite(v) ? (unsigned long long)__double_as_longlong(fabs(v)) : ~0ull);
        else atomicAdd(q, (unsigned long long)lin_fx(v, gexp[idx]));
      };
      for (int j = 0; j < 6; ++j) put(6 * (int64_t)c + j, (double)Je[0][j] * rc0 + (double)Je[1][j] * rc1);
      for (int j = 0; j < K; ++j) put(6 * nc + K * (int64_t)g + j, (double)Jk[0][j] * rc0 + (double)Jk[1][j] * rc1);
      for (int j = 0; j < 3; ++j)
        put(6 * nc + K * ni + 3 * (int64_t)p + j, (double)Jx[0][j] * rc0 + (double)Jx[1][j] * rc1);
    }
  }
}

// Between the gradient's passes: each entry's scale exponent from its largest
// term, and the entry cleared for the fixed-point sum; after them: back to
// FP64 (NaN for an entry with a non-finite term).
__global__ void k_grad_exp(int64_t n, double nobs, double* __restrict__ grad, int* __restrict__ gexp) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long* q = reinterpret_cast<unsigned long long*>(grad + i);
    gexp[i] = lin_exp(*q, nobs);
    *q = 0ull;
  }
}
__global__ void k_grad_conv(int64_t n, double* __restrict__ grad, const int* __restrict__ gexp) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const long long v = __double_as_longlong(grad[i]);
    grad[i] = gexp[i] >= kFxNonFinite ? CUDART_NAN : ldexp((double)v, -gexp[i]);
  }
}

struct Staged {
  const double *ext, *intr, *pts, *obs;
  const uint32_t *cam, *icam, *pt;
};

// Make the problem's arrays device-resident (copies for host memory) and check indices.
static Staged stage(gbba_handle* h, const gbba_problem* P, size_t extra_bytes, char** extra) {
  const int64_t no = P->num_observations, nc = P->num_cameras, ni = P->num_intrinsics, np = P->num_points;
  const int k = model_k(P->camera_model);
  cudaStream_t st = h->active;
  Planner pl;
  pl.take<double>(6 * nc);
  pl.take<double>(k * ni);
  pl.take<double>(3 * np);
  pl.take<double>(2 * no);
  pl.take<uint32_t>(3 * no);
  pl.take<int>(1);
  pl.take<char>(extra_bytes);
  h->arena.reset();
  h->arena.reserve(pl.used + 4096);
  Staged s;
  const bool host = P->memory == GBBA_MEMORY_HOST;
  auto put = [&](const void* src, size_t bytes) -> void* {
    void* d = h->arena.take<char>(bytes);
    if (bytes) GBBA_CUDA(cudaMemcpyAsync(d, src, bytes, host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    return d;
  };
  s.ext = (const double*)put(P->extrinsics, sizeof(double) * 6 * nc);
  s.intr = (const double*)put(P->intrinsics, sizeof(double) * k * ni);
  s.pts = (const double*)put(P->points, sizeof(double) * 3 * np);
  s.obs = (const double*)put(P->observations, sizeof(double) * 2 * no);
  s.cam = (const uint32_t*)put(P->camera_index, sizeof(uint32_t) * no);
  s.icam = (const uint32_t*)put(P->intrinsic_index, sizeof(uint32_t) * no);
  s.pt = (const uint32_t*)put(P->point_index, sizeof(uint32_t) * no);
  int* err = h->arena.take<int>(1);
  *extra = h->arena.take<char>(extra_bytes);
  GBBA_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (no > 0) {
    const int grid = std::max(1, std::min<int>((int)ceil_div(no, 256), h->sm_count * 8));
    k_check_indices<<<grid, 256, 0, st>>>(s.cam, s.icam, s.pt, no, nc, ni, np, err);
    check_launch(h);
  }
  int herr = 0;
  GBBA_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  GBBA_CUDA(cudaStreamSynchronize(st));
  GBBA_REQUIRE(herr == 0, GBBA_ERROR_INVALID_ARGUMENT, "observation index out of range");
  return s;
}

}  // namespace gbba

using namespace gbba;

extern "C" {

int gbba_abi_version(void) { return GBBA_ABI_VERSION; }

const char* gbba_status_string(gbba_status s) {
  switch (s) {
    case GBBA_SUCCESS: return "success";
    case GBBA_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case GBBA_ERROR_CUDA: return "CUDA error";
    case GBBA_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case GBBA_ERROR_NUMERICAL: return "non-finite cost at the initial point";
    case GBBA_ERROR_NOT_SUPPORTED: return "not supported";
    case GBBA_ERROR_TOO_LARGE: return "problem exceeds a documented limit";
    case GBBA_ERROR_NO_DEVICE: return "no CUDA device";
    case GBBA_ERROR_TIMEOUT: return "bounded device wait expired";
  }
  return "unknown status";
}

void gbba_default_options(gbba_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->max_num_iterations = 50;
  o->max_num_consecutive_invalid_steps = 5;
  o->function_tolerance = 1e-6;
  o->gradient_tolerance = 1e-10;
  o->parameter_tolerance = 1e-8;
  o->initial_trust_region_radius = 1e4;
  o->max_trust_region_radius = 1e16;
  o->min_trust_region_radius = 1e-32;
  o->min_relative_decrease = 1e-3;
  o->min_lm_diagonal = 1e-6;
  o->max_lm_diagonal = 1e32;
  o->jacobi_scaling = 1;
  o->loss_type = GBBA_LOSS_SQUARED;
  o->loss_scale = 1.0;
  o->linear_solver = GBBA_SOLVER_AUTO;
  o->precision = GBBA_PRECISION_FP64;
  o->max_linear_solver_iterations = 500;
  o->dense_schur_max_size = 16384;
  o->eta = 0.1;
  o->refinement_interval = 10;
  o->use_cuda_graphs = 1;
  o->stream = nullptr;
  o->fp64_polish_iterations = 10;
  o->schur_build = GBBA_SCHUR_BUILD_AUTO;
}

gbba_status gbba_create(int device, gbba_handle** out) {
  if (!out) return GBBA_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GBBA_ERROR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return GBBA_ERROR_INVALID_ARGUMENT;
  gbba_handle* h = new gbba_handle();
  h->device = device;
  try {
    GBBA_CUDA(cudaSetDevice(device));
    GBBA_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    int least = 0;
    GBBA_CUDA(cudaDeviceGetStreamPriorityRange(&least, &h->prio_hi));
    GBBA_CUDA(cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, least));
    GBBA_CUDA(cudaEventCreateWithFlags(&h->ev_main, cudaEventDisableTiming));
    GBBA_CUDA(cudaEventCreateWithFlags(&h->ev_side, cudaEventDisableTiming));
    GBBA_CUDA(cudaEventCreate(&h->ev_k0));
    GBBA_CUDA(cudaEventCreate(&h->ev_k1));
    GBBA_CUDA(cudaHostAlloc((void**)&h->pinned, 256 * sizeof(double), cudaHostAllocDefault));
    GBBA_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
  } catch (const Error& e) {
    delete h;
    return e.status;
  }
  *out = h;
  return GBBA_SUCCESS;
}

void gbba_destroy(gbba_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->arena.release();
  h->pair_arena.release();
  h->item_arena.release();
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->ev_main) cudaEventDestroy(h->ev_main);
  if (h->ev_side) cudaEventDestroy(h->ev_side);
  if (h->ev_k0) cudaEventDestroy(h->ev_k0);
  if (h->ev_k1) cudaEventDestroy(h->ev_k1);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int64_t gbba_launch_count(const gbba_handle* h) { return h ? h->launches : 0; }

gbba_status gbba_last_kernel_time(gbba_handle* h, double* seconds) {
  if (!h || !seconds) return GBBA_ERROR_INVALID_ARGUMENT;
  if (!h->kernel_timed) return GBBA_ERROR_NOT_SUPPORTED;
  if (cudaSetDevice(h->device) != cudaSuccess) {
    cudaGetLastError();
    return GBBA_ERROR_CUDA;
  }
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, h->ev_k0, h->ev_k1) != cudaSuccess) {
    cudaGetLastError();
    return GBBA_ERROR_CUDA;
  }
  *seconds = ms * 1e-3;
  return GBBA_SUCCESS;
}

gbba_status gbba_solve(gbba_handle* h, const gbba_problem* P, const gbba_options* o, gbba_summary* sum) {
  if (!o || !sum) return GBBA_ERROR_INVALID_ARGUMENT;
  const gbba_status pc = check_problem(P);
  if (pc != GBBA_SUCCESS) return pc;
  std::memset(sum, 0, sizeof(*sum));
  return guarded(h, o->stream, [&]() { return solve_impl(h, P, o, sum); });
}

gbba_status gbba_solve_batched(gbba_handle* h, const gbba_problem* problems, int32_t num_problems,
                               const gbba_options* o, gbba_summary* summaries) {
  if (!problems || !o || !summaries || num_problems < 0) return GBBA_ERROR_INVALID_ARGUMENT;
  if (num_problems == 0) return GBBA_SUCCESS;
  for (int32_t i = 0; i < num_problems; ++i) {
    const gbba_status pc = check_problem(&problems[i]);
    if (pc != GBBA_SUCCESS) return pc;
  }
  return guarded(h, o->stream, [&]() { return solve_batched_impl(h, problems, num_problems, o, summaries); });
}

gbba_status gbba_autotune(gbba_handle* h, const gbba_problem* P, const gbba_options* o, int32_t iterations,
                          gbba_tuning* out) {
  if (!o || !out || iterations < 1) return GBBA_ERROR_INVALID_ARGUMENT;
  const gbba_status pc = check_problem(P);
  if (pc != GBBA_SUCCESS) return pc;
  std::memset(out, 0, sizeof(*out));
  return guarded(h, o->stream, [&]() -> gbba_status {
    const int k = P->camera_model == kPinholeF ? 1 : P->camera_model == kRadialK3 ? 6 : 8;
    const size_t ne = 6 * (size_t)P->num_cameras, ni = k * (size_t)P->num_intrinsics, np = 3 * (size_t)P->num_points;
    const bool dev = P->memory == GBBA_MEMORY_DEVICE;
    cudaStream_t st = h->active;
    // the parameters, restored after every trial
    std::vector<double> keep(ne + ni + np);
    auto move = [&](bool save) {
      double* arr[3] = {P->extrinsics, P->intrinsics, P->points};
      const size_t cnt[3] = {ne, ni, np};
      size_t off = 0;
      for (int a = 0; a < 3; ++a) {
        if (cnt[a]) {
          double* host = keep.data() + off;
          if (!dev) std::memcpy(save ? host : arr[a], save ? arr[a] : host, 8 * cnt[a]);
          else
            GBBA_CUDA(cudaMemcpyAsync(save ? (void*)host : (void*)arr[a], save ? (const void*)arr[a] : (const void*)host,
                                      8 * cnt[a], save ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice, st));
        }
        off += cnt[a];
      }
      if (dev) GBBA_CUDA(cudaStreamSynchronize(st));
    };
    move(true);
    // fixed work per trial: exactly `iterations` LM iterations
    gbba_options t = *o;
    t.max_num_iterations = iterations;
    t.function_tolerance = 0.0;
    t.gradient_tolerance = 0.0;
    t.parameter_tolerance = 0.0;
    t.fp64_polish_iterations = 0;
    // one trial: two solves (the first warms the workspace), the second's
    // summary; the handle's choices are restored if a solve fails
    const int keep_chunk = h->pair_chunk, keep_cw = h->camera_warps;
    const bool keep_ft = h->factor_tensor;
    gbba_summary sum;
    auto trial = [&]() -> gbba_status {
      for (int rep = 0; rep < 2; ++rep) {
        std::memset(&sum, 0, sizeof(sum));
        gbba_status s = GBBA_SUCCESS;
        try {
          s = solve_impl(h, P, &t, &sum);
        } catch (...) {
          h->pair_chunk = keep_chunk;
          h->camera_warps = keep_cw;
          h->factor_tensor = keep_ft;
          throw;
        }
        move(false);
        if (s != GBBA_SUCCESS) {
          h->pair_chunk = keep_chunk;
          h->camera_warps = keep_cw;
          h->factor_tensor = keep_ft;
          return s;
        }
      }
      return GBBA_SUCCESS;
    };
    auto per_iter = [&](double total) { return sum.num_iterations > 0 ? total / sum.num_iterations : total; };
    // 1. work-item size of the camera-pair products
    const int32_t cand[3] = {32, 64, 128};
    out->num_candidates = 3;
    int best = -1;
    bool iterative = false;
    for (int c = 0; c < 3; ++c) {
      h->pair_chunk = cand[c];
      const gbba_status s = trial();
      if (s != GBBA_SUCCESS) return s;
      iterative = sum.linear_solver_iterations > 0;
      out->candidates[c] = cand[c];
      out->schur_time_s[c] = per_iter(sum.schur_kernel_time_s);
      if (best < 0 || out->schur_time_s[c] < out->schur_time_s[best]) best = c;
      if (iterative) break;  // the iterative path forms no camera-pair products
    }
    if (iterative) {
      h->pair_chunk = keep_chunk;
      out->num_candidates = 0;
      out->pair_chunk = keep_chunk;
    } else {
      h->pair_chunk = cand[best];
      out->pair_chunk = cand[best];
    }
    out->factor_tensor = -1;
    out->camera_warps = 0;
    if (!iterative && t.precision == GBBA_PRECISION_MIXED) {
      // 2. trailing-update engine of the dense FP32 factorisation
      for (int e = 0; e < 2; ++e) {
        h->factor_tensor = e == 1;
        const gbba_status s = trial();
        if (s != GBBA_SUCCESS) return s;
        out->factor_time_s[e] = per_iter(sum.factor_time_s);
      }
      h->factor_tensor = out->factor_time_s[1] <= out->factor_time_s[0];
      out->factor_tensor = h->factor_tensor ? 1 : 0;
    } else if (iterative) {
      // 3. warps per camera of the PCG camera kernels
      const int warps[3] = {2, 4, 8};
      for (int w = 0; w < 3; ++w) {
        h->camera_warps = warps[w];
        const gbba_status s = trial();
        if (s != GBBA_SUCCESS) return s;
        out->pcg_time_s[w] = per_iter(sum.linear_solver_time_s + sum.jacobian_time_s);
      }
      int wb = 0;  // the fastest, once all three are timed
      for (int w = 1; w < 3; ++w)
        if (out->pcg_time_s[w] < out->pcg_time_s[wb]) wb = w;
      h->camera_warps = warps[wb];
      out->camera_warps = warps[wb];
    }
    return GBBA_SUCCESS;
  });
}

gbba_status gbba_project_forward(gbba_handle* h, const gbba_problem* P, int32_t loss_type, double loss_scale,
                                 double* residuals, double* cost) {
  const gbba_status pc = check_problem(P);
  if (pc != GBBA_SUCCESS) return pc;
  return guarded(h, nullptr, [&]() {
    const int64_t no = P->num_observations;
    const int grid = std::max(1, std::min<int>((int)ceil_div(std::max<int64_t>(no, 1), 256), h->sm_count * 8));
    const size_t res_bytes = residuals ? sizeof(double) * 2 * no : 0;
    char* extra;
    Staged s = stage(h, P, res_bytes + sizeof(double) * grid, &extra);
    double* dres = residuals ? (double*)extra : nullptr;
    double* part = (double*)(extra + res_bytes);
    cudaStream_t st = h->active;
    switch (P->camera_model) {
      case kPinholeF: k_forward<kPinholeF><<<grid, 256, 0, st>>>(s.ext, s.intr, s.pts, s.obs, s.cam, s.icam, s.pt, no, loss_type, loss_scale, dres, part); break;
      case kRadialK3: k_forward<kRadialK3><<<grid, 256, 0, st>>>(s.ext, s.intr, s.pts, s.obs, s.cam, s.icam, s.pt, no, loss_type, loss_scale, dres, part); break;
      default: k_forward<kBrownT2><<<grid, 256, 0, st>>>(s.ext, s.intr, s.pts, s.obs, s.cam, s.icam, s.pt, no, loss_type, loss_scale, dres, part); break;
    }
    check_launch(h);
    std::vector<double> hp(grid);
    GBBA_CUDA(cudaMemcpyAsync(hp.data(), part, sizeof(double) * grid, cudaMemcpyDeviceToHost, st));
    if (residuals)
      GBBA_CUDA(cudaMemcpyAsync(residuals, dres, res_bytes,
                                P->memory == GBBA_MEMORY_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    double c = 0.0;
    for (double v : hp) c += v;
    if (cost) *cost = c;
    return GBBA_SUCCESS;
  });
}

static gbba_status project_backward(gbba_handle* h, const gbba_problem* P, int32_t loss_type, double loss_scale,
                                    bool fp32, double* jac_extrinsic, double* jac_intrinsic, double* jac_point,
                                    double* gradient) {
  const gbba_status pc = check_problem(P);
  if (pc != GBBA_SUCCESS) return pc;
  return guarded(h, nullptr, [&]() {
    const int64_t no = P->num_observations, nc = P->num_cameras, ni = P->num_intrinsics, np = P->num_points;
    const int k = model_k(P->camera_model);
    const size_t be = jac_extrinsic ? sizeof(double) * no * 12 : 0;
    const size_t bk = jac_intrinsic ? sizeof(double) * no * 2 * k : 0;
    const size_t bx = jac_point ? sizeof(double) * no * 6 : 0;
    const int64_t ng = 6 * nc + k * ni + 3 * np;
    const size_t bg = gradient ? sizeof(double) * ng : 0;
    const size_t bgx = gradient ? sizeof(int) * ng : 0;  // the gradient entries' scale exponents
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    char* extra;
    Staged s = stage(h, P, al(be) + al(bk) + al(bx) + al(bg) + al(bgx), &extra);
    double* dje = be ? (double*)extra : nullptr;
    double* djk = bk ? (double*)(extra + al(be)) : nullptr;
    double* djx = bx ? (double*)(extra + al(be) + al(bk)) : nullptr;
    double* dg = bg ? (double*)(extra + al(be) + al(bk) + al(bx)) : nullptr;
    int* dgx = bgx ? (int*)(extra + al(be) + al(bk) + al(bx) + al(bg)) : nullptr;
    cudaStream_t st = h->active;
    if (dg) GBBA_CUDA(cudaMemsetAsync(dg, 0, bg, st));
    const int grid = std::max(1, std::min<int>((int)ceil_div(std::max<int64_t>(no, 1), 256), h->sm_count * 8));
    const unsigned gg = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(ng, 256), 4096));
    auto run = [&](auto kern) {
      // with a gradient: a pass for the largest terms, the exponents, then
      // the fixed-point sums (and the Jacobians), then back to FP64
      if (dg) {
        kern<<<grid, 256, 0, st>>>(s.ext, s.intr, s.pts, s.obs, s.cam, s.icam, s.pt, no, nc, ni, loss_type,
                                   loss_scale, dje, djk, djx, dg, dgx, 0);
        check_launch(h);
        k_grad_exp<<<gg, 256, 0, st>>>(ng, (double)std::max<int64_t>(1, no), dg, dgx);
        check_launch(h);
      }
      kern<<<grid, 256, 0, st>>>(s.ext, s.intr, s.pts, s.obs, s.cam, s.icam, s.pt, no, nc, ni, loss_type, loss_scale,
                                 dje, djk, djx, dg, dgx, 1);
      check_launch(h);
      if (dg) {
        k_grad_conv<<<gg, 256, 0, st>>>(ng, dg, dgx);
        check_launch(h);
      }
    };
    switch (P->camera_model) {
      case kPinholeF: fp32 ? run(k_backward<kPinholeF, float>) : run(k_backward<kPinholeF, double>); break;
      case kRadialK3: fp32 ? run(k_backward<kRadialK3, float>) : run(k_backward<kRadialK3, double>); break;
      default: fp32 ? run(k_backward<kBrownT2, float>) : run(k_backward<kBrownT2, double>); break;
    }
    const cudaMemcpyKind kind = P->memory == GBBA_MEMORY_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (be) GBBA_CUDA(cudaMemcpyAsync(jac_extrinsic, dje, be, kind, st));
    if (bk) GBBA_CUDA(cudaMemcpyAsync(jac_intrinsic, djk, bk, kind, st));
    if (bx) GBBA_CUDA(cudaMemcpyAsync(jac_point, djx, bx, kind, st));
    if (bg) GBBA_CUDA(cudaMemcpyAsync(gradient, dg, bg, kind, st));
    GBBA_CUDA(cudaStreamSynchronize(st));
    return GBBA_SUCCESS;
  });
}

gbba_status gbba_project_backward(gbba_handle* h, const gbba_problem* P, int32_t loss_type, double loss_scale,
                                  double* jac_extrinsic, double* jac_intrinsic, double* jac_point, double* gradient) {
  return project_backward(h, P, loss_type, loss_scale, false, jac_extrinsic, jac_intrinsic, jac_point, gradient);
}

gbba_status gbba_project_backward_mixed(gbba_handle* h, const gbba_problem* P, int32_t loss_type, double loss_scale,
                                        double* jac_extrinsic, double* jac_intrinsic, double* jac_point,
                                        double* gradient) {
  return project_backward(h, P, loss_type, loss_scale, true, jac_extrinsic, jac_intrinsic, jac_point, gradient);
}

}  // extern "C"
