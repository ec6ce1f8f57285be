// gbba_project_forward_noalloc: the forward projection (residuals + robust
// cost) for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host application
// whose device memory is owned by its own pool allocator (everything reserved
// up front, nothing left for a second allocator), or a real-time loop that may
// not take the implicit device synchronisation and unbounded latency of an
// allocation.  They pass device-resident inputs and outputs; the only scratch
// this entry point needs -- one partial cost per block and an error slot -- is
// the file-scope array below, which every GPU that loads the library holds
// until the process exits (GBBA_NOALLOC_MAX_BLOCKS + 32 doubles, ~128 KB).
//
// The array's name is only a host-side stand-in in host code; its device
// address is looked up once per device with cudaGetSymbolAddress and passed to
// the kernels.  Every call shares the array: the error slot is cleared at the
// start of each call, the partials are fully rewritten for the blocks the call
// uses, and calls that overlap on the GPU (two streams, or two host threads)
// race on it.
#include <mutex>

#include "gbba_device.cuh"
#include "gbba_internal.h"

namespace gbba {
namespace {

constexpr int kBlocks = GBBA_NOALLOC_MAX_BLOCKS;
constexpr int kObsPerBlock = GBBA_NOALLOC_OBS_PER_BLOCK;
constexpr int kThreads = 256;

static __device__ __align__(256) double g_noalloc_scratch[kBlocks + 32];

struct DeviceScratch {
  std::mutex lock;
  double* addr = nullptr;
};
constexpr int kMaxDevices = 64;
DeviceScratch g_device_scratch[kMaxDevices];

// Device address of the scratch array on the current device.  The lookup runs
// with that device current and only a success is kept: after a failed lookup
// (a context that is not ready yet, a module that failed to load) the next
// call on that device tries again.
cudaError_t scratch_address(int device, double** out) {
  DeviceScratch& d = g_device_scratch[device];
  std::lock_guard<std::mutex> guard(d.lock);
  if (!d.addr) {
    double* addr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress((void**)&addr, g_noalloc_scratch);
    if (err != cudaSuccess || !addr) {
      *out = nullptr;
      return err != cudaSuccess ? err : cudaErrorInvalidSymbol;
    }
    d.addr = addr;
  }
  *out = d.addr;
  return cudaSuccess;
}

// Block b reduces observations [b*kObsPerBlock, (b+1)*kObsPerBlock) into
// scratch[b]; an out-of-range index sets scratch[kBlocks] and gives NaN.
template <int M>
__global__ void __launch_bounds__(kThreads) k_forward_noalloc(const double* __restrict__ ext,
                                                              const double* __restrict__ intr,
                                                              const double* __restrict__ pts,
                                                              const double* __restrict__ obs,
                                                              const uint32_t* __restrict__ cam,
                                                              const uint32_t* __restrict__ icam,
                                                              const uint32_t* __restrict__ pt, int64_t no, int64_t nc,
                                                              int64_t ni, int64_t np, int loss_type, double a,
                                                              double* __restrict__ res, double* __restrict__ scratch) {
  constexpr int K = Model<M>::K;
  __shared__ double sh[kThreads / 32];
  const int64_t o0 = (int64_t)blockIdx.x * kObsPerBlock;
  const int64_t o1 = min(no, o0 + kObsPerBlock);
  double acc = 0.0;
  for (int64_t o = o0 + threadIdx.x; o < o1; o += kThreads) {
    const uint32_t c = cam[o], g = icam[o], p = pt[o];
    double r[2];
    if (c >= nc || g >= ni || p >= np) {
      scratch[kBlocks] = 1.0;
      r[0] = r[1] = nan("");
      acc += r[0];
    } else {
      double E[6], Kp[K], X[3], dJe[2][6], dJk[2][K], dJx[2][3];
      for (int i = 0; i < 6; ++i) E[i] = ext[6 * (int64_t)c + i];
      for (int i = 0; i < K; ++i) Kp[i] = intr[K * (int64_t)g + i];
      for (int i = 0; i < 3; ++i) X[i] = pts[3 * (int64_t)p + i];
      residual<M, double, false>(Kp, E, X, obs[2 * o], obs[2 * o + 1], r, dJe, dJk, dJx, (double*)nullptr);
      double sr1;
      acc += robust<double>(loss_type, a, r[0] * r[0] + r[1] * r[1], &sr1);
    }
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
    for (int w = 0; w < kThreads / 32; ++w) s += sh[w];
    scratch[blockIdx.x] = s;
  }
}

// Fixed-order sum of this call's block partials into *cost.
__global__ void __launch_bounds__(kThreads) k_finish_noalloc(const double* __restrict__ scratch, int nblocks,
                                                             double* __restrict__ cost) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += kThreads) s += scratch[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *cost = scratch[kBlocks] != 0.0 ? nan("") : sh[0];
}

}  // namespace
}  // namespace gbba

extern "C" gbba_status gbba_project_forward_noalloc(const gbba_problem* P, int32_t loss_type, double loss_scale,
                                                    double* residuals, double* cost, void* stream) {
  using namespace gbba;
  if (!P || P->memory != GBBA_MEMORY_DEVICE || P->camera_model < 0 || P->camera_model > 2) return GBBA_ERROR_INVALID_ARGUMENT;
  if (P->num_observations < 0 || P->num_cameras < 0 || P->num_intrinsics < 0 || P->num_points < 0)
    return GBBA_ERROR_INVALID_ARGUMENT;
  if (P->num_observations > (int64_t)kBlocks * kObsPerBlock) return GBBA_ERROR_TOO_LARGE;
  if (P->num_observations > 0 && (!P->observations || !P->camera_index || !P->intrinsic_index || !P->point_index ||
                                  !P->extrinsics || !P->intrinsics || !P->points))
    return GBBA_ERROR_INVALID_ARGUMENT;
  // An error that earlier work of the caller left pending on this thread is
  // not ours to clear or to report as this call's failure: leave it visible
  // to the caller and do nothing.
  if (cudaPeekAtLastError() != cudaSuccess) return GBBA_ERROR_CUDA;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
    cudaGetLastError();
    return GBBA_ERROR_NO_DEVICE;
  }
  double* scratch = nullptr;
  if (scratch_address(device, &scratch) != cudaSuccess || !scratch) {
    cudaGetLastError();
    return GBBA_ERROR_CUDA;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t no = P->num_observations;
  const int nblocks = (int)((no + kObsPerBlock - 1) / kObsPerBlock);
  if (cudaMemsetAsync(scratch + kBlocks, 0, sizeof(double), st) != cudaSuccess) {
    cudaGetLastError();
    return GBBA_ERROR_CUDA;
  }
  if (nblocks > 0) {
    switch (P->camera_model) {
      case kPinholeF:
        k_forward_noalloc<kPinholeF><<<nblocks, kThreads, 0, st>>>(P->extrinsics, P->intrinsics, P->points, P->observations,
                                                                  P->camera_index, P->intrinsic_index, P->point_index, no,
                                                                  P->num_cameras, P->num_intrinsics, P->num_points, loss_type,
                                                                  loss_scale, residuals, scratch);
        break;
      case kRadialK3:
        k_forward_noalloc<kRadialK3><<<nblocks, kThreads, 0, st>>>(P->extrinsics, P->intrinsics, P->points, P->observations,
                                                                  P->camera_index, P->intrinsic_index, P->point_index, no,
                                                                  P->num_cameras, P->num_intrinsics, P->num_points, loss_type,
                                                                  loss_scale, residuals, scratch);
        break;
      default:
        k_forward_noalloc<kBrownT2><<<nblocks, kThreads, 0, st>>>(P->extrinsics, P->intrinsics, P->points, P->observations,
                                                                 P->camera_index, P->intrinsic_index, P->point_index, no,
                                                                 P->num_cameras, P->num_intrinsics, P->num_points, loss_type,
                                                                 loss_scale, residuals, scratch);
        break;
    }
  }
  if (cost) k_finish_noalloc<<<1, kThreads, 0, st>>>(scratch, nblocks, cost);
  if (cudaGetLastError() != cudaSuccess) return GBBA_ERROR_CUDA;
  return GBBA_SUCCESS;
}
