// Host-side internals shared by the translation units of libgbba: the handle,
// its device workspace, error plumbing and launch accounting.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbba.h"
#include "../../include/gbtri.h"

namespace gbba {

// Error type carried across internal C++ calls; converted to gbba_status at
// the C boundary (no exception crosses it).
struct Error {
  gbba_status status;
  std::string what;
};

#define GBBA_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      throw ::gbba::Error{e_ == cudaErrorMemoryAllocation ? GBBA_ERROR_OUT_OF_MEMORY      \
                                                          : GBBA_ERROR_CUDA,              \
                          std::string(#call) + ": " + cudaGetErrorString(e_)};            \
    }                                                                                     \
  } while (0)

#define GBBA_REQUIRE(cond, st, msg)                    \
  do {                                                 \
    if (!(cond)) throw ::gbba::Error{(st), (msg)};     \
  } while (0)

// Per-process set-up that belongs to a device (kernel attributes such as the
// opt-in to more than 48 KB of dynamic shared memory): `configure` runs with
// the current device, under a lock, at most once per device, and only a
// success is remembered, so a failed set-up is tried again by the next call.
struct PerDeviceOnce {
  std::mutex lock;
  uint64_t done = 0;  // bit d: device d is configured
  template <typename F>
  void run(F&& configure) {
    int dev = 0;
    GBBA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> guard(lock);
    if (dev < 64 && ((done >> dev) & 1u)) return;
    configure();  // throws gbba::Error on failure
    if (dev < 64) done |= uint64_t(1) << dev;
  }
};

// A device arena: one growable allocation carved by a bump pointer.  Solves
// reuse it across calls, so the steady state makes no cudaMalloc.
struct Arena {
  char* base = nullptr;
  size_t capacity = 0;
  size_t used = 0;
  size_t high_water = 0;
  void reset() { used = 0; }
  void reserve(size_t bytes) {
    if (bytes <= capacity) return;
    if (base) cudaFree(base);
    base = nullptr;
    capacity = 0;
    GBBA_CUDA(cudaMalloc(&base, bytes));
    capacity = bytes;
  }
  template <typename T>
  T* take(size_t count) {
    const size_t bytes = ((count * sizeof(T)) + 255) & ~size_t(255);
    GBBA_REQUIRE(used + bytes <= capacity, GBBA_ERROR_OUT_OF_MEMORY, "workspace overflow");
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    if (used > high_water) high_water = used;
    return p;
  }
  void release() {
    if (base) cudaFree(base);
    base = nullptr;
    capacity = used = 0;
  }
};

// Size planner: the same sequence of take() calls run against a counter so
// that the arena can be reserved once before the real carve.
struct Planner {
  size_t used = 0;
  template <typename T>
  T* take(size_t count) {
    used += ((count * sizeof(T)) + 255) & ~size_t(255);
    return nullptr;
  }
};

}  // namespace gbba

struct gbba_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  gbba::Arena arena;
  gbba::Arena pair_arena;  // pair list + camera CSR of the atomic-free Schur build
  gbba::Arena item_arena;  // work items and partial sums of the pair kernel
  // small pinned host buffer for per-iteration scalars
  double* pinned = nullptr;
  int64_t launches = 0;
  int sm_count = 0;
  cudaStream_t active = nullptr;  // stream of the current call
  cudaGraphExec_t graph_exec = nullptr;
  // Dense factorisation look-ahead: the trailing update runs on `side` while
  // the next panel is factored on the call's stream at priority `prio_hi`.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_main = nullptr, ev_side = nullptr;
  int prio_hi = 0;
  // observation pairs per work item of the camera-pair products (gbba_autotune)
  int pair_chunk = 128;
  // FP32 dense factorisation: trailing update on the tensor cores (3xTF32
  // tcgen05) or on the FP32 pipes (gbba_autotune)
  bool factor_tensor = true;
  // iterative path: warps per camera of the camera-side PCG kernels (2, 4 or 8; gbba_autotune)
  int camera_warps = 4;
  // device time of the main kernel(s) of the last triangulation or engine-scan call
  cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;
  bool kernel_timed = false;
};

namespace gbba {

inline void count_launch(gbba_handle* h, int n = 1) { h->launches += n; }

inline void check_launch(gbba_handle* h) {
  count_launch(h);
  GBBA_CUDA(cudaGetLastError());
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Runs the body of an engine-side entry point (gbsfm_*) on the handle's
// device and stream, turning an internal error into its status.
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

// Grid of a grid-stride loop over n items: enough blocks to cover them, at
// most 16 per SM.
inline unsigned grid_for(gbba_handle* h, int64_t n, int threads) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), (int64_t)h->sm_count * 16));
}

// Brackets the main kernel(s) of a call with the handle's events; the span is
// read back by gbba_last_kernel_time.
struct KernelTimer {
  gbba_handle* h;
  explicit KernelTimer(gbba_handle* hh) : h(hh) { GBBA_CUDA(cudaEventRecord(h->ev_k0, h->active)); }
  void stop() {
    GBBA_CUDA(cudaEventRecord(h->ev_k1, h->active));
    h->kernel_timed = true;
  }
};

// Device view of an input array: the caller's pointer (device memory) or a
// staged copy (host memory).
template <typename T>
inline const T* in_view(gbba_handle* h, const T* p, size_t count, int memory) {
  if (!p || memory == GBBA_MEMORY_DEVICE) return p;
  T* d = h->arena.take<T>(count);
  if (count) GBBA_CUDA(cudaMemcpyAsync(d, p, count * sizeof(T), cudaMemcpyHostToDevice, h->active));
  return d;
}
template <typename T>
inline T* out_view(gbba_handle* h, T* p, size_t count, int memory) {
  if (!p || memory == GBBA_MEMORY_DEVICE) return p;
  return h->arena.take<T>(count);
}
template <typename T>
inline void out_back(gbba_handle* h, T* user, const T* dev, size_t count, int memory) {
  if (!user || memory == GBBA_MEMORY_DEVICE || count == 0) return;
  GBBA_CUDA(cudaMemcpyAsync(user, dev, count * sizeof(T), cudaMemcpyDeviceToHost, h->active));
}

// Vector type of 16-byte loads and stores.
template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

// Four consecutive values through 16-byte accesses (p 16-byte aligned).
template <typename T>
__device__ __forceinline__ void ld4(const T* p, T v[4]) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n;
#pragma unroll
  for (int q = 0; q < 4 / W; ++q) {
    const V x = reinterpret_cast<const V*>(p)[q];
    const T* e = reinterpret_cast<const T*>(&x);
#pragma unroll
    for (int w = 0; w < W; ++w) v[q * W + w] = e[w];
  }
}
template <typename T>
__device__ __forceinline__ void st4(T* p, const T v[4]) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n;
#pragma unroll
  for (int q = 0; q < 4 / W; ++q) {
    V x;
    T* e = reinterpret_cast<T*>(&x);
#pragma unroll
    for (int w = 0; w < W; ++w) e[w] = v[q * W + w];
    reinterpret_cast<V*>(p)[q] = x;
  }
}


}  // namespace gbba
