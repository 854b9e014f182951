// Shared helpers of libcolagb: error state, element-type conversion, warp/block reductions and
// the bounded grid barrier used by the persistent (cooperative) kernels.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string>

#include "../../include/colagb.h"

namespace colagb {

// ---- host-side error state (per calling thread) -----------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);

#define COLAGB_CUDA(call)                                  \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return check_cuda(_e, #call);   \
  } while (0)

#define COLAGB_TRY(call)          \
  do {                            \
    int _s = (call);              \
    if (_s != COLAGB_OK) return _s; \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int num_sms();                 // SM count of the current device (cached per device)
unsigned long long current_context_id();  // unique id of the calling thread's current CUDA context, 0 if none
__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align_up(size_t v, size_t a = 256) { return (v + a - 1) / a * a; }

// Simple bump allocator over a caller-provided workspace.  With base == nullptr it only
// measures, so the same code path computes workspace sizes and hands out pointers.
struct Bump {
  char* base;
  size_t cap;
  bool measure;  // size queries only: nothing is launched
  size_t used = 0;
  size_t peak = 0;
  Bump(void* b, size_t c, bool measure_only = false) : base(static_cast<char*>(b)), cap(c), measure(measure_only) {}
  static Bump measuring() { return Bump(nullptr, 0, true); }
  template <class T>
  T* take(size_t count) {
    size_t off = align_up(used);
    used = off + align_up(count * sizeof(T));
    if (used > peak) peak = used;
    if (base == nullptr) return nullptr;
    return reinterpret_cast<T*>(base + off);
  }
  void release(size_t mark) { used = mark; }
  bool overflow() const { return !measure && peak > cap; }
};

// ---- device-side element conversion ------------------------------------------------------
template <class T> __device__ __forceinline__ float to_f(T v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <class C, class S> __device__ __forceinline__ C ld_as(const S* p) { return static_cast<C>(p[0]); }
template <> __device__ __forceinline__ float ld_as<float, __nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(p[0]);
}
template <> __device__ __forceinline__ double ld_as<double, __nv_bfloat16>(const __nv_bfloat16* p) {
  return static_cast<double>(__bfloat162float(p[0]));
}
template <class C, class S> __device__ __forceinline__ C cvt(S v) { return static_cast<C>(v); }
template <> __device__ __forceinline__ float cvt<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ double cvt<double, __nv_bfloat16>(__nv_bfloat16 v) {
  return static_cast<double>(__bfloat162float(v));
}

// ---- reductions ----------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; every thread gets the result.  `scratch` must hold >= 32 values.
template <class T>
__device__ __forceinline__ T block_sum(T v, T* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  T t = (threadIdx.x < nwarps) ? scratch[threadIdx.x] : T(0);
  if (warp == 0) t = warp_sum(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  T r = scratch[0];
  __syncthreads();
  return r;
}

// ---- bounded grid barrier ---------------------------------------------------------------
// Used only by kernels launched with cudaLaunchCooperativeKernel (all CTAs co-resident).
// Sense/generation barrier on two global words.  A CTA that spins more than `spin_limit`
// times records COLAGB_ERR_TIMEOUT in *err and reports failure; every caller then leaves the
// kernel, so a lost CTA can never hang the GPU.
struct GridBarrier {
  unsigned int* count;
  unsigned int* generation;
  int* err;
  unsigned int nblocks;
  long long spin_limit;
};

__device__ __forceinline__ unsigned int ld_volatile(const unsigned int* p) {
  return *reinterpret_cast<const volatile unsigned int*>(p);
}
__device__ __forceinline__ int ld_volatile_i(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Returns true when every CTA arrived; false on timeout or when another CTA flagged an error.
__device__ __forceinline__ bool grid_sync(const GridBarrier& gb) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned int gen = ld_volatile(gb.generation);
    __threadfence();
    const unsigned int arrived = atomicAdd(gb.count, 1u);
    if (arrived == gb.nblocks - 1) {
      atomicExch(gb.count, 0u);
      __threadfence();
      atomicAdd(gb.generation, 1u);
    } else {
      long long spins = 0;
      while (ld_volatile(gb.generation) == gen) {
        if (ld_volatile_i(gb.err) != 0) { ok = 0; break; }
        if (++spins > gb.spin_limit) {
          atomicCAS(gb.err, 0, COLAGB_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __threadfence();
    if (ld_volatile_i(gb.err) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// A learned (FSAI) preconditioner whose FP32 residual stalls would never reach the 10x drop that
// triggers an FP64 residual replacement, and so would never be judged: while a system runs with
// the FSAI factor and the Jacobi fallback is enabled, a replacement (and with it the judge) is also
// forced after this many steps without one.  Converging FSAI-PCG replaces far more often.
constexpr int kJudgeSteps = 1000;

constexpr long long kDefaultSpinLimit = 20000000LL;  // ~ a few seconds of 20 ns naps

}  // namespace colagb
