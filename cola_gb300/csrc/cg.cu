// Conjugate gradients (cola/linalg/inverse/cg.py) on sm_103a.
//
// Reference loop (run_batched_cg, cg.py:94-119; take_cg_step :141-154):
//   mult = |b|_col ; b <- b / mult (safe division, :96-97)
//   r0 = b - A x0 ; z0 = P r0 ; p0 = z0 ; gamma0 = <r0, z0>              (initialize :122-130)
//   tol_eff = tol * |r0| + tol                                           (:101)
//   while any(|r| > tol_eff) and k < max_iters:                          (cond_fun :133-138)
//     conv = |r| < 1e-40 ; Ap = A p ; alpha = gamma / <p, Ap> (0 if conv) (:143-147, :157-162)
//     x += alpha p ; r -= alpha Ap ; z = P r                             (:148-150)
//     gamma' = <r, z> ; beta = gamma' / gamma (0 if conv) ; p = z + beta p (:151-152, :165-170)
//   return x * mult                                                      (:119)
// Divisions use do_safe_div (:173-178): |denominator| < 1e-40 is replaced by 1e-40.
//
// Two executions of that loop:
//   * fused: one cooperative persistent kernel runs the whole solve for a Dense or CSR operator
//     (optionally + c*I) with P = identity or Diagonal; three bounded grid barriers per step.
//   * generic: any operator program / preconditioner; four launches per step, the stop test is
//     evaluated on the device and the host polls it every `check_every` steps (the reference
//     syncs twice per step, torch_tqdm.py:42 and cg.py:136).
// Column sums are reduced in a fixed order so every CTA derives bit-identical alpha / beta.
#include <cooperative_groups.h>
#include <cuda.h>

#include <cmath>
#include <mutex>
#include <type_traits>
#include <string>
#include <vector>

#include "common.cuh"
#include "ops.cuh"

namespace colagb {

// Unique id of the calling thread's current CUDA context (0 when there is none yet or it cannot be
// read), through the runtime's driver entry points so that the library does not link libcuda.
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);

unsigned long long current_context_id() {
  static PfnCtxGetCurrent get_cur = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<PfnCtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PfnCtxGetId>(f);
    cudaGetLastError();
  });
  if (!get_cur || !get_id) return 0;
  CUcontext ctx = nullptr;
  if (get_cur(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}


// A private non-blocking stream per CUDA context, used only to capture the generic CG loop's launch
// block into a graph (capture is not allowed on the legacy default stream callers often use); the
// graph is then launched on the caller's stream.  Null when no context id can be read.
static cudaStream_t capture_stream() {
  static std::mutex mu;
  static std::vector<std::pair<unsigned long long, cudaStream_t>> streams;
  const unsigned long long id = current_context_id();
  if (id == 0) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  for (const auto& e : streams)
    if (e.first == id) return e.second;
  cudaStream_t cs = nullptr;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  streams.emplace_back(id, cs);
  return cs;
}

template <class T> struct SmallValue;
template <> struct SmallValue<float> { static constexpr float v = 1e-40f; };
template <> struct SmallValue<double> { static constexpr double v = 1e-40; };

template <class T>
__device__ __forceinline__ T safe_div(T num, T den) {
  const T eps = SmallValue<T>::v;
  return num / (fabs(den) < eps ? eps : den);
}

template <class T>
__device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------------------------
// Column reductions.  Threads of a block are arranged as (rows_per_pass x kc) with kc = min(k, 256);
// f(i, c) is evaluated for every owned unit and summed per column; the block writes partials[c].
template <class T, class F>
__device__ __forceinline__ void block_col_partials(int64_t row_base, int64_t row_end, int64_t bidx, int64_t nblk,
                                                   int64_t k, F f, T* partials_out, T* smem) {
  // rows row_base + bidx*rpp + my_r, stepping rpp*nblk; bidx/nblk = (blockIdx, gridDim) for a
  // grid-stride sweep or (0, 1) for a block-private row range.
  const int t = threadIdx.x;
  for (int64_t c0 = 0; c0 < k; c0 += blockDim.x) {
    const int kc = (int)((k - c0) < (int64_t)blockDim.x ? (k - c0) : (int64_t)blockDim.x);
    const int rpp = blockDim.x / kc;
    const int my_c = t % kc, my_r = t / kc;
    T acc = T(0);
    if (my_r < rpp) {
      const int64_t c = c0 + my_c;
      for (int64_t i = row_base + bidx * rpp + my_r; i < row_end; i += (int64_t)rpp * nblk) acc += f(i, c);
    }
    smem[t] = acc;
    __syncthreads();
    // tree over the rpp row slots of each column (a serial sum by one thread per column costs
    // ~rpp dependent shared-memory round trips, 256 of them for a single right-hand side)
    for (int w = rpp; w > 1;) {
      const int h = (w + 1) >> 1;
      if (my_r < w - h) smem[t] += smem[t + h * kc];
      __syncthreads();
      w = h;
    }
    if (t < kc) partials_out[c0 + t] = smem[t];
    __syncthreads();
  }
}

// Fixed-order sum of partials[b * k + c] over b < nb (reads bypass L1).
template <class T>
__device__ __forceinline__ T sum_partials(const T* partials, int nb, int64_t k, int64_t c) {
  T s = T(0);
  for (int b = 0; b < nb; ++b) s += ldcg(partials + (int64_t)b * k + c);
  return s;
}

// Sum of column c of the per-CTA partials, formed by the whole block (every thread gets it).
template <class T>
__device__ __forceinline__ T block_total(const T* partials, int nb, int64_t k, int64_t c, T* red) {
  T v = T(0);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) v += ldcg(partials + (int64_t)b * k + c);
  return block_sum(v, red);
}

// Column totals of the per-CTA partials for the first kStage columns, block-parallel, into shared
// memory (one thread summing nb partials from L2 in sequence costs nb dependent round trips);
// total_at reads them, summing serially only for columns beyond kStage.
constexpr int kStage = 64;
template <class T>
__device__ __forceinline__ void stage_totals(const T* partials, int nb, int64_t k, T* tot, T* red) {
  const int64_t kk = k < kStage ? k : kStage;
  for (int64_t c = 0; c < kk; ++c) {
    const T v = block_total(partials, nb, k, c, red);
    if (threadIdx.x == 0) tot[c] = v;
  }
  __syncthreads();
}
template <class T>
__device__ __forceinline__ T total_at(const T* partials, int nb, int64_t k, int64_t c, const T* tot) {
  return c < kStage ? tot[c] : sum_partials(partials, nb, k, c);
}

__device__ __forceinline__ bool is_last_block(unsigned int* counter) {
  __shared__ int s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

// ---------------------------------------------------------------------------------------------
// State of one solve in device memory
template <class T>
struct CgScalars {
  T* mult;     // |b| per column
  T* tol_eff;  // tol * |r0| + tol
  T* gamma;    // <r, z>
  T* alpha;
  T* beta;
  T* rnorm;    // |r|
  int* conv;   // |r| < 1e-40 at the start of the current step
  int* done;   // loop finished
  int* iters;  // k
  T* pA;       // partials [nb][k] for <p, Ap> / |b|
  T* pB;       // partials [nb][k] for <r, z>
  T* pC;       // partials [nb][k] for |r|^2
  unsigned int* counters;  // 4 last-block counters
};

// ---------------------------------------------------------------------------------------------
// generic-path kernels (grid = nb blocks of 256 threads)

template <class T>
__global__ void __launch_bounds__(256) k_colnorm_b(const T* B, int64_t ldb, int64_t n, int64_t k, CgScalars<T> s) {
  __shared__ T smem[256];
  block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                        [&](int64_t i, int64_t c) { const T v = B[i * ldb + c]; return v * v; },
                        s.pA + (int64_t)blockIdx.x * k, smem);
  if (is_last_block(s.counters + 0)) {
    __shared__ T totA[kStage], red[32];
    stage_totals(s.pA, gridDim.x, k, totA, red);
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) s.mult[c] = sqrt(total_at(s.pA, gridDim.x, k, c, totA));
    if (threadIdx.x == 0) s.counters[0] = 0;
  }
}

// r = b / mult
template <class T>
__global__ void k_scale_b(const T* B, int64_t ldb, T* R, int64_t n, int64_t k, CgScalars<T> s) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * k; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / k, c = u - i * k;
    R[u] = safe_div(B[i * ldb + c], s.mult[c]);
  }
}

// p = z (z = dinv*r, r, or Z); partials <r,z>, |r|^2; last block: gamma, rnorm, tol_eff, done
template <class T, int PK>
__global__ void __launch_bounds__(256) k_init(const T* R, const T* Z, const T* dinv, T* P, int64_t n, int64_t k,
                                              double tol, int max_iters, T* hist, CgScalars<T> s) {
  __shared__ T smem[256];
  block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                        [&](int64_t i, int64_t c) {
                          const T r = R[i * k + c];
                          const T z = PK == 0 ? r : (PK == 1 ? dinv[i] * r : Z[i * k + c]);
                          P[i * k + c] = z;
                          return r * z;
                        },
                        s.pB + (int64_t)blockIdx.x * k, smem);
  block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                        [&](int64_t i, int64_t c) { const T r = R[i * k + c]; return r * r; },
                        s.pC + (int64_t)blockIdx.x * k, smem);
  if (is_last_block(s.counters + 1)) {
    __shared__ int s_any;
    __shared__ T s_mean;
    __shared__ T totB[kStage], totC[kStage], red[32];
    stage_totals(s.pB, gridDim.x, k, totB, red);
    stage_totals(s.pC, gridDim.x, k, totC, red);
    if (threadIdx.x == 0) { s_any = 0; s_mean = T(0); }
    __syncthreads();
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
      const T g = total_at(s.pB, gridDim.x, k, c, totB);
      const T rn = sqrt(total_at(s.pC, gridDim.x, k, c, totC));
      s.gamma[c] = g;
      s.rnorm[c] = rn;
      s.alpha[c] = T(0);
      s.beta[c] = T(0);
      const T te = (T)tol * rn + (T)tol;
      s.tol_eff[c] = te;
      if (rn > te) atomicOr(&s_any, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      T m = T(0);
      for (int64_t c = 0; c < k; ++c) m += s.rnorm[c];
      if (hist) hist[0] = m / (T)k;
      *s.iters = 0;
      *s.done = !(s_any && 0 < max_iters);
      s.counters[1] = 0;
    }
  }
}

// <p, Ap> partials; last block: conv flags and alpha
template <class T>
__global__ void __launch_bounds__(256) k_alpha(const T* P, const T* AP, int64_t n, int64_t k, CgScalars<T> s) {
  if (*s.done) return;
  __shared__ T smem[256];
  block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                        [&](int64_t i, int64_t c) { return P[i * k + c] * AP[i * k + c]; },
                        s.pA + (int64_t)blockIdx.x * k, smem);
  if (is_last_block(s.counters + 2)) {
    __shared__ T totA[kStage], red[32];
    stage_totals(s.pA, gridDim.x, k, totA, red);
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
      const int cv = s.rnorm[c] < SmallValue<T>::v;
      s.conv[c] = cv;
      const T a = safe_div(s.gamma[c], total_at(s.pA, gridDim.x, k, c, totA));
      s.alpha[c] = cv ? T(0) : a;
    }
    if (threadIdx.x == 0) s.counters[2] = 0;
  }
}

// x += alpha p ; r -= alpha Ap ; (PK 0/1: z from r) partials <r,z>, |r|^2 ; last block: beta, stop test.
// PK == 2 (general P): only x, r and |r|^2 here; <r, z> comes from k_gamma after z = P r.
template <class T, int PK>
__global__ void __launch_bounds__(256) k_update(T* X, int64_t ldx, T* R, const T* P, const T* AP, const T* dinv,
                                                int64_t n, int64_t k, int max_iters, T* hist, CgScalars<T> s) {
  if (*s.done) return;
  __shared__ T smem[256];
  block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                        [&](int64_t i, int64_t c) {
                          const T a = s.alpha[c];
                          X[i * ldx + c] += a * P[i * k + c];
                          const T r = R[i * k + c] - a * AP[i * k + c];
                          R[i * k + c] = r;
                          return r * r;
                        },
                        s.pC + (int64_t)blockIdx.x * k, smem);
  if (PK != 2)
    block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                          [&](int64_t i, int64_t c) {
                            const T r = R[i * k + c];
                            return r * (PK == 0 ? r : dinv[i] * r);
                          },
                          s.pB + (int64_t)blockIdx.x * k, smem);
  if (PK == 2) {
    if (is_last_block(s.counters + 3)) {
      __shared__ T totC2[kStage], red2[32];
      stage_totals(s.pC, gridDim.x, k, totC2, red2);
      for (int64_t c = threadIdx.x; c < k; c += blockDim.x) s.rnorm[c] = sqrt(total_at(s.pC, gridDim.x, k, c, totC2));
      if (threadIdx.x == 0) s.counters[3] = 0;
    }
    return;
  }
  if (is_last_block(s.counters + 3)) {
    __shared__ int s_any;
    __shared__ T totB[kStage], totC[kStage], red[32];
    stage_totals(s.pB, gridDim.x, k, totB, red);
    stage_totals(s.pC, gridDim.x, k, totC, red);
    if (threadIdx.x == 0) s_any = 0;
    __syncthreads();
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
      const T g1 = total_at(s.pB, gridDim.x, k, c, totB);
      const T b = safe_div(g1, s.gamma[c]);
      s.beta[c] = s.conv[c] ? T(0) : b;
      s.gamma[c] = g1;
      const T rn = sqrt(total_at(s.pC, gridDim.x, k, c, totC));
      s.rnorm[c] = rn;
      if (rn > s.tol_eff[c]) atomicOr(&s_any, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int it = *s.iters + 1;
      *s.iters = it;
      if (hist) {
        T m = T(0);
        for (int64_t c = 0; c < k; ++c) m += s.rnorm[c];
        hist[it] = m / (T)k;
      }
      *s.done = !(s_any && it < max_iters);
      s.counters[3] = 0;
    }
  }
}

// general P: <r, z> partials with z = P r already formed; last block: beta, stop test
template <class T>
__global__ void __launch_bounds__(256) k_gamma(const T* R, const T* Z, int64_t n, int64_t k, int max_iters, T* hist,
                                               CgScalars<T> s) {
  if (*s.done) return;
  __shared__ T smem[256];
  block_col_partials<T>(0, n, blockIdx.x, gridDim.x, k,
                        [&](int64_t i, int64_t c) { return R[i * k + c] * Z[i * k + c]; },
                        s.pB + (int64_t)blockIdx.x * k, smem);
  if (is_last_block(s.counters + 2)) {
    __shared__ int s_any;
    __shared__ T totB[kStage], red[32];
    stage_totals(s.pB, gridDim.x, k, totB, red);
    if (threadIdx.x == 0) s_any = 0;
    __syncthreads();
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
      const T g1 = total_at(s.pB, gridDim.x, k, c, totB);
      const T b = safe_div(g1, s.gamma[c]);
      s.beta[c] = s.conv[c] ? T(0) : b;
      s.gamma[c] = g1;
      if (s.rnorm[c] > s.tol_eff[c]) atomicOr(&s_any, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int it = *s.iters + 1;
      *s.iters = it;
      if (hist) {
        T m = T(0);
        for (int64_t c = 0; c < k; ++c) m += s.rnorm[c];
        hist[it] = m / (T)k;
      }
      *s.done = !(s_any && it < max_iters);
      s.counters[2] = 0;
    }
  }
}

// p = z + beta p   (z = r, dinv*r or Z)
// Skipped once `done` is set: p is not read after the last step.
template <class T, int PK>
__global__ void k_pupdate(T* P, const T* R, const T* Z, const T* dinv, int64_t n, int64_t k, CgScalars<T> s,
                          const int* done) {
  if (*done) return;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * k; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / k, c = u - i * k;
    const T r = R[u];
    const T z = PK == 0 ? r : (PK == 1 ? dinv[i] * r : Z[u]);
    P[u] = z + s.beta[c] * P[u];
  }
}

template <class T>
__global__ void k_scale_x(T* X, int64_t ldx, int64_t n, int64_t k, CgScalars<T> s) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * k; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / k, c = u - i * k;
    X[i * ldx + c] *= s.mult[c];
  }
}

// ---------------------------------------------------------------------------------------------
// fused persistent kernel

template <class T, class S>
struct FusedArgs {
  int kind;            // COLAGB_OP_DENSE or COLAGB_OP_CSR
  const S* vals;       // dense matrix or CSR values
  int64_t lda;
  const int32_t* indptr;
  const int32_t* indices;
  T shift;             // A + shift * I
  const T* dinv;       // Jacobi diagonal (PK == 1)
  const T* B;
  int64_t ldb;
  T* X;
  int64_t ldx;
  T* R;
  T* P;
  T* AP;
  int64_t n, k;
  double tol;
  int max_iters;
  int vec4;            // dense rows and the vector are 16-byte aligned and n % 4 == 0
  T* hist;
  CgScalars<T> s;
  GridBarrier gb;
};

// OUT[i, c] = shift * V[i, c] + (A V)[i, c] for the CTA's rows [r0, r1) and all k columns.
// CSR: one thread per (row, column) unit.  Dense: one warp per row, lanes stride the row
// (128-bit loads when the row is 16-byte aligned).  Ends with __syncthreads so the CTA can read
// OUT back.
template <class T, class S>
__device__ __forceinline__ void own_matvec(const FusedArgs<T, S>& a, const T* V, T* OUT, int64_t r0, int64_t r1) {
  const int64_t k = a.k, n = a.n;
  if (a.kind == COLAGB_OP_CSR) {
    for (int64_t u = threadIdx.x; u < (r1 - r0) * k; u += blockDim.x) {
      const int64_t i = r0 + u / k, c = u % k;
      T acc = a.shift * V[i * k + c];
      const int32_t b = a.indptr[i], e = a.indptr[i + 1];
      // entries in groups of four: indices and values, then the gathers, in flight together
      for (int32_t j0 = b; j0 < e; j0 += 4) {
        int32_t col[4];
        T v[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const bool ok = j0 + t < e;
          col[t] = ok ? a.indices[j0 + t] : 0;
          v[t] = ok ? cvt<T>(a.vals[j0 + t]) : T(0);
        }
        T x[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) x[t] = j0 + t < e ? V[(int64_t)col[t] * k + c] : T(0);
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (j0 + t < e) acc += v[t] * x[t];
      }
      OUT[i * k + c] = acc;
    }
  } else {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t i_rest = r0;
    if constexpr (std::is_same<S, float>::value && std::is_same<T, float>::value) {
      if (a.vec4 && k == 1) {
        // four rows per warp at a time: one vector load feeds four matrix-row loads, so each lane
        // keeps ~20 128-bit loads in flight (the row-at-a-time loop left the SM latency-bound);
        // each row's sum runs in the same order as the one-row loop below
        const float4* v4 = reinterpret_cast<const float4*>(V);
        const int64_t n4 = n / 4, l4 = a.lda / 4;
        const int64_t nfull = r0 + (r1 - r0) / 4 * 4;
        for (int64_t i = r0 + 4 * warp; i < nfull; i += 4 * nw) {
          const float4* ra = reinterpret_cast<const float4*>(a.vals + i * a.lda);
          float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
#pragma unroll 4
          for (int64_t j = lane; j < n4; j += 32) {
            const float4 vv = v4[j];
            const float4 q0 = ra[j], q1 = ra[l4 + j], q2 = ra[2 * l4 + j], q3 = ra[3 * l4 + j];
            c0 += q0.x * vv.x + q0.y * vv.y + q0.z * vv.z + q0.w * vv.w;
            c1 += q1.x * vv.x + q1.y * vv.y + q1.z * vv.z + q1.w * vv.w;
            c2 += q2.x * vv.x + q2.y * vv.y + q2.z * vv.z + q2.w * vv.w;
            c3 += q3.x * vv.x + q3.y * vv.y + q3.z * vv.z + q3.w * vv.w;
          }
          c0 = warp_sum(c0);
          c1 = warp_sum(c1);
          c2 = warp_sum(c2);
          c3 = warp_sum(c3);
          if (lane == 0) {
            OUT[i] = c0 + a.shift * V[i];
            OUT[i + 1] = c1 + a.shift * V[i + 1];
            OUT[i + 2] = c2 + a.shift * V[i + 2];
            OUT[i + 3] = c3 + a.shift * V[i + 3];
          }
        }
        i_rest = nfull;
      }
    }
    for (int64_t i = i_rest + warp; i < r1; i += nw) {
      const S* row = a.vals + i * a.lda;
      for (int64_t c = 0; c < k; ++c) {
        T acc = T(0);
        if constexpr (std::is_same<S, float>::value && std::is_same<T, float>::value) {
          if (a.vec4 && k == 1) {
            const float4* r4 = reinterpret_cast<const float4*>(row);
            const float4* v4 = reinterpret_cast<const float4*>(V);
            for (int64_t j = lane; j < n / 4; j += 32) {
              const float4 av = r4[j], vv = v4[j];
              acc += av.x * vv.x + av.y * vv.y + av.z * vv.z + av.w * vv.w;
            }
          } else {
            for (int64_t j = lane; j < n; j += 32) acc += row[j] * V[j * k + c];
          }
        } else {
          for (int64_t j = lane; j < n; j += 32) acc += cvt<T>(row[j]) * V[j * k + c];
        }
        acc = warp_sum(acc);
        if (lane == 0) OUT[i * k + c] = acc + a.shift * V[i * k + c];
      }
    }
  }
  __syncthreads();
}

// Every CTA computes the column totals itself from the per-CTA partials (same order everywhere).
template <class T>
__device__ __forceinline__ void all_totals(const T* partials, int nb, int64_t k, T* out_smem, T* red) {
  // block-parallel per column (k <= 64 on the fused path): every CTA forms the same totals
  for (int64_t c = 0; c < k; ++c) {
    const T v = block_total(partials, nb, k, c, red);
    if (threadIdx.x == 0) out_smem[c] = v;
  }
  __syncthreads();
}

// Barrier between the phases of the fused kernel: the cooperative grid's bounded software barrier,
// or -- when the whole grid is one thread-block cluster -- the hardware cluster barrier
// (release/acquire at cluster scope, global memory included).
template <bool CLUSTER>
__device__ __forceinline__ bool phase_sync(const GridBarrier& gb) {
  if constexpr (CLUSTER) {
    cooperative_groups::this_cluster().sync();
    return true;
  } else {
    return grid_sync(gb);
  }
}

// Cluster-wide sums of NQ values for the one-cluster fused kernel with a single right-hand side:
// warp shuffles, one block barrier, then lane r of warp 0 stores the CTA's sums into CTA r's shared
// memory (slot [q][rank]); after the cluster barrier (release / acquire) every CTA adds the 16 slots
// in rank order, so all CTAs hold the same totals and nothing is loaded from global memory or a peer
// on the critical path.  Two slot buffers alternate: a CTA can be at most one reduction ahead of
// another, because each reduction ends in a cluster barrier.
constexpr int kK1MaxCtas = 16;
template <int NQ, class T>
__device__ __forceinline__ void k1_cluster_sum(T (&v)[NQ], T* wsum, T* slots, int& buf) {
  namespace cgx = cooperative_groups;
  cgx::cluster_group cl = cgx::this_cluster();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int ncta = (int)cl.num_blocks(), rank = (int)cl.block_rank();
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) wsum[q * 32 + warp] = v[q];
  __syncthreads();
  T* sl = slots + buf * NQ * kK1MaxCtas;
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      T x = lane < nw ? wsum[q * 32 + lane] : T(0);
      v[q] = warp_sum(x);
    }
    if (lane < ncta)
#pragma unroll
      for (int q = 0; q < NQ; ++q) *cl.map_shared_rank(sl + q * kK1MaxCtas + rank, lane) = v[q];
  }
  cl.sync();
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    T tot = T(0);
    for (int r = 0; r < ncta; ++r) tot += sl[q * kK1MaxCtas + r];
    v[q] = tot;
  }
  buf ^= 1;
}

// The fused CG for one right-hand side on one thread-block cluster (<= 16 CTAs): the same algorithm,
// stop rule and history as the general body of k_cg_fused below (cg.py:94-178), with every inner
// product reduced by k1_cluster_sum -- two of them per step, <p, Ap> and (<r, z>, |r|^2) -- instead of
// per-CTA partials in global memory read back after the barrier.
template <class T, class S, int PK>
__device__ __forceinline__ void cg_fused_k1(const FusedArgs<T, S>& a, int64_t r0, int64_t r1) {
  __shared__ T wsum[2 * 32];
  __shared__ T slots[2 * 2 * kK1MaxCtas];
  int buf = 0;
  namespace cgx = cooperative_groups;
  cgx::cluster_group cl = cgx::this_cluster();
  const int t = threadIdx.x;
  auto z_of = [&](int64_t i, T r) { return PK == 0 ? r : a.dinv[i] * r; };
  // mult = |b|
  T q1[1] = {T(0)};
  for (int64_t i = r0 + t; i < r1; i += blockDim.x) {
    const T v = a.B[i * a.ldb];
    q1[0] += v * v;
  }
  k1_cluster_sum<1, T>(q1, wsum, slots, buf);
  const T mult = sqrt(q1[0]);
  // r = b / mult - A x0 (x0 through P)
  for (int64_t i = r0 + t; i < r1; i += blockDim.x) a.P[i] = a.X[i * a.ldx];
  cl.sync();
  own_matvec(a, a.P, a.AP, r0, r1);
  for (int64_t i = r0 + t; i < r1; i += blockDim.x) a.R[i] = safe_div(a.B[i * a.ldb], mult) - a.AP[i];
  cl.sync();  // every CTA is done reading x0 out of P
  T q2[2] = {T(0), T(0)};
  for (int64_t i = r0 + t; i < r1; i += blockDim.x) {
    const T r = a.R[i];
    const T z = z_of(i, r);
    a.P[i] = z;
    q2[0] += r * z;
    q2[1] += r * r;
  }
  k1_cluster_sum<2, T>(q2, wsum, slots, buf);  // also publishes P
  T gamma = q2[0];
  T rn = sqrt(q2[1]);
  const T tol_eff = (T)a.tol * rn + (T)a.tol;
  bool conv = rn < SmallValue<T>::v;
  if (blockIdx.x == 0 && t == 0 && a.hist) a.hist[0] = rn;
  int it = 0;
  bool running = rn > tol_eff && it < a.max_iters;
  while (running) {
    // A: Ap = A p, <p, Ap>
    own_matvec(a, a.P, a.AP, r0, r1);
    T qa[1] = {T(0)};
    for (int64_t i = r0 + t; i < r1; i += blockDim.x) qa[0] += a.P[i] * a.AP[i];
    k1_cluster_sum<1, T>(qa, wsum, slots, buf);
    const T alpha = conv ? T(0) : safe_div(gamma, qa[0]);
    // B: x, r updates, <r, z>, |r|^2
    T qb[2] = {T(0), T(0)};
    for (int64_t i = r0 + t; i < r1; i += blockDim.x) {
      const T p = a.P[i];
      a.X[i * a.ldx] += alpha * p;
      const T r = a.R[i] - alpha * a.AP[i];
      a.R[i] = r;
      qb[0] += r * z_of(i, r);
      qb[1] += r * r;
    }
    k1_cluster_sum<2, T>(qb, wsum, slots, buf);
    const T beta = conv ? T(0) : safe_div(qb[0], gamma);
    gamma = qb[0];
    rn = sqrt(qb[1]);
    conv = rn < SmallValue<T>::v;
    ++it;
    if (blockIdx.x == 0 && t == 0 && a.hist) a.hist[it] = rn;
    running = rn > tol_eff && it < a.max_iters;
    if (!running) break;
    // C: p = z + beta p
    for (int64_t i = r0 + t; i < r1; i += blockDim.x) a.P[i] = z_of(i, a.R[i]) + beta * a.P[i];
    cl.sync();
  }
  for (int64_t i = r0 + t; i < r1; i += blockDim.x) a.X[i * a.ldx] *= mult;
  if (blockIdx.x == 0 && t == 0) *a.s.iters = it;
}

template <class T, class S, int PK, bool CLUSTER>
__global__ void __launch_bounds__(CLUSTER ? 512 : 256) k_cg_fused(FusedArgs<T, S> a) {
  extern __shared__ unsigned char smem_raw[];
  T* red = reinterpret_cast<T*>(smem_raw);           // blockDim.x reduction slots
  T* tot1 = red + blockDim.x;                         // k column totals
  T* tot2 = tot1 + a.k;                               // k column totals
  T* alpha = tot2 + a.k;                              // k
  T* beta = alpha + a.k;                              // k
  T* gamma = beta + a.k;                              // k
  T* tol_eff = gamma + a.k;                           // k
  T* mult = tol_eff + a.k;                            // k
  int* conv = reinterpret_cast<int*>(mult + a.k);     // k
  __shared__ int s_any;

  const int64_t n = a.n, k = a.k;
  const int nb = gridDim.x;
  const int64_t rows_per_block = ceil_div(n, nb);
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = (r0 + rows_per_block < n) ? r0 + rows_per_block : n;
  const int64_t kc = k < 256 ? k : 256;
  if constexpr (CLUSTER) {
    if (k == 1 && gridDim.x <= kK1MaxCtas) {
      cg_fused_k1<T, S, PK>(a, r0, r1);
      return;
    }
  }
  T* pA = a.s.pA + (int64_t)blockIdx.x * k;
  T* pB = a.s.pB + (int64_t)blockIdx.x * k;
  T* pC = a.s.pC + (int64_t)blockIdx.x * k;
  (void)kc;

  // row-range iteration helper: f(i, c) over owned units, summed per column into `part`
  auto own_partials = [&](auto f, T* part) { block_col_partials<T>(r0, r1, 0, 1, k, f, part, red); };

  // ---- init: mult = |b| ----
  own_partials([&](int64_t i, int64_t c) { const T v = a.B[i * a.ldb + c]; return v * v; }, pA);
  if (!phase_sync<CLUSTER>(a.gb)) return;
  all_totals(a.s.pA, nb, k, tot1, red);
  for (int64_t c = threadIdx.x; c < k; c += blockDim.x) mult[c] = sqrt(tot1[c]);
  __syncthreads();
  // r = b / mult - A x0 (x0 gathered through P as scratch: P <- x0 first)
  for (int64_t i = r0; i < r1; ++i)
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) a.P[i * k + c] = a.X[i * a.ldx + c];
  if (!phase_sync<CLUSTER>(a.gb)) return;
  own_matvec(a, a.P, a.AP, r0, r1);
  for (int64_t u = threadIdx.x; u < (r1 - r0) * k; u += blockDim.x) {
    const int64_t i = r0 + u / k, c = u % k;
    a.R[i * k + c] = safe_div(a.B[i * a.ldb + c], mult[c]) - a.AP[i * k + c];
  }
  if (!phase_sync<CLUSTER>(a.gb)) return;  // everyone done reading x0 out of P
  own_partials([&](int64_t i, int64_t c) {
    const T r = a.R[i * k + c];
    const T z = PK == 0 ? r : a.dinv[i] * r;
    a.P[i * k + c] = z;
    return r * z;
  }, pB);
  own_partials([&](int64_t i, int64_t c) { const T r = a.R[i * k + c]; return r * r; }, pC);
  if (!phase_sync<CLUSTER>(a.gb)) return;
  all_totals(a.s.pB, nb, k, tot1, red);
  all_totals(a.s.pC, nb, k, tot2, red);
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
    gamma[c] = tot1[c];
    const T rn = sqrt(tot2[c]);
    tot2[c] = rn;
    tol_eff[c] = (T)a.tol * rn + (T)a.tol;
    conv[c] = rn < SmallValue<T>::v;
    if (rn > tol_eff[c]) atomicOr(&s_any, 1);
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0 && a.hist) {
    T m = T(0);
    for (int64_t c = 0; c < k; ++c) m += tot2[c];
    a.hist[0] = m / (T)k;
  }
  int it = 0;
  bool running = s_any && it < a.max_iters;
  __syncthreads();

  while (running) {
    // ---- phase A: Ap = A p, <p, Ap> ----
    own_matvec(a, a.P, a.AP, r0, r1);
    own_partials([&](int64_t i, int64_t c) { return a.P[i * k + c] * a.AP[i * k + c]; }, pA);
    if (!phase_sync<CLUSTER>(a.gb)) return;
    all_totals(a.s.pA, nb, k, tot1, red);
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) alpha[c] = conv[c] ? T(0) : safe_div(gamma[c], tot1[c]);
    __syncthreads();
    // ---- phase B: x, r updates, <r, z>, |r|^2 ----
    own_partials([&](int64_t i, int64_t c) {
      const T al = alpha[c];
      a.X[i * a.ldx + c] += al * a.P[i * k + c];
      const T r = a.R[i * k + c] - al * a.AP[i * k + c];
      a.R[i * k + c] = r;
      return r * r;
    }, pC);
    own_partials([&](int64_t i, int64_t c) {
      const T r = a.R[i * k + c];
      return r * (PK == 0 ? r : a.dinv[i] * r);
    }, pB);
    if (!phase_sync<CLUSTER>(a.gb)) return;
    all_totals(a.s.pB, nb, k, tot1, red);
    all_totals(a.s.pC, nb, k, tot2, red);
    if (threadIdx.x == 0) s_any = 0;
    __syncthreads();
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
      const T g1 = tot1[c];
      beta[c] = conv[c] ? T(0) : safe_div(g1, gamma[c]);
      gamma[c] = g1;
      const T rn = sqrt(tot2[c]);
      tot2[c] = rn;
      conv[c] = rn < SmallValue<T>::v;
      if (rn > tol_eff[c]) atomicOr(&s_any, 1);
    }
    __syncthreads();
    ++it;
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.hist) {
      T m = T(0);
      for (int64_t c = 0; c < k; ++c) m += tot2[c];
      a.hist[it] = m / (T)k;
    }
    running = s_any && it < a.max_iters;
    __syncthreads();
    if (!running) break;
    // ---- phase C: p = z + beta p ----
    for (int64_t u = threadIdx.x; u < (r1 - r0) * k; u += blockDim.x) {
      const int64_t i = r0 + u / k, c = u % k;
      const T r = a.R[i * k + c];
      const T z = PK == 0 ? r : a.dinv[i] * r;
      a.P[i * k + c] = z + beta[c] * a.P[i * k + c];
    }
    if (!phase_sync<CLUSTER>(a.gb)) return;
  }
  // ---- x *= mult ----
  for (int64_t u = threadIdx.x; u < (r1 - r0) * k; u += blockDim.x) {
    const int64_t i = r0 + u / k, c = u % k;
    a.X[i * a.ldx + c] *= mult[c];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.s.iters = it;
}

// ---------------------------------------------------------------------------------------------
// host side

struct CgPlan {
  int64_t n = 0, k = 0;
  int nb = 1;          // blocks of the generic kernels
  int pk = 0;          // 0 identity, 1 diagonal (fused into the kernels), 2 general operator
  const colagb_op_node* pdiag = nullptr;
  bool fused_ok = false;
  FusedForm ff;
  int fused_blocks = 0;
};

template <class T>
static CgScalars<T> carve(Bump& ws, int64_t k, int nb) {
  CgScalars<T> s;
  s.mult = ws.take<T>(k);
  s.tol_eff = ws.take<T>(k);
  s.gamma = ws.take<T>(k);
  s.alpha = ws.take<T>(k);
  s.beta = ws.take<T>(k);
  s.rnorm = ws.take<T>(k);
  s.conv = ws.take<int>(k);
  s.done = ws.take<int>(4);
  s.iters = ws.take<int>(4);
  s.pA = ws.take<T>((size_t)nb * k);
  s.pB = ws.take<T>((size_t)nb * k);
  s.pC = ws.take<T>((size_t)nb * k);
  s.counters = ws.take<unsigned int>(8);
  return s;
}

static int generic_blocks(int64_t n, int64_t k) {
  const int64_t want = ceil_div(n * k, 1024);
  const int64_t cap = (int64_t)num_sms() * 4;
  return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

template <class T, class S, int PK>
static int fused_blocks_for() {
  int occ = 0;
  const size_t smem = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cg_fused<T, S, PK, false>, 256, smem);
  if (occ < 1) occ = 1;
  return num_sms() * (occ < 2 ? occ : 2);
}

static int plan_cg(const colagb_op* A, const colagb_op* P, int64_t k, CgPlan& pl) {
  const colagb_op_node& r = A->nodes[A->root];
  if (r.rows != r.cols) return fail(COLAGB_ERR_INVALID, "CG needs a square operator");
  pl.n = r.rows;
  pl.k = k;
  pl.nb = generic_blocks(pl.n, k);
  pl.pk = 0;
  if (P) {
    const colagb_op_node& pr = P->nodes[P->root];
    if (pr.rows != pl.n || pr.cols != pl.n) return fail(COLAGB_ERR_INVALID, "preconditioner shape mismatch");
    if (P->compute_dtype != A->compute_dtype)
      return fail(COLAGB_ERR_INVALID, "preconditioner and operator compute types differ");
    if (pr.kind == COLAGB_OP_IDENTITY) pl.pk = 0;
    else if (pr.kind == COLAGB_OP_DIAG &&
             (pr.dtype == A->compute_dtype)) { pl.pk = 1; pl.pdiag = &pr; }
    else pl.pk = 2;
  }
  pl.ff = fused_form(A);
  pl.fused_ok = pl.ff.ok && pl.pk != 2 && k <= 64 && pl.n > 0 &&
                (pl.ff.leaf->kind == COLAGB_OP_CSR || k <= 8) &&
                (pl.ff.leaf->dtype == A->compute_dtype || pl.ff.leaf->dtype == COLAGB_BF16);
  return COLAGB_OK;
}

// Carves the solver's buffers out of ws; fails when an operator's own workspace cannot be sized.
template <class T>
static int cg_ws(const colagb_op* A, const colagb_op* P, const CgPlan& pl, Bump& ws, CgScalars<T>* out,
                 T** R, T** Pv, T** AP, T** Z, T** hist_dummy, void** opws, size_t* opws_bytes) {
  const int64_t n = pl.n, k = pl.k;
  CgScalars<T> s = carve<T>(ws, k, pl.nb > pl.fused_blocks ? pl.nb : pl.fused_blocks);
  *R = ws.take<T>(n * k);
  *Pv = ws.take<T>(n * k);
  *AP = ws.take<T>(n * k);
  *Z = pl.pk == 2 ? ws.take<T>(n * k) : nullptr;
  (void)hist_dummy;
  size_t a_b = 0, p_b = 0;
  COLAGB_TRY(colagb_matmat_workspace_bytes(A, k, &a_b));
  if (P && pl.pk == 2) COLAGB_TRY(colagb_matmat_workspace_bytes(P, k, &p_b));
  *opws_bytes = a_b > p_b ? a_b : p_b;
  *opws = ws.take<char>(*opws_bytes > 0 ? *opws_bytes : 1);
  if (out) *out = s;
  return COLAGB_OK;
}

template <class T>
static int run_generic(const colagb_op* A, const colagb_op* P, const CgPlan& pl, const T* B, int64_t ldb, T* X,
                       int64_t ldx, const colagb_cg_params& prm, T* hist, CgScalars<T> s, T* R, T* Pv, T* AP, T* Z,
                       void* opws, size_t opws_bytes, colagb_cg_result* res, cudaStream_t st) {
  const int64_t n = pl.n, k = pl.k;
  const int nb = pl.nb;
  const T* dinv = pl.pk == 1 ? static_cast<const T*>(pl.pdiag->data) : nullptr;
  const int eg = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n * k, 256), 1), (int64_t)num_sms() * 8);
  COLAGB_CUDA(cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned int), st));
  k_colnorm_b<T><<<nb, 256, 0, st>>>(B, ldb, n, k, s);
  k_scale_b<T><<<eg, 256, 0, st>>>(B, ldb, R, n, k, s);
  COLAGB_CUDA(cudaGetLastError());
  {
    Bump w(opws, opws_bytes);
    COLAGB_TRY(op_apply<T>(A, A->root, X, ldx, 0, R, k, 0, k, 1, T(-1), T(1), w, nullptr, st));
  }
  if (pl.pk == 2) {
    Bump w(opws, opws_bytes);
    COLAGB_TRY(op_apply<T>(P, P->root, R, k, 0, Z, k, 0, k, 1, T(1), T(0), w, nullptr, st));
  }
  switch (pl.pk) {
    case 0: k_init<T, 0><<<nb, 256, 0, st>>>(R, Z, dinv, Pv, n, k, prm.tol, prm.max_iters, hist, s); break;
    case 1: k_init<T, 1><<<nb, 256, 0, st>>>(R, Z, dinv, Pv, n, k, prm.tol, prm.max_iters, hist, s); break;
    default: k_init<T, 2><<<nb, 256, 0, st>>>(R, Z, dinv, Pv, n, k, prm.tol, prm.max_iters, hist, s); break;
  }
  COLAGB_CUDA(cudaGetLastError());
  int h_done[2] = {0, 0};
  const int every = prm.check_every > 0 ? prm.check_every : 16;
  // One step of the loop: Ap, alpha, x / r update (+ z = P r and gamma for a general P), p update.
  // Every kernel reads the device stop flag and does nothing once it is set, so a block of steps may
  // run past convergence or max_iters (the device counts the steps and enforces max_iters).
  auto enqueue_steps = [&](cudaStream_t q, int nsteps) -> int {
    for (int j = 0; j < nsteps; ++j) {
      Bump w(opws, opws_bytes);
      COLAGB_TRY(op_apply<T>(A, A->root, Pv, k, 0, AP, k, 0, k, 1, T(1), T(0), w, s.done, q));
      k_alpha<T><<<nb, 256, 0, q>>>(Pv, AP, n, k, s);
      switch (pl.pk) {
        case 0: k_update<T, 0><<<nb, 256, 0, q>>>(X, ldx, R, Pv, AP, dinv, n, k, prm.max_iters, hist, s); break;
        case 1: k_update<T, 1><<<nb, 256, 0, q>>>(X, ldx, R, Pv, AP, dinv, n, k, prm.max_iters, hist, s); break;
        default: {
          k_update<T, 2><<<nb, 256, 0, q>>>(X, ldx, R, Pv, AP, dinv, n, k, prm.max_iters, hist, s);
          Bump w2(opws, opws_bytes);
          COLAGB_TRY(op_apply<T>(P, P->root, R, k, 0, Z, k, 0, k, 1, T(1), T(0), w2, s.done, q));
          k_gamma<T><<<nb, 256, 0, q>>>(R, Z, n, k, prm.max_iters, hist, s);
        }
      }
      // p update runs only when the step did not finish the loop (done flag now set => skip)
      switch (pl.pk) {
        case 0: k_pupdate<T, 0><<<eg, 256, 0, q>>>(Pv, R, Z, dinv, n, k, s, s.done); break;
        case 1: k_pupdate<T, 1><<<eg, 256, 0, q>>>(Pv, R, Z, dinv, n, k, s, s.done); break;
        default: k_pupdate<T, 2><<<eg, 256, 0, q>>>(Pv, R, Z, dinv, n, k, s, s.done); break;
      }
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return check_cuda(e, "cg step launch");
    }
    return COLAGB_OK;
  };
  // The loop's launch block of `every` steps has the same arguments every time (all state lives on
  // the device), so it is captured once as a CUDA graph and replayed: one launch per block instead of
  // four to six per step.  Falls back to plain launches when capture is not possible.
  cudaGraphExec_t exec = nullptr;
  if (prm.graph == 0 && prm.max_iters >= 2 * every) {
    cudaStream_t cs = capture_stream();
    if (cs && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int sb = enqueue_steps(cs, every);
      cudaGraph_t g = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(cs, &g);
      if (sb == COLAGB_OK && ee == cudaSuccess && g) {
        if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) exec = nullptr;
      }
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
    } else {
      cudaGetLastError();
    }
  }
  int launched = 0;
  int status = COLAGB_OK;
  while (true) {
    if (exec) {
      cudaError_t e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) { status = check_cuda(e, "cg graph launch"); break; }
      launched += every;
    } else {
      const int nsteps = std::min(every, prm.max_iters - launched);
      status = enqueue_steps(st, nsteps);
      if (status != COLAGB_OK) break;
      launched += nsteps;
    }
    cudaError_t e = cudaMemcpyAsync(h_done, s.done, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { status = check_cuda(e, "cg poll"); break; }
    if (h_done[0] || launched >= prm.max_iters) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  res->graph = exec != nullptr ? 1 : 0;
  if (status != COLAGB_OK) return status;
  k_scale_x<T><<<eg, 256, 0, st>>>(X, ldx, n, k, s);
  COLAGB_CUDA(cudaGetLastError());
  int it = 0;
  COLAGB_CUDA(cudaMemcpyAsync(&it, s.iters, sizeof(int), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaStreamSynchronize(st));
  res->iterations = it;
  res->fused = 0;
  res->status = COLAGB_OK;
  return COLAGB_OK;
}

// Step count and barrier status of a finished fused solve.
template <class T>
static int finish_fused(const CgScalars<T>& s, colagb_cg_result* res, cudaStream_t st) {
  int h[2] = {0, 0};
  COLAGB_CUDA(cudaMemcpyAsync(&h[0], s.iters, sizeof(int), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaMemcpyAsync(&h[1], s.counters + 6, sizeof(int), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaStreamSynchronize(st));
  res->iterations = h[0];
  res->fused = 1;
  res->graph = 0;
  res->status = h[1];
  if (h[1] != 0) return fail(COLAGB_ERR_TIMEOUT, "fused CG: a grid barrier timed out");
  return COLAGB_OK;
}

template <class T, class S, int PK>
static int run_fused(const CgPlan& pl, const T* B, int64_t ldb, T* X, int64_t ldx, const colagb_cg_params& prm, T* hist,
                     CgScalars<T> s, T* R, T* Pv, T* AP, colagb_cg_result* res, cudaStream_t st) {
  FusedArgs<T, S> a;
  const colagb_op_node* leaf = pl.ff.leaf;
  a.kind = leaf->kind;
  a.vals = static_cast<const S*>(leaf->data);
  a.lda = leaf->ld;
  a.indptr = leaf->indptr;
  a.indices = leaf->indices;
  a.shift = (T)pl.ff.shift;
  a.dinv = PK == 1 ? static_cast<const T*>(pl.pdiag->data) : nullptr;
  a.B = B;
  a.ldb = ldb;
  a.X = X;
  a.ldx = ldx;
  a.R = R;
  a.P = Pv;
  a.AP = AP;
  a.n = pl.n;
  a.k = pl.k;
  a.tol = prm.tol;
  a.max_iters = prm.max_iters;
  a.hist = hist;
  a.vec4 = leaf->kind == COLAGB_OP_DENSE && (pl.n % 4 == 0) && (leaf->ld % 4 == 0) &&
           ((uintptr_t)leaf->data % 16 == 0) && ((uintptr_t)Pv % 16 == 0);
  a.s = s;
  a.gb.count = s.counters + 4;
  a.gb.generation = s.counters + 5;
  a.gb.err = reinterpret_cast<int*>(s.counters + 6);
  a.gb.spin_limit = prm.spin_limit > 0 ? prm.spin_limit : kDefaultSpinLimit;
  const size_t smem = 256 * sizeof(T) + 7 * (size_t)pl.k * sizeof(T) + (size_t)pl.k * sizeof(int);
  const size_t smem512 = smem + 256 * sizeof(T);  // the cluster variant runs 512 threads per CTA
  // An operator of at most ~32 MB is streamed from L2 by one 16-CTA cluster faster than the whole
  // grid can pass three software grid barriers per step (measured: 2048 x 2048 FP32, ~24 us per step
  // on 64 CTAs); larger operators use the cooperative grid (HBM-bound).
  const double abytes0 = leaf->kind == COLAGB_OP_DENSE ? (double)leaf->rows * (double)leaf->cols * sizeof(S)
                                                       : (double)leaf->nnz * (double)(sizeof(S) + 4);
  if (abytes0 <= 32.0 * 1024 * 1024 && pl.fused_blocks >= 16) {
    a.gb.nblocks = 16;
    COLAGB_CUDA(cudaFuncSetAttribute(k_cg_fused<T, S, PK, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = smem512;
    cfg.stream = st;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, k_cg_fused<T, S, PK, true>, &cfg) == cudaSuccess && ncl >= 1) {
      COLAGB_CUDA(cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned int), st));
      COLAGB_CUDA(cudaLaunchKernelEx(&cfg, k_cg_fused<T, S, PK, true>, a));
      return finish_fused(s, res, st);
    }
    cudaGetLastError();
  }
  int occ = 0;
  COLAGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cg_fused<T, S, PK, false>, 256, smem));
  if (occ < 1) return fail(COLAGB_ERR_UNSUPPORTED, "fused CG kernel cannot be resident");
  // Grid sized to the operator: ~256 KB of matrix per CTA (at least 16 CTAs).  Every step ends in
  // three grid barriers whose arrivals are atomics on one word, so a CTA with only a few rows of a
  // small matrix costs more in barrier time than it saves in streaming time (n = 2048 dense: 64
  // CTAs instead of two per SM).
  const int nb_max = num_sms() * (occ < 2 ? occ : 2);
  const double abytes = leaf->kind == COLAGB_OP_DENSE ? (double)leaf->rows * (double)leaf->cols * sizeof(S)
                                                      : (double)leaf->nnz * (double)(sizeof(S) + 4);
  const double want = abytes / (256.0 * 1024.0);
  const int nb = (int)(want < 16.0 ? 16.0 : (want > (double)nb_max ? (double)nb_max : want + 0.999));
  if (nb > pl.fused_blocks) return fail(COLAGB_ERR_WORKSPACE, "fused CG block count exceeds planned partials");
  a.gb.nblocks = (unsigned)nb;
  COLAGB_CUDA(cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned int), st));
  void* args[] = {&a};
  COLAGB_CUDA(cudaLaunchCooperativeKernel((const void*)k_cg_fused<T, S, PK, false>, dim3(nb), dim3(256), args, smem, st));
  return finish_fused(s, res, st);
}

template <class T>
static int cg_solve_t(const colagb_op* A, const colagb_op* P, const void* Bv, int64_t ldb, void* Xv, int64_t ldx,
                      int64_t k, const colagb_cg_params& prm, void* histv, void* workspace, size_t ws_bytes,
                      colagb_cg_result* res, cudaStream_t st) {
  CgPlan pl;
  COLAGB_TRY(plan_cg(A, P, k, pl));
  pl.fused_blocks = num_sms() * 2;
  Bump ws(workspace, ws_bytes);
  CgScalars<T> s;
  T *R, *Pv, *AP, *Z, *hd;
  void* opws;
  size_t opws_b;
  COLAGB_TRY(cg_ws<T>(A, P, pl, ws, &s, &R, &Pv, &AP, &Z, &hd, &opws, &opws_b));
  if (ws.overflow() || workspace == nullptr)
    return fail(COLAGB_ERR_WORKSPACE, "colagb_cg_solve: workspace too small (need " + std::to_string(ws.peak) + ")");
  const T* B = static_cast<const T*>(Bv);
  T* X = static_cast<T*>(Xv);
  T* hist = static_cast<T*>(histv);
  if (pl.n == 0 || k == 0) {
    res->iterations = 0;
    res->graph = 0;
    res->fused = 0;
    res->status = COLAGB_OK;
    return COLAGB_OK;
  }
  if (prm.allow_fused && pl.fused_ok) {
    const int sd = pl.ff.leaf->dtype;
    if (sd == COLAGB_BF16) {
      return pl.pk == 0 ? run_fused<T, __nv_bfloat16, 0>(pl, B, ldb, X, ldx, prm, hist, s, R, Pv, AP, res, st)
                        : run_fused<T, __nv_bfloat16, 1>(pl, B, ldb, X, ldx, prm, hist, s, R, Pv, AP, res, st);
    }
    return pl.pk == 0 ? run_fused<T, T, 0>(pl, B, ldb, X, ldx, prm, hist, s, R, Pv, AP, res, st)
                      : run_fused<T, T, 1>(pl, B, ldb, X, ldx, prm, hist, s, R, Pv, AP, res, st);
  }
  return run_generic<T>(A, P, pl, B, ldb, X, ldx, prm, hist, s, R, Pv, AP, Z, opws, opws_b, res, st);
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_cg_workspace_bytes(const colagb_op* A, const colagb_op* P, int64_t k, size_t* bytes) {
  if (!A || !bytes || k < 0) return fail(COLAGB_ERR_INVALID, "colagb_cg_workspace_bytes: bad arguments");
  CgPlan pl;
  COLAGB_TRY(plan_cg(A, P, k, pl));
  pl.fused_blocks = num_sms() * 2;
  Bump ws = Bump::measuring();
  void* opws;
  size_t ob;
  if (A->compute_dtype == COLAGB_F64) {
    double *R, *Pv, *AP, *Z, *h;
    COLAGB_TRY(cg_ws<double>(A, P, pl, ws, nullptr, &R, &Pv, &AP, &Z, &h, &opws, &ob));
  } else {
    float *R, *Pv, *AP, *Z, *h;
    COLAGB_TRY(cg_ws<float>(A, P, pl, ws, nullptr, &R, &Pv, &AP, &Z, &h, &opws, &ob));
  }
  *bytes = ws.peak;
  return COLAGB_OK;
}

extern "C" int colagb_cg_solve(const colagb_op* A, const colagb_op* P, const void* B, int64_t ldb, void* X,
                               int64_t ldx, int64_t k, const colagb_cg_params* params, void* residual_history,
                               void* workspace, size_t workspace_bytes, colagb_cg_result* result, void* stream) {
  if (!A || !params || !result) return fail(COLAGB_ERR_INVALID, "colagb_cg_solve: null argument");
  if (k < 0 || ldb < k || ldx < k) return fail(COLAGB_ERR_INVALID, "colagb_cg_solve: bad k / leading dimensions");
  if (params->max_iters < 0) return fail(COLAGB_ERR_INVALID, "colagb_cg_solve: max_iters < 0");
  const int64_t n = A->nodes[A->root].rows;
  if (n * k > 0 && (!B || !X)) return fail(COLAGB_ERR_INVALID, "colagb_cg_solve: null B/X");
  cudaStream_t st = as_stream(stream);
  if (A->compute_dtype == COLAGB_F64)
    return cg_solve_t<double>(A, P, B, ldb, X, ldx, k, *params, residual_history, workspace, workspace_bytes, result, st);
  return cg_solve_t<float>(A, P, B, ldb, X, ldx, k, *params, residual_history, workspace, workspace_bytes, result, st);
}

// ---------------------------------------------------------------------------------------------
// CG without any allocation, for callers that cannot allocate device memory themselves (for example
// a host runtime that owns a fixed memory pool, or a driver calling from a context where
// cudaMalloc is not allowed).  The solver's scratch lives in one file-scope device array of
// kNoAllocScratchBytes that every GPU loading this library holds until the process exits.
namespace colagb {
constexpr size_t kNoAllocScratchBytes = (size_t)8 << 20;  // 8 MiB
static __device__ __align__(256) unsigned char g_cg_noalloc_scratch[kNoAllocScratchBytes];

// The array's device address belongs to a CUDA context, not to a device: a caller that pushes its
// own driver context, or a cudaDeviceReset, makes the runtime load the library's module again at
// another address.  So the address is looked up once per context (keyed on the driver's unique
// context id, reached through the runtime's driver entry points without linking libcuda) and cached.
// Device address of the scratch array in the calling thread's current context.
static int noalloc_scratch(void** out) {
  static std::mutex mu;
  static std::vector<std::pair<unsigned long long, void*>> addr;  // (context id, address)
  unsigned long long id = current_context_id();
  if (id == 0) {
    // no context current yet (or no driver entry points): the lookup itself makes the device's
    // primary context current; cache under that context when its id can be read
    COLAGB_CUDA(cudaGetSymbolAddress(out, g_cg_noalloc_scratch));
    id = current_context_id();
    if (id == 0) return COLAGB_OK;
    std::lock_guard<std::mutex> lk(mu);
    addr.emplace_back(id, *out);
    return COLAGB_OK;
  }
  std::lock_guard<std::mutex> lk(mu);
  for (const auto& e : addr)
    if (e.first == id) {
      *out = e.second;
      return COLAGB_OK;
    }
  void* p = nullptr;
  COLAGB_CUDA(cudaGetSymbolAddress(&p, g_cg_noalloc_scratch));
  addr.emplace_back(id, p);
  *out = p;
  return COLAGB_OK;
}
}  // namespace colagb

extern "C" int colagb_cg_solve_noalloc(const colagb_op* A, const colagb_op* P, const void* B, int64_t ldb, void* X,
                                       int64_t ldx, int64_t k, const colagb_cg_params* params, void* residual_history,
                                       colagb_cg_result* result, void* stream) {
  if (!A || !params || !result) return fail(COLAGB_ERR_INVALID, "colagb_cg_solve_noalloc: null argument");
  size_t need = 0;
  COLAGB_TRY(colagb_cg_workspace_bytes(A, P, k, &need));
  if (need > kNoAllocScratchBytes)
    return fail(COLAGB_ERR_INVALID, "colagb_cg_solve_noalloc: this problem needs " + std::to_string(need) +
                                        " bytes of scratch, more than the fixed " +
                                        std::to_string(kNoAllocScratchBytes) + " bytes; use colagb_cg_solve");
  void* scratch = nullptr;
  COLAGB_TRY(noalloc_scratch(&scratch));
  // every buffer the solver reads is written or cleared by the solver itself before use
  return colagb_cg_solve(A, P, B, ldb, X, ldx, k, params, residual_history, scratch, kNoAllocScratchBytes, result,
                         stream);
}
