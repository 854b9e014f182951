// Operator-program runtime and the structured matvec kernels (Dense, Sparse CSR, Diagonal,
// ScalarMul/Identity, and the Sum / Product / Kronecker / BlockDiag compositions).
//
// Reference behaviour (cola/ops/operators.py):
//   Dense._matmat      :26-28   A @ X
//   Sparse._matmat     :77-78   CSR @ X
//   ScalarMul._matmat  :97-98   c * X
//   Identity._matmat   :122-123 X
//   Product._matmat    :153-156 right-to-left chain
//   Sum._matmat        :182-183 sum of child products
//   Kronecker._matmat  :216-223 one contraction per factor along its own axis
//   BlockDiag._matmat  :299-310 each block (times its multiplicity) on its row slice
//   Diagonal._matmat   :338-339 d[:, None] * X
// Kronecker factors are applied as strided-batched contractions on the (pre, c_i, post*k) view,
// so no moveaxis copy is materialised.
#include <mutex>
#include <type_traits>
#include <string>
#include <vector>

#include "common.cuh"
#include "ops.cuh"

namespace colagb {

// --------------------------------------------------------------------------------------------
// error state
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}
int check_cuda(cudaError_t e, const char* what) {
  return fail(COLAGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int num_sms() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = v > 0 ? v : 1;
  }
  return cache[dev];
}

// --------------------------------------------------------------------------------------------
// leaf kernels

template <class T>
__device__ __forceinline__ T combine(T acc, T alpha, T beta, const T* y) {
  return beta == T(0) ? alpha * acc : alpha * acc + beta * (*y);
}

// Dense, few columns (k <= 4): one warp per output row, lanes stride over the row.
template <class T, class S, int K>
__global__ void __launch_bounds__(256) dense_gemv_kernel(const S* __restrict__ A, int64_t lda, int64_t rows,
                                                         int64_t cols, const T* __restrict__ X, int64_t ldx,
                                                         int64_t bsx, T* __restrict__ Y, int64_t ldy,
                                                         int64_t bsy, T alpha, T beta, const int* skip) {
  if (skip && *skip) return;
  const int64_t b = blockIdx.y;
  X += b * bsx;
  Y += b * bsy;
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= rows) return;
  const S* a = A + row * lda;
  T acc[K];
#pragma unroll
  for (int c = 0; c < K; ++c) acc[c] = T(0);
  for (int64_t j = lane; j < cols; j += 32) {
    const T av = cvt<T>(a[j]);
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] += av * X[j * ldx + c];
  }
#pragma unroll
  for (int c = 0; c < K; ++c) {
    const T s = warp_sum(acc[c]);
    if (lane == 0) Y[row * ldy + c] = combine(s, alpha, beta, Y + row * ldy + c);
  }
}

// Dense, many columns: 64x64 output tile, 16-deep k-slices through shared memory,
// 256 threads each owning a 4x4 micro-tile.  blockIdx.z = batch.
template <class T, class S>
__global__ void __launch_bounds__(256) dense_gemm_kernel(const S* __restrict__ A, int64_t lda, int64_t M,
                                                         int64_t K, const T* __restrict__ X, int64_t ldx,
                                                         int64_t bsx, T* __restrict__ Y, int64_t ldy,
                                                         int64_t bsy, int64_t N, T alpha, T beta,
                                                         const int* skip) {
  if (skip && *skip) return;
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ T As[BK][BM + 1];
  __shared__ T Xs[BK][BN];
  const int64_t b = blockIdx.z;
  X += b * bsx;
  Y += b * bsy;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    // A tile: BM x BK, 1024 elements, 4 per thread
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = threadIdx.x + r * 256;
      const int mm = idx / BK, kk = idx % BK;
      const int64_t gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? cvt<T>(A[gm * lda + gk]) : T(0);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = threadIdx.x + r * 256;
      const int kk = idx / BN, nn = idx % BN;
      const int64_t gk = k0 + kk, gn = n0 + nn;
      Xs[kk][nn] = (gk < K && gn < N) ? X[gk * ldx + gn] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T av[4], xv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) xv[j] = Xs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += av[i] * xv[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gn = n0 + tx * 4 + j;
      if (gn < N) Y[gm * ldy + gn] = combine(acc[i][j], alpha, beta, Y + gm * ldy + gn);
    }
  }
}

// CSR, one column: TPR lanes per row, lanes stride over the row's entries.
template <class T, class S, int TPR>
__global__ void __launch_bounds__(256) csr_spmv_kernel(const int32_t* __restrict__ indptr,
                                                       const int32_t* __restrict__ indices,
                                                       const S* __restrict__ vals, int64_t rows,
                                                       const T* __restrict__ X, int64_t ldx, int64_t bsx,
                                                       T* __restrict__ Y, int64_t ldy, int64_t bsy, T alpha,
                                                       T beta, const int32_t* __restrict__ operm, const int* skip) {
  if (skip && *skip) return;
  const int64_t b = blockIdx.y;
  X += b * bsx;
  Y += b * bsy;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = gt / TPR;
  const int sub = (int)(gt % TPR);
  T acc = T(0);
  if (row < rows) {
    const int32_t beg = indptr[row], end = indptr[row + 1];
    for (int32_t j = beg + sub; j < end; j += TPR) acc += cvt<T>(vals[j]) * X[(int64_t)indices[j] * ldx];
  }
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (row < rows && sub == 0) {
    const int64_t orow = operm ? (int64_t)operm[row] : row;  // a permuted node writes row perm[row]
    Y[orow * ldy] = combine(acc, alpha, beta, Y + orow * ldy);
  }
}

// CSR, one column, short rows ("CSR-stream"): one warp per group of 32 consecutive rows.  The group's
// nonzeros are one contiguous span [beg, end) of the index and value arrays: the warp streams it with
// 128-bit loads (4 entries per lane per pass, two passes in flight), gathers the four x entries of
// each load independently, and parks the products in shared memory; lane r then sums row r's
// products in entry order.  A group whose span exceeds the buffer is done row by row, lanes striding
// over the row.  On a graph with unordered columns the x gathers are scattered L2 sectors; this keeps
// ~8 of them in flight per lane instead of one dependent index -> x chain per entry.
constexpr int kStreamWarps = 8;
template <class T> struct StreamCap { static constexpr int value = 4096 / (int)sizeof(T); };

template <class T, class S> struct Load4;
template <class T> struct Load4<T, float> {
  __device__ static void run(const float* p, T v[4]) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = T(q.x); v[1] = T(q.y); v[2] = T(q.z); v[3] = T(q.w);
  }
};
template <class T> struct Load4<T, double> {
  __device__ static void run(const double* p, T v[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p)), b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    v[0] = T(a.x); v[1] = T(a.y); v[2] = T(b.x); v[3] = T(b.y);
  }
};
template <class T> struct Load4<T, __nv_bfloat16> {
  __device__ static void run(const __nv_bfloat16* p, T v[4]) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
    const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.x));
    const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.y));
    v[0] = T(a.x); v[1] = T(a.y); v[2] = T(b.x); v[3] = T(b.y);
  }
};

// entries base .. base+3 (those inside [beg, end)) -> their products val * x[col]; others 0
template <class T, class S, bool VEC>
__device__ __forceinline__ void stream_pass(const int32_t* __restrict__ indices, const S* __restrict__ vals,
                                            int64_t nnz, int32_t beg, int32_t end, int64_t base,
                                            const T* __restrict__ X, int64_t ldx, T pr[4]) {
  int32_t id[4];
  T v[4];
  if (base >= end) {
#pragma unroll
    for (int c = 0; c < 4; ++c) pr[c] = T(0);
    return;
  }
  if (VEC && base + 3 < nnz) {
    const int4 q = __ldg(reinterpret_cast<const int4*>(indices + base));
    id[0] = q.x; id[1] = q.y; id[2] = q.z; id[3] = q.w;
    Load4<T, S>::run(vals + base, v);
  } else {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int64_t e = base + c;
      const bool ok = e >= beg && e < end;
      id[c] = ok ? indices[e] : 0;
      v[c] = ok ? cvt<T>(vals[e]) : T(0);
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int64_t e = base + c;
    pr[c] = (e >= beg && e < end) ? v[c] * X[(int64_t)id[c] * ldx] : T(0);
  }
}

template <class T, class S, bool VEC>
__global__ void __launch_bounds__(kStreamWarps * 32) csr_stream_kernel(
    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, const S* __restrict__ vals,
    int64_t rows, int64_t nnz, const T* __restrict__ X, int64_t ldx, int64_t bsx, T* __restrict__ Y, int64_t ldy,
    int64_t bsy, T alpha, T beta, const int32_t* __restrict__ operm, const int* skip) {
  constexpr int CAP = StreamCap<T>::value;
  __shared__ T prod[kStreamWarps][CAP];
  if (skip && *skip) return;
  const int64_t b = blockIdx.y;
  X += b * bsx;
  Y += b * bsy;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t r0 = ((int64_t)blockIdx.x * kStreamWarps + w) * 32;
  if (r0 >= rows) return;  // the whole warp leaves; nothing below synchronises beyond the warp
  const int nr = (int)(rows - r0 < 32 ? rows - r0 : 32);
  const int32_t my_lo = indptr[r0 + (lane < nr ? lane : nr)];
  const int32_t my_hi = lane < nr ? indptr[r0 + lane + 1] : my_lo;
  const int32_t beg = __shfl_sync(0xffffffffu, my_lo, 0);
  const int32_t end = __shfl_sync(0xffffffffu, my_hi, nr - 1);
  T acc = T(0);
  if (end - beg <= CAP) {
    T* pw = prod[w];
    const int64_t abeg = VEC ? (beg & ~3) : beg;
    for (int64_t base = abeg + lane * 4; base < end; base += 256) {
      T p0[4], p1[4];
      stream_pass<T, S, VEC>(indices, vals, nnz, beg, end, base, X, ldx, p0);
      stream_pass<T, S, VEC>(indices, vals, nnz, beg, end, base + 128, X, ldx, p1);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int64_t e0 = base + c, e1 = base + 128 + c;
        if (e0 >= beg && e0 < end) pw[e0 - beg] = p0[c];
        if (e1 >= beg && e1 < end) pw[e1 - beg] = p1[c];
      }
    }
    __syncwarp();
    for (int32_t j = my_lo - beg; j < my_hi - beg; ++j) acc += pw[j];
  } else {
    for (int rr = 0; rr < nr; ++rr) {
      const int32_t lo = __shfl_sync(0xffffffffu, my_lo, rr), hi = __shfl_sync(0xffffffffu, my_hi, rr);
      T sum = T(0);
      for (int32_t j = lo + lane; j < hi; j += 32) sum += cvt<T>(vals[j]) * X[(int64_t)indices[j] * ldx];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == rr) acc = sum;
    }
  }
  if (lane < nr) {
    const int64_t orow = operm ? (int64_t)operm[r0 + lane] : r0 + lane;
    Y[orow * ldy] = combine(acc, alpha, beta, Y + orow * ldy);
  }
}

// CSR, k columns: one warp per row, lanes over 32-column chunks; each entry reads a contiguous
// row segment of X (coalesced).
template <class T, class S>
__global__ void __launch_bounds__(256) csr_spmm_kernel(const int32_t* __restrict__ indptr,
                                                       const int32_t* __restrict__ indices,
                                                       const S* __restrict__ vals, int64_t rows,
                                                       const T* __restrict__ X, int64_t ldx, int64_t bsx,
                                                       T* __restrict__ Y, int64_t ldy, int64_t bsy, int64_t k,
                                                       T alpha, T beta, const int32_t* __restrict__ operm,
                                                       const int* skip) {
  if (skip && *skip) return;
  const int64_t b = blockIdx.z;
  X += b * bsx;
  Y += b * bsy;
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t c = (int64_t)blockIdx.y * 32 + lane;
  if (row >= rows) return;
  const int32_t beg = indptr[row], end = indptr[row + 1];
  T acc = T(0);
  if (c < k)
    // entries in groups of four: indices and values, then the four gathers, in flight together;
    // products added in entry order
    for (int32_t j0 = beg; j0 < end; j0 += 4) {
      int32_t col[4];
      T v[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const bool ok = j0 + t < end;
        col[t] = ok ? indices[j0 + t] : 0;
        v[t] = ok ? cvt<T>(vals[j0 + t]) : T(0);
      }
      T x[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) x[t] = j0 + t < end ? X[(int64_t)col[t] * ldx + c] : T(0);
#pragma unroll
      for (int t = 0; t < 4; ++t)
        if (j0 + t < end) acc += v[t] * x[t];
    }
  const int64_t orow = operm ? (int64_t)operm[row] : row;
  if (c < k) Y[orow * ldy + c] = combine(acc, alpha, beta, Y + orow * ldy + c);
}

// Diagonal: Y = alpha * d * X + beta * Y
template <class T, class S>
__global__ void diag_kernel(const S* __restrict__ d, int64_t rows, const T* __restrict__ X, int64_t ldx,
                            int64_t bsx, T* __restrict__ Y, int64_t ldy, int64_t bsy, int64_t k, T alpha,
                            T beta, const int* skip) {
  if (skip && *skip) return;
  const int64_t b = blockIdx.y;
  X += b * bsx;
  Y += b * bsy;
  const int64_t total = rows * k;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / k, c = u - i * k;
    const T v = cvt<T>(d[i]) * X[i * ldx + c];
    Y[i * ldy + c] = combine(v, alpha, beta, Y + i * ldy + c);
  }
}

// Y = alpha * X + beta * Y  (ScalarMul, Identity, Sum accumulation)
template <class T>
__global__ void axpby_kernel(const T* __restrict__ X, int64_t ldx, int64_t bsx, T* __restrict__ Y, int64_t ldy,
                             int64_t bsy, int64_t rows, int64_t k, T alpha, T beta, const int* skip) {
  if (skip && *skip) return;
  const int64_t b = blockIdx.y;
  X += b * bsx;
  Y += b * bsy;
  const int64_t total = rows * k;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / k, c = u - i * k;
    Y[i * ldy + c] = combine(X[i * ldx + c], alpha, beta, Y + i * ldy + c);
  }
}

// xp[b][i][c] = X[b][perm[i]][c]: the input of a permuted Sparse node in its stored order.
template <class T>
__global__ void k_perm_gather(const int32_t* __restrict__ perm, int64_t n, const T* __restrict__ X, int64_t ldx,
                              int64_t bsx, T* __restrict__ xp, int64_t k, const int* skip) {
  if (skip && *skip) return;
  const int64_t b = blockIdx.y;
  X += b * bsx;
  xp += b * n * k;
  const int64_t total = n * k;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / k, c = u - i * k;
    xp[u] = X[(int64_t)perm[i] * ldx + c];
  }
}

// --------------------------------------------------------------------------------------------
// launch helpers

static int elementwise_grid(int64_t total) {
  const int64_t want = ceil_div(total, 256);
  const int64_t cap = (int64_t)num_sms() * 8;
  return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

template <class T>
int launch_axpby_b(const T* X, int64_t ldx, int64_t bsx, T* Y, int64_t ldy, int64_t bsy, int64_t rows, int64_t k,
                   int64_t batch, T alpha, T beta, const int* skip, cudaStream_t st) {
  if (rows * k == 0) return COLAGB_OK;
  dim3 grid(elementwise_grid(rows * k), (unsigned)batch);
  axpby_kernel<T><<<grid, 256, 0, st>>>(X, ldx, bsx, Y, ldy, bsy, rows, k, alpha, beta, skip);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

template <class T>
int launch_axpby(const T* X, int64_t ldx, T* Y, int64_t ldy, int64_t rows, int64_t k, T alpha, T beta,
                 const int* skip, cudaStream_t st) {
  return launch_axpby_b<T>(X, ldx, 0, Y, ldy, 0, rows, k, 1, alpha, beta, skip, st);
}
template int launch_axpby<float>(const float*, int64_t, float*, int64_t, int64_t, int64_t, float, float,
                                 const int*, cudaStream_t);
template int launch_axpby<double>(const double*, int64_t, double*, int64_t, int64_t, int64_t, double, double,
                                  const int*, cudaStream_t);

template <class T>
int launch_perm_gather(const int32_t* perm, int64_t n, const T* X, int64_t ldx, int64_t bsx, T* xp, int64_t k,
                       int64_t batch, const int* skip, cudaStream_t st) {
  if (n * k == 0) return COLAGB_OK;
  dim3 grid(elementwise_grid(n * k), (unsigned)batch);
  k_perm_gather<T><<<grid, 256, 0, st>>>(perm, n, X, ldx, bsx, xp, k, skip);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

template <class T, class S>
static int launch_dense(const colagb_op_node& nd, const T* X, int64_t ldx, int64_t bsx, T* Y, int64_t ldy,
                        int64_t bsy, int64_t k, int64_t batch, T alpha, T beta, const int* skip, cudaStream_t st) {
  const S* A = static_cast<const S*>(nd.data);
  if (nd.rows == 0 || k == 0) return COLAGB_OK;
  if (k <= 4) {
    dim3 grid((unsigned)ceil_div(nd.rows, 8), (unsigned)batch);
    switch (k) {
      case 1: dense_gemv_kernel<T, S, 1><<<grid, 256, 0, st>>>(A, nd.ld, nd.rows, nd.cols, X, ldx, bsx, Y, ldy, bsy, alpha, beta, skip); break;
      case 2: dense_gemv_kernel<T, S, 2><<<grid, 256, 0, st>>>(A, nd.ld, nd.rows, nd.cols, X, ldx, bsx, Y, ldy, bsy, alpha, beta, skip); break;
      case 3: dense_gemv_kernel<T, S, 3><<<grid, 256, 0, st>>>(A, nd.ld, nd.rows, nd.cols, X, ldx, bsx, Y, ldy, bsy, alpha, beta, skip); break;
      default: dense_gemv_kernel<T, S, 4><<<grid, 256, 0, st>>>(A, nd.ld, nd.rows, nd.cols, X, ldx, bsx, Y, ldy, bsy, alpha, beta, skip); break;
    }
  } else {
    dim3 grid((unsigned)ceil_div(k, 64), (unsigned)ceil_div(nd.rows, 64), (unsigned)batch);
    dense_gemm_kernel<T, S><<<grid, 256, 0, st>>>(A, nd.ld, nd.rows, nd.cols, X, ldx, bsx, Y, ldy, bsy, k, alpha,
                                                  beta, skip);
  }
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

template <class T, class S>
static int launch_csr(const colagb_op_node& nd, const T* X, int64_t ldx, int64_t bsx, T* Y, int64_t ldy,
                      int64_t bsy, int64_t k, int64_t batch, T alpha, T beta, const int* skip, cudaStream_t st) {
  const S* v = static_cast<const S*>(nd.data);
  if (nd.rows == 0 || k == 0) return COLAGB_OK;
  const double avg = nd.rows > 0 ? (double)nd.nnz / (double)nd.rows : 0.0;
  if (k == 1 && avg <= StreamCap<T>::value / 48.0) {
    // short rows: the streaming kernel (most 32-row groups fit its per-warp buffer)
    const bool vec = (reinterpret_cast<uintptr_t>(nd.indices) % 16 == 0) &&
                     (reinterpret_cast<uintptr_t>(v) % (sizeof(S) * 4 < 16 ? sizeof(S) * 4 : 16) == 0);
    dim3 grid((unsigned)ceil_div(nd.rows, (int64_t)kStreamWarps * 32), (unsigned)batch);
    if (vec)
      csr_stream_kernel<T, S, true><<<grid, kStreamWarps * 32, 0, st>>>(nd.indptr, nd.indices, v, nd.rows, nd.nnz, X,
                                                                         ldx, bsx, Y, ldy, bsy, alpha, beta, nd.perm,
                                                                         skip);
    else
      csr_stream_kernel<T, S, false><<<grid, kStreamWarps * 32, 0, st>>>(nd.indptr, nd.indices, v, nd.rows, nd.nnz,
                                                                          X, ldx, bsx, Y, ldy, bsy, alpha, beta, nd.perm,
                                                                          skip);
  } else if (k == 1) {
    int tpr = 1;
    while (tpr < 32 && tpr * 2 <= avg) tpr *= 2;
    dim3 grid((unsigned)ceil_div(nd.rows * tpr, 256), (unsigned)batch);
#define COLAGB_CSR_CASE(N)                                                                                  \
  case N:                                                                                                   \
    csr_spmv_kernel<T, S, N><<<grid, 256, 0, st>>>(nd.indptr, nd.indices, v, nd.rows, X, ldx, bsx, Y, ldy, \
                                                   bsy, alpha, beta, nd.perm, skip);                        \
    break;
    switch (tpr) {
      COLAGB_CSR_CASE(1)
      COLAGB_CSR_CASE(2)
      COLAGB_CSR_CASE(4)
      COLAGB_CSR_CASE(8)
      COLAGB_CSR_CASE(16)
      COLAGB_CSR_CASE(32)
    }
#undef COLAGB_CSR_CASE
  } else {
    dim3 grid((unsigned)ceil_div(nd.rows, 8), (unsigned)ceil_div(k, 32), (unsigned)batch);
    csr_spmm_kernel<T, S><<<grid, 256, 0, st>>>(nd.indptr, nd.indices, v, nd.rows, X, ldx, bsx, Y, ldy, bsy, k,
                                                alpha, beta, nd.perm, skip);
  }
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

template <class T, class S>
static int launch_diag(const colagb_op_node& nd, const T* X, int64_t ldx, int64_t bsx, T* Y, int64_t ldy,
                       int64_t bsy, int64_t k, int64_t batch, T alpha, T beta, const int* skip, cudaStream_t st) {
  if (nd.rows * k == 0) return COLAGB_OK;
  dim3 grid(elementwise_grid(nd.rows * k), (unsigned)batch);
  diag_kernel<T, S><<<grid, 256, 0, st>>>(static_cast<const S*>(nd.data), nd.rows, X, ldx, bsx, Y, ldy, bsy, k,
                                          alpha, beta, skip);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

template <class T>
struct LeafLaunch {
  static int run(int kind, int32_t dtype, const colagb_op_node& nd, const T* X, int64_t ldx, int64_t bsx, T* Y,
                 int64_t ldy, int64_t bsy, int64_t k, int64_t batch, T alpha, T beta, const int* skip,
                 cudaStream_t st) {
#define COLAGB_LEAF(S)                                                                                      \
  do {                                                                                                      \
    if (kind == COLAGB_OP_DENSE) return launch_dense<T, S>(nd, X, ldx, bsx, Y, ldy, bsy, k, batch, alpha, beta, skip, st); \
    if (kind == COLAGB_OP_CSR) return launch_csr<T, S>(nd, X, ldx, bsx, Y, ldy, bsy, k, batch, alpha, beta, skip, st);     \
    return launch_diag<T, S>(nd, X, ldx, bsx, Y, ldy, bsy, k, batch, alpha, beta, skip, st);                \
  } while (0)
    if (dtype == COLAGB_F32) COLAGB_LEAF(float);
    if (dtype == COLAGB_BF16) COLAGB_LEAF(__nv_bfloat16);
    if (dtype == COLAGB_F64) {
      if constexpr (std::is_same<T, double>::value) COLAGB_LEAF(double);
    }
#undef COLAGB_LEAF
    return fail(COLAGB_ERR_UNSUPPORTED, "leaf storage dtype not supported for this compute dtype");
  }
};

// --------------------------------------------------------------------------------------------
// executor

// Whether factor f of a Kronecker node is contracted on the tensor cores (FP32 compute only; see
// COLAGB_KRON_* in colagb.h), and with the three-product split.  pre / q as in the KRON branch below.
template <class T>
static bool kron_on_tensor_cores(int32_t precision, const colagb_op_node& f, int64_t pre, int64_t q, int64_t r,
                                 int64_t c, bool* split) {
  if (!std::is_same<T, float>::value || precision == COLAGB_KRON_FP32) return false;
  if (f.kind != COLAGB_OP_DENSE || (f.dtype != COLAGB_F32 && f.dtype != COLAGB_BF16)) return false;
  if (q > 1 && q < 32) return false;  // few columns per block: the axis-swapped SIMT form
  const int64_t batch = q > 1 ? pre : 1, M = q > 1 ? q : pre;
  if (!tc_contract_supported(batch, M, r, c)) return false;
  // AUTO: only contractions long enough to be compute-bound (c >= 256) and large; with short factors
  // (e.g. 64 x 64) the extra operand pass costs more than the tensor cores save (measured on the
  // 64^3 Kronecker SLQ: 0.41 s on the tensor cores, 0.40 s in FP32 SIMT)
  if (precision == COLAGB_KRON_AUTO &&
      (c < 256 || (double)pre * (double)q * (double)r * (double)c < (double)(1 << 26)))
    return false;
  *split = precision != COLAGB_KRON_BF16;
  return true;
}

template <class T>
int op_apply(const colagb_op* op, int node, const T* X, int64_t ldx, int64_t bsx, T* Y, int64_t ldy, int64_t bsy,
             int64_t k, int64_t batch, T alpha, T beta, Bump& ws, const int* skip, cudaStream_t st) {
  const colagb_op_node& nd = op->nodes[node];
  const std::vector<int32_t>& ch = op->children[node];
  const bool measuring = ws.measure;
  switch (nd.kind) {
    case COLAGB_OP_CSR:
      if (nd.perm) {  // stored P A P^T: gather x through perm, the product writes y through it
        const size_t mark = ws.used;
        T* xp = ws.take<T>((size_t)nd.cols * k * batch);
        if (!measuring) {
          COLAGB_TRY(launch_perm_gather<T>(nd.perm, nd.cols, X, ldx, bsx, xp, k, batch, skip, st));
          COLAGB_TRY(LeafLaunch<T>::run(nd.kind, nd.dtype, nd, xp, k, nd.cols * k, Y, ldy, bsy, k, batch, alpha, beta,
                                        skip, st));
        }
        ws.release(mark);
        return COLAGB_OK;
      }
      if (measuring) return COLAGB_OK;
      return LeafLaunch<T>::run(nd.kind, nd.dtype, nd, X, ldx, bsx, Y, ldy, bsy, k, batch, alpha, beta, skip, st);
    case COLAGB_OP_DENSE:
    case COLAGB_OP_DIAG:
      if (measuring) return COLAGB_OK;
      return LeafLaunch<T>::run(nd.kind, nd.dtype, nd, X, ldx, bsx, Y, ldy, bsy, k, batch, alpha, beta, skip, st);
    case COLAGB_OP_SCALAR:
      if (measuring) return COLAGB_OK;
      return launch_axpby_b<T>(X, ldx, bsx, Y, ldy, bsy, nd.rows, k, batch, alpha * (T)nd.scalar, beta, skip, st);
    case COLAGB_OP_IDENTITY:
      if (measuring) return COLAGB_OK;
      return launch_axpby_b<T>(X, ldx, bsx, Y, ldy, bsy, nd.rows, k, batch, alpha, beta, skip, st);
    case COLAGB_OP_SUM: {
      for (size_t c = 0; c < ch.size(); ++c)
        COLAGB_TRY(op_apply<T>(op, ch[c], X, ldx, bsx, Y, ldy, bsy, k, batch, alpha, c == 0 ? beta : T(1), ws, skip, st));
      return COLAGB_OK;
    }
    case COLAGB_OP_PRODUCT: {
      // c * I factors commute: fold them into alpha; then v <- M_last v, ..., Y = alpha * M_0 v + beta * Y
      std::vector<int32_t> chain;
      T a_eff = alpha;
      for (int32_t c : ch) {
        const colagb_op_node& m = op->nodes[c];
        if (m.kind == COLAGB_OP_SCALAR) a_eff *= (T)m.scalar;
        else if (m.kind != COLAGB_OP_IDENTITY) chain.push_back(c);
      }
      if (chain.empty()) {
        if (measuring) return COLAGB_OK;
        return launch_axpby_b<T>(X, ldx, bsx, Y, ldy, bsy, nd.rows, k, batch, a_eff, beta, skip, st);
      }
      const size_t mark = ws.used;
      for (int64_t b = 0; b < batch; ++b) {
        ws.used = mark;
        const T* cur = X + b * bsx;
        int64_t cur_ld = ldx;
        for (int c = (int)chain.size() - 1; c >= 1; --c) {
          const colagb_op_node& m = op->nodes[chain[c]];
          T* tmp = ws.take<T>((size_t)m.rows * k);
          COLAGB_TRY(op_apply<T>(op, chain[c], cur, cur_ld, 0, tmp, k, 0, k, 1, T(1), T(0), ws, skip, st));
          cur = tmp;
          cur_ld = k;
        }
        COLAGB_TRY(op_apply<T>(op, chain[0], cur, cur_ld, 0, Y + b * bsy, ldy, 0, k, 1, a_eff, beta, ws, skip, st));
        if (measuring) break;
      }
      ws.release(mark);
      return COLAGB_OK;
    }
    case COLAGB_OP_KRON: {
      // X viewed as (c_0, ..., c_{m-1}, k).  Factor i contracts axis i:
      //   out[pre, r_i, post*k] = M_i (r_i x c_i) @ in[pre, c_i, post*k]
      // i.e. a batch of `pre` (c_i x post*k) blocks with row stride post*k.
      const int m = (int)ch.size();
      std::vector<int64_t> r(m), c(m);
      for (int i = 0; i < m; ++i) {
        r[i] = op->nodes[ch[i]].rows;
        c[i] = op->nodes[ch[i]].cols;
      }
      int64_t maxsz = 1;
      for (int i = -1; i < m; ++i) {  // i = -1: the input itself
        int64_t s = 1;
        for (int j = 0; j <= i; ++j) s *= r[j];
        for (int j = i + 1; j < m; ++j) s *= c[j];
        if (s > maxsz) maxsz = s;
      }
      const size_t mark = ws.used;
      T* buf[2] = {ws.take<T>((size_t)maxsz * k), ws.take<T>((size_t)maxsz * k)};
      // scratch for the axis-swapped form of a factor with few columns per block (below)
      T* sw[2] = {ws.take<T>((size_t)maxsz * k), ws.take<T>((size_t)maxsz * k)};
      for (int64_t b = 0; b < batch && !measuring; ++b) {
        const T* in = X + b * bsx;
        int which = 0;  // next scratch buffer to write
        if (ldx != k) {  // make the input contiguous first
          COLAGB_TRY(launch_axpby_b<T>(in, ldx, 0, buf[1], k, 0, nd.cols, k, 1, T(1), T(0), skip, st));
          in = buf[1];
          which = 0;
        }
        for (int i = 0; i < m; ++i) {
          int64_t pre = 1, post = 1;
          for (int j = 0; j < i; ++j) pre *= r[j];
          for (int j = i + 1; j < m; ++j) post *= c[j];
          const bool last = (i == m - 1);
          const bool direct = last && ldy == k;
          T* out = direct ? (Y + b * bsy) : buf[which];
          const int64_t q = post * k;
          bool split = true;
          if (kron_on_tensor_cores<T>(nd.precision, op->nodes[ch[i]], pre, q, r[i], c[i], &split)) {
            // out[p, r, q] on the tensor cores: the operand (p, c, q) transposed per p into K-major
            // BF16 when q > 1, taken row by row when q == 1
            const colagb_op_node& f = op->nodes[ch[i]];
            const float a_f = direct ? (float)alpha : 1.f, b_f = direct ? (float)beta : 0.f;
            float* o = reinterpret_cast<float*>(out);
            const float* a_in = reinterpret_cast<const float*>(in);
            const size_t tmark = ws.used;
            if (q > 1)
              COLAGB_TRY(tc_contract(a_in, true, pre, q, c[i], f.data, f.dtype, f.ld, r[i], o, r[i] * q, 1, q, a_f, b_f,
                                     split, ws, skip, st));
            else
              COLAGB_TRY(tc_contract(a_in, false, 1, pre, c[i], f.data, f.dtype, f.ld, r[i], o, 0, r[i], 1, a_f, b_f,
                                     split, ws, skip, st));
            ws.release(tmark);
          } else if (q <= 8 && pre >= 16 && pre <= 65535 && c[i] <= 65535) {
            // `pre` products of M_i with (c_i x q) blocks re-read M_i `pre` times; with the first two
            // axes swapped they are one product M_i @ (c_i x pre*q), then swapped back
            COLAGB_TRY(launch_axpby_b<T>(in, c[i] * q, q, sw[0], q, pre * q, pre, q, c[i], T(1), T(0), skip, st));
            COLAGB_TRY(op_apply<T>(op, ch[i], sw[0], pre * q, 0, sw[1], pre * q, 0, pre * q, 1, T(1), T(0), ws, skip,
                                   st));
            COLAGB_TRY(launch_axpby_b<T>(sw[1], pre * q, q, out, q, r[i] * q, r[i], q, pre, direct ? alpha : T(1),
                                         direct ? beta : T(0), skip, st));
          } else {
            COLAGB_TRY(op_apply<T>(op, ch[i], in, post * k, c[i] * post * k, out, post * k, r[i] * post * k,
                                   post * k, pre, direct ? alpha : T(1), direct ? beta : T(0), ws, skip, st));
          }
          if (last && !direct)
            COLAGB_TRY(launch_axpby_b<T>(out, k, 0, Y + b * bsy, ldy, 0, nd.rows, k, 1, alpha, beta, skip, st));
          in = out;
          which ^= 1;
        }
      }
      if (measuring) {  // children of a Kronecker may need workspace of their own, and so do the
                        // tensor-core contractions
        for (int i = 0; i < m; ++i)
          COLAGB_TRY(op_apply<T>(op, ch[i], nullptr, k, 0, nullptr, k, 0, k, 1, T(1), T(0), ws, skip, st));
        for (int i = 0; i < m; ++i) {
          int64_t pre = 1, post = 1;
          for (int j = 0; j < i; ++j) pre *= r[j];
          for (int j = i + 1; j < m; ++j) post *= c[j];
          const int64_t q = post * k;
          bool split = true;
          if (!kron_on_tensor_cores<T>(nd.precision, op->nodes[ch[i]], pre, q, r[i], c[i], &split)) continue;
          const colagb_op_node& f = op->nodes[ch[i]];
          const size_t tmark = ws.used;
          COLAGB_TRY(tc_contract(nullptr, q > 1, q > 1 ? pre : 1, q > 1 ? q : pre, c[i], f.data, f.dtype, f.ld, r[i],
                                 nullptr, 0, 1, 1, 1.f, 0.f, split, ws, skip, st));
          ws.release(tmark);
        }
      }
      ws.release(mark);
      return COLAGB_OK;
    }
    case COLAGB_OP_BLOCKDIAG: {
      int64_t ri = 0, ci = 0;
      for (size_t cidx = 0; cidx < ch.size(); ++cidx) {
        const colagb_op_node& m = op->nodes[ch[cidx]];
        const int64_t mult = op->mult[node].empty() ? 1 : op->mult[node][cidx];
        for (int64_t b = 0; b < batch; ++b) {
          // the `mult` copies act on consecutive row slices: a batched apply
          COLAGB_TRY(op_apply<T>(op, ch[cidx], X + b * bsx + ci * ldx, ldx, m.cols * ldx, Y + b * bsy + ri * ldy,
                                 ldy, m.rows * ldy, k, mult, alpha, beta, ws, skip, st));
          if (measuring) break;
        }
        ri += mult * m.rows;
        ci += mult * m.cols;
      }
      return COLAGB_OK;
    }
    default:
      return fail(COLAGB_ERR_UNSUPPORTED, "unknown operator node kind");
  }
}

template int op_apply<float>(const colagb_op*, int, const float*, int64_t, int64_t, float*, int64_t, int64_t,
                             int64_t, int64_t, float, float, Bump&, const int*, cudaStream_t);
template int op_apply<double>(const colagb_op*, int, const double*, int64_t, int64_t, double*, int64_t, int64_t,
                              int64_t, int64_t, double, double, Bump&, const int*, cudaStream_t);

FusedForm fused_form(const colagb_op* op) {
  FusedForm f;
  const colagb_op_node& r = op->nodes[op->root];
  auto is_leaf = [](const colagb_op_node& n) {
    return (n.kind == COLAGB_OP_CSR || n.kind == COLAGB_OP_DENSE) && n.rows == n.cols && n.perm == nullptr;
  };
  if (is_leaf(r)) {
    f.ok = true;
    f.leaf = &r;
    return f;
  }
  if (r.kind == COLAGB_OP_SUM && op->children[op->root].size() == 2) {
    const auto& ch = op->children[op->root];
    for (int a = 0; a < 2; ++a) {
      const colagb_op_node& L = op->nodes[ch[a]];
      const colagb_op_node& Sn = op->nodes[ch[1 - a]];
      if (is_leaf(L) && (Sn.kind == COLAGB_OP_SCALAR || Sn.kind == COLAGB_OP_IDENTITY)) {
        f.ok = true;
        f.leaf = &L;
        f.shift = Sn.kind == COLAGB_OP_SCALAR ? Sn.scalar : 1.0;
        return f;
      }
    }
  }
  return f;
}

}  // namespace colagb

// --------------------------------------------------------------------------------------------
// C ABI
using namespace colagb;

extern "C" const char* colagb_last_error(void) { return g_last_error.c_str(); }

extern "C" int colagb_version(int32_t* version, int32_t* arch) {
  if (version) *version = 100;
  if (arch) *arch = 1003;
  return COLAGB_OK;
}

static int validate_node(const colagb_op_node& n, int idx, int num_nodes) {
  auto bad = [&](const char* what) {
    return fail(COLAGB_ERR_INVALID, "operator node " + std::to_string(idx) + ": " + what);
  };
  if (n.rows < 0 || n.cols < 0) return bad("negative shape");
  if (n.perm && n.kind != COLAGB_OP_CSR) return bad("a permutation on a node that is not Sparse");
  switch (n.kind) {
    case COLAGB_OP_DENSE:
      if (!n.data && n.rows * n.cols > 0) return bad("Dense without data");
      if (n.ld < n.cols) return bad("Dense leading dimension smaller than cols");
      break;
    case COLAGB_OP_CSR:
      if ((!n.indptr || !n.indices || !n.data) && n.nnz > 0) return bad("Sparse without indptr/indices/values");
      if (!n.indptr && n.rows > 0) return bad("Sparse without indptr");
      if (n.perm && n.rows != n.cols) return bad("a permuted Sparse must be square");
      break;
    case COLAGB_OP_DIAG:
      if (n.rows != n.cols) return bad("Diagonal must be square");
      if (!n.data && n.rows > 0) return bad("Diagonal without data");
      break;
    case COLAGB_OP_SCALAR:
    case COLAGB_OP_IDENTITY:
      if (n.rows != n.cols) return bad("ScalarMul/Identity must be square");
      break;
    case COLAGB_OP_SUM:
    case COLAGB_OP_PRODUCT:
    case COLAGB_OP_KRON:
    case COLAGB_OP_BLOCKDIAG:
      if (n.num_children <= 0 || !n.children) return bad("composite without children");
      for (int c = 0; c < n.num_children; ++c)
        if (n.children[c] < 0 || n.children[c] >= num_nodes) return bad("child index out of range");
      break;
    default:
      return bad("unknown kind");
  }
  if (n.kind == COLAGB_OP_DENSE || n.kind == COLAGB_OP_CSR || n.kind == COLAGB_OP_DIAG) {
    if (n.dtype != COLAGB_F32 && n.dtype != COLAGB_F64 && n.dtype != COLAGB_BF16) return bad("unknown dtype");
  }
  return COLAGB_OK;
}

static int check_shapes(const colagb_op* op, int node, std::vector<int>& state) {
  // state: 0 = unvisited, 1 = on stack, 2 = done (cycle detection)
  if (state[node] == 1) return fail(COLAGB_ERR_INVALID, "operator graph has a cycle");
  if (state[node] == 2) return COLAGB_OK;
  state[node] = 1;
  const colagb_op_node& n = op->nodes[node];
  const auto& ch = op->children[node];
  for (int c : ch) COLAGB_TRY(check_shapes(op, c, state));
  auto dims = [&](int c) { return std::make_pair(op->nodes[c].rows, op->nodes[c].cols); };
  switch (n.kind) {
    case COLAGB_OP_SUM:
      for (int c : ch)
        if (dims(c) != std::make_pair(n.rows, n.cols)) return fail(COLAGB_ERR_INVALID, "Sum child shape mismatch");
      break;
    case COLAGB_OP_PRODUCT:
      if (op->nodes[ch.front()].rows != n.rows || op->nodes[ch.back()].cols != n.cols)
        return fail(COLAGB_ERR_INVALID, "Product outer shape mismatch");
      for (size_t i = 0; i + 1 < ch.size(); ++i)
        if (op->nodes[ch[i]].cols != op->nodes[ch[i + 1]].rows)
          return fail(COLAGB_ERR_INVALID, "Product inner dimension mismatch");
      break;
    case COLAGB_OP_KRON: {
      int64_t r = 1, c = 1;
      for (int x : ch) {
        r *= op->nodes[x].rows;
        c *= op->nodes[x].cols;
      }
      if (r != n.rows || c != n.cols) return fail(COLAGB_ERR_INVALID, "Kronecker shape mismatch");
      break;
    }
    case COLAGB_OP_BLOCKDIAG: {
      int64_t r = 0, c = 0;
      for (size_t i = 0; i < ch.size(); ++i) {
        const int64_t m = op->mult[node].empty() ? 1 : op->mult[node][i];
        if (m < 1) return fail(COLAGB_ERR_INVALID, "BlockDiag multiplicity must be >= 1");
        r += m * op->nodes[ch[i]].rows;
        c += m * op->nodes[ch[i]].cols;
      }
      if (r != n.rows || c != n.cols) return fail(COLAGB_ERR_INVALID, "BlockDiag shape mismatch");
      break;
    }
    default:
      break;
  }
  state[node] = 2;
  return COLAGB_OK;
}

extern "C" int colagb_op_create(const colagb_op_node* nodes, int32_t num_nodes, int32_t root, colagb_op** out) {
  if (!nodes || !out || num_nodes <= 0 || root < 0 || root >= num_nodes)
    return fail(COLAGB_ERR_INVALID, "colagb_op_create: bad arguments");
  *out = nullptr;
  for (int i = 0; i < num_nodes; ++i) COLAGB_TRY(validate_node(nodes[i], i, num_nodes));
  colagb_op* op = new colagb_op();
  op->nodes.assign(nodes, nodes + num_nodes);
  op->children.resize(num_nodes);
  op->mult.resize(num_nodes);
  op->root = root;
  bool any64 = false;
  for (int i = 0; i < num_nodes; ++i) {
    const colagb_op_node& n = nodes[i];
    if (n.num_children > 0) op->children[i].assign(n.children, n.children + n.num_children);
    if (n.kind == COLAGB_OP_BLOCKDIAG && n.multiplicities)
      op->mult[i].assign(n.multiplicities, n.multiplicities + n.num_children);
    op->nodes[i].children = nullptr;        // the copies above own these now
    op->nodes[i].multiplicities = nullptr;
    if ((n.kind == COLAGB_OP_DENSE || n.kind == COLAGB_OP_CSR || n.kind == COLAGB_OP_DIAG) && n.dtype == COLAGB_F64)
      any64 = true;
  }
  op->compute_dtype = any64 ? COLAGB_F64 : COLAGB_F32;
  std::vector<int> state(num_nodes, 0);
  int s = check_shapes(op, root, state);
  if (s != COLAGB_OK) {
    delete op;
    return s;
  }
  *out = op;
  return COLAGB_OK;
}

extern "C" int colagb_op_free(colagb_op* op) {
  delete op;
  return COLAGB_OK;
}

extern "C" int colagb_op_info(const colagb_op* op, int64_t* rows, int64_t* cols, int32_t* compute_dtype) {
  if (!op) return fail(COLAGB_ERR_INVALID, "null operator");
  if (rows) *rows = op->nodes[op->root].rows;
  if (cols) *cols = op->nodes[op->root].cols;
  if (compute_dtype) *compute_dtype = op->compute_dtype;
  return COLAGB_OK;
}

extern "C" int colagb_matmat_workspace_bytes(const colagb_op* op, int64_t k, size_t* bytes) {
  if (!op || !bytes || k < 0) return fail(COLAGB_ERR_INVALID, "colagb_matmat_workspace_bytes: bad arguments");
  Bump ws = Bump::measuring();
  int s = op->compute_dtype == COLAGB_F64
              ? op_apply<double>(op, op->root, nullptr, k, 0, nullptr, k, 0, k, 1, 1.0, 0.0, ws, nullptr, 0)
              : op_apply<float>(op, op->root, nullptr, k, 0, nullptr, k, 0, k, 1, 1.f, 0.f, ws, nullptr, 0);
  if (s != COLAGB_OK) return s;
  *bytes = ws.peak;
  return COLAGB_OK;
}

extern "C" int colagb_matmat(const colagb_op* op, const void* X, int64_t ldx, void* Y, int64_t ldy, int64_t k,
                             double alpha, double beta, void* workspace, size_t workspace_bytes, void* stream) {
  if (!op) return fail(COLAGB_ERR_INVALID, "null operator");
  const colagb_op_node& r = op->nodes[op->root];
  if (k < 0 || ldx < k || ldy < k) return fail(COLAGB_ERR_INVALID, "colagb_matmat: bad k / leading dimensions");
  if ((r.cols * k > 0 && !X) || (r.rows * k > 0 && !Y)) return fail(COLAGB_ERR_INVALID, "colagb_matmat: null X/Y");
  size_t need = 0;
  COLAGB_TRY(colagb_matmat_workspace_bytes(op, k, &need));
  if (need > 0 && (workspace == nullptr || workspace_bytes < need))
    return fail(COLAGB_ERR_WORKSPACE, "colagb_matmat: workspace too small (need " + std::to_string(need) + " bytes)");
  Bump ws(workspace, workspace_bytes);
  cudaStream_t st = as_stream(stream);
  if (op->compute_dtype == COLAGB_F64)
    return op_apply<double>(op, op->root, static_cast<const double*>(X), ldx, 0, static_cast<double*>(Y), ldy, 0, k,
                            1, alpha, beta, ws, nullptr, st);
  return op_apply<float>(op, op->root, static_cast<const float*>(X), ldx, 0, static_cast<float*>(Y), ldy, 0, k, 1,
                         (float)alpha, (float)beta, ws, nullptr, st);
}
