// Lanczos with full reorthogonalisation and the tridiagonal eigensolver (FP64, or FP32 for FP32 recurrences).
//
// Reference (cola/linalg/decompositions/lanczos.py):
//   init_lanczos :275-284   V[..., 1] = rhs / |rhs|, i = 1
//   lanczos_fact :235-272   while i <= max_iters and any(subdiag[i-1] > tol*subdiag[1] or i <= 1):
//       V[i] /= |V[i]| ; w = A V[i] ; diag[i-1] = <w, V[i]>
//       w -= diag[i-1] V[i] + subdiag[i-1] V[i-1] ; w = CGS2(V, w) ; V[i+1] = w ; subdiag[i] = |w| ; i++
//   do_double_gram :287-296 two passes of w -= V (V^T w) over the basis.
// The reference's CGS passes run over all max_iters+2 slots; the unfilled ones are zero, so only
// slots 1..i are visited here (same values, fewer bytes).
//
// Basis layout: slot j is an n x bs row-major block at basis + j*n*bs (probe index fastest), so
// every pass reads contiguous, coalesced rows.  Per step: 1 operator application, 2 column-norm
// reductions, 1 dot, and 2 x (V^T w then w -= V h) passes over the filled slots.
#include <cmath>
#include <string>
#include <vector>

#include <type_traits>

#include "common.cuh"
#include "ops.cuh"

namespace colagb {

template <class T>
struct LzState {
  T* nrm;         // bs
  T* hbuf;        // (max_iters + 2) x bs projection coefficients
  T* hpart;       // nblk x (max_iters + 2) x bs partial projections
  T* npart;       // nblk x bs partial norms / dots
  int* done;
  int* step;      // current i
  unsigned int* counters;
};

__device__ __forceinline__ bool lz_last_block(unsigned int* counter) {
  __shared__ int s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

// Per-probe column reduction over rows of an n x bs block: f(r, b) summed per b.
// Block layout: threads = (rows_per_pass x bsc), bsc = min(bs, 256).
template <class T, class F>
__device__ __forceinline__ void lz_partials(int64_t n, int64_t bs, F f, T* out, T* smem) {
  const int t = threadIdx.x;
  for (int64_t b0 = 0; b0 < bs; b0 += blockDim.x) {
    const int bc = (int)((bs - b0) < (int64_t)blockDim.x ? (bs - b0) : (int64_t)blockDim.x);
    const int rpp = blockDim.x / bc;
    const int my_b = t % bc, my_r = t / bc;
    T acc = T(0);
    if (my_r < rpp)
      for (int64_t r = (int64_t)blockIdx.x * rpp + my_r; r < n; r += (int64_t)rpp * gridDim.x) acc += f(r, b0 + my_b);
    smem[t] = acc;
    __syncthreads();
    // tree over the rpp row slots (a serial sum by one thread per column is rpp dependent
    // shared-memory round trips)
    for (int w = rpp; w > 1;) {
      const int h = (w + 1) >> 1;
      if (my_r < w - h) smem[t] += smem[t + h * bc];
      __syncthreads();
      w = h;
    }
    if (t < bc) out[b0 + t] = smem[t];
    __syncthreads();
  }
}

// The same per-column sums of a[r][b] * c[r][b] for FP32 blocks with bs a multiple of 4 (bs <= 1024):
// thread t takes column quad t % (bs / 4) and rows t / (bs / 4), t / (bs / 4) + rpp, ... with 128-bit
// loads, four rows per round on independent accumulators (a thread per column and row with scalar
// loads waited on one load at a time: ~0.6 TB/s on 64-column blocks).  Row slots are then summed in a
// fixed tree as in lz_partials.
__device__ __forceinline__ void lz_partials4(int64_t n, int64_t bs, const float* __restrict__ a,
                                             const float* __restrict__ c, float4* out4, float4* smem4) {
  const int t = threadIdx.x;
  const int qd = (int)(bs / 4);
  const int rpp = (int)blockDim.x / qd;
  const int my_q = t % qd, my_r = t / qd;
  float4 acc[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (my_r < rpp) {
    const int64_t stride = (int64_t)rpp * gridDim.x;
    int64_t r = (int64_t)blockIdx.x * rpp + my_r;
    for (; r + 3 * stride < n; r += 4 * stride) {
      float4 x[4], y[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t o = (r + u * stride) * bs + 4 * my_q;
        x[u] = __ldg(reinterpret_cast<const float4*>(a + o));
        y[u] = __ldg(reinterpret_cast<const float4*>(c + o));
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        acc[u].x += x[u].x * y[u].x;
        acc[u].y += x[u].y * y[u].y;
        acc[u].z += x[u].z * y[u].z;
        acc[u].w += x[u].w * y[u].w;
      }
    }
    for (; r < n; r += stride) {
      const int64_t o = r * bs + 4 * my_q;
      const float4 x = __ldg(reinterpret_cast<const float4*>(a + o)), y = __ldg(reinterpret_cast<const float4*>(c + o));
      acc[0].x += x.x * y.x;
      acc[0].y += x.y * y.y;
      acc[0].z += x.z * y.z;
      acc[0].w += x.w * y.w;
    }
  }
  float4 tot;
  tot.x = (acc[0].x + acc[1].x) + (acc[2].x + acc[3].x);
  tot.y = (acc[0].y + acc[1].y) + (acc[2].y + acc[3].y);
  tot.z = (acc[0].z + acc[1].z) + (acc[2].z + acc[3].z);
  tot.w = (acc[0].w + acc[1].w) + (acc[2].w + acc[3].w);
  smem4[t] = tot;
  __syncthreads();
  for (int w = rpp; w > 1;) {
    const int h = (w + 1) >> 1;
    if (my_r < w - h) {
      const float4 o = smem4[t + h * qd];
      smem4[t].x += o.x;
      smem4[t].y += o.y;
      smem4[t].z += o.z;
      smem4[t].w += o.w;
    }
    __syncthreads();
    w = h;
  }
  if (t < qd) out4[t] = smem4[t];
  __syncthreads();
}

// Column sums of a .* c into this CTA's partials: the 128-bit path for FP32 blocks of 4..1024 columns
// and for single FP32 columns with n % 4 == 0 (16-byte aligned), the generic one otherwise.
template <class T>
__device__ __forceinline__ void lz_colsum(int64_t n, int64_t bs, const T* a, const T* c, T* out, T* smem) {
  if constexpr (std::is_same<T, float>::value) {
    const bool al = (reinterpret_cast<uintptr_t>(a) % 16) == 0 && (reinterpret_cast<uintptr_t>(c) % 16) == 0;
    if (al && bs % 4 == 0 && bs <= 1024) {
      __shared__ float4 smem4[256];
      lz_partials4(n, bs, a, c, reinterpret_cast<float4*>(out), smem4);
      return;
    }
    if (al && bs == 1 && n % 4 == 0) {  // one column: four consecutive rows per 128-bit load
      __shared__ float4 smem4b[256];
      __shared__ float4 quad;
      lz_partials4(n / 4, 4, a, c, &quad, smem4b);
      if (threadIdx.x == 0) out[0] = (quad.x + quad.y) + (quad.z + quad.w);
      __syncthreads();
      return;
    }
  }
  lz_partials<T>(n, bs, [&](int64_t r, int64_t b) { return a[r * bs + b] * c[r * bs + b]; }, out, smem);
}

// Sum over the nb per-CTA partials of column b, formed by the whole block (all threads get it).
template <class T>
__device__ __forceinline__ T lz_block_total(const T* part, int nb, int64_t bs, int64_t b, T* red) {
  T v = T(0);
  for (int q = threadIdx.x; q < nb; q += blockDim.x) v += __ldcg(part + (int64_t)q * bs + b);
  return block_sum(v, red);
}

// Totals of the first kLzStage columns into shared memory, block-parallel; lz_total reads them
// (serial sum only beyond kLzStage columns).
constexpr int kLzStage = 64;
template <class T>
__device__ __forceinline__ void lz_stage(const T* part, int nb, int64_t bs, T* tot, T* red, T* scratch) {
  const int64_t kk = bs < kLzStage ? bs : kLzStage;
  if (kk >= 8 && blockDim.x % kk == 0) {
    // all columns at once: thread (b, g) sums partials g, g + G, ... of column b (consecutive threads,
    // consecutive columns), then the G group sums of each column are added in order
    const int G = (int)(blockDim.x / kk);
    const int b = (int)(threadIdx.x % kk), g = (int)(threadIdx.x / kk);
    T acc = T(0);
#pragma unroll 4
    for (int q = g; q < nb; q += G) acc += __ldcg(part + (int64_t)q * bs + b);
    scratch[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < kk) {
      T sum = T(0);
      for (int gg = 0; gg < G; ++gg) sum += scratch[gg * kk + threadIdx.x];
      tot[threadIdx.x] = sum;
    }
    __syncthreads();
    return;
  }
  for (int64_t b = 0; b < kk; ++b) {
    const T v = lz_block_total(part, nb, bs, b, red);
    if (threadIdx.x == 0) tot[b] = v;
  }
  __syncthreads();
}

template <class T>
__device__ __forceinline__ T lz_sum(const T* part, int nb, int64_t bs, int64_t b) {
  T s = T(0);
  for (int q = 0; q < nb; ++q) s += __ldcg(part + (int64_t)q * bs + b);
  return s;
}

template <class T>
__device__ __forceinline__ T lz_total(const T* part, int nb, int64_t bs, int64_t b, const T* tot) {
  return b < kLzStage ? tot[b] : lz_sum(part, nb, bs, b);
}

// V[i] /= |V[i]|   (norm pass; the division is k_lz_scale)
template <class T>
__global__ void __launch_bounds__(256) k_lz_norm(const T* v, int64_t n, int64_t bs, LzState<T> s) {
  if (*s.done) return;
  __shared__ T smem[256];
  lz_colsum<T>(n, bs, v, v, s.npart + (int64_t)blockIdx.x * bs, smem);
  if (lz_last_block(s.counters + 0)) {
    __shared__ T tot[kLzStage], red[32];
    lz_stage(s.npart, gridDim.x, bs, tot, red, smem);
    for (int64_t b = threadIdx.x; b < bs; b += blockDim.x) s.nrm[b] = sqrt(lz_total(s.npart, gridDim.x, bs, b, tot));
    if (threadIdx.x == 0) s.counters[0] = 0;
  }
}

template <class T>
__global__ void k_lz_scale(T* v, int64_t n, int64_t bs, LzState<T> s) {
  if (*s.done) return;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * bs; u += (int64_t)gridDim.x * blockDim.x)
    v[u] = v[u] / s.nrm[u % bs];
}

// diag[b][i-1] = <w, V[i]>
template <class T>
__global__ void __launch_bounds__(256) k_lz_alpha(const T* w, const T* vi, int64_t n, int64_t bs, T* diag,
                                                  int max_iters, LzState<T> s) {
  if (*s.done) return;
  __shared__ T smem[256];
  lz_colsum<T>(n, bs, w, vi, s.npart + (int64_t)blockIdx.x * bs, smem);
  if (lz_last_block(s.counters + 1)) {
    __shared__ T tot[kLzStage], red[32];
    lz_stage(s.npart, gridDim.x, bs, tot, red, smem);
    const int i = *s.step;
    for (int64_t b = threadIdx.x; b < bs; b += blockDim.x)
      diag[b * max_iters + (i - 1)] = lz_total(s.npart, gridDim.x, bs, b, tot);
    if (threadIdx.x == 0) s.counters[1] = 0;
  }
}

// w -= diag[i-1] V[i] + subdiag[i-1] V[i-1]
template <class T>
__global__ void k_lz_three_term(T* w, const T* vi, const T* vim1, int64_t n, int64_t bs, const T* diag,
                                const T* subdiag, int max_iters, LzState<T> s) {
  if (*s.done) return;
  const int i = *s.step;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * bs; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = u % bs;
    w[u] -= diag[b * max_iters + (i - 1)] * vi[u] + subdiag[b * (max_iters + 1) + (i - 1)] * vim1[u];
  }
}

// Projection partials: hpart[blk][j][b] = sum over the block's rows of V[j][r][b] * w[r][b], j = 1..i.
// Each block owns a contiguous row range.  Four basis slots per pass: w is read once for the four,
// and the four partial sums share one tree reduction (one pass per slot re-read w and waited on a
// reduction per slot -- this kernel is most of an SLQ run's time).
template <class T>
__global__ void __launch_bounds__(256) k_lz_project(const T* basis, const T* w, int64_t n, int64_t bs,
                                                    int64_t slots, LzState<T> s) {
  if (*s.done) return;
  constexpr int JB = 4;
  __shared__ T smem[JB * 256];
  const int i = *s.step;
  const int64_t rows_per_block = ceil_div(n, gridDim.x);
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = r0 + rows_per_block < n ? r0 + rows_per_block : n;
  T* out = s.hpart + (int64_t)blockIdx.x * slots * bs;
  const int t = threadIdx.x;
  const int64_t slot = n * bs;
  for (int64_t b0 = 0; b0 < bs; b0 += blockDim.x) {
    const int bc = (int)((bs - b0) < (int64_t)blockDim.x ? (bs - b0) : (int64_t)blockDim.x);
    const int rpp = blockDim.x / bc;
    const int my_b = t % bc, my_r = t / bc;
    for (int j0 = 1; j0 <= i; j0 += JB) {
      const int nj = (i - j0 + 1) < JB ? (i - j0 + 1) : JB;
      T acc[JB] = {T(0), T(0), T(0), T(0)};
      if (my_r < rpp) {
        const T* v0 = basis + (int64_t)j0 * slot + b0 + my_b;
        for (int64_t r = r0 + my_r; r < r1; r += rpp) {
          const T wv = w[r * bs + b0 + my_b];
#pragma unroll
          for (int q = 0; q < JB; ++q)
            if (q < nj) acc[q] += v0[(int64_t)q * slot + r * bs] * wv;
        }
      }
#pragma unroll
      for (int q = 0; q < JB; ++q) smem[q * 256 + t] = acc[q];
      __syncthreads();
      for (int wd = rpp; wd > 1;) {  // tree over the row slots, all JB sums at once
        const int h = (wd + 1) >> 1;
        if (my_r < wd - h) {
#pragma unroll
          for (int q = 0; q < JB; ++q) smem[q * 256 + t] += smem[q * 256 + t + h * bc];
        }
        __syncthreads();
        wd = h;
      }
      if (t < bc) {
        for (int q = 0; q < nj; ++q) out[(int64_t)(j0 + q) * bs + b0 + t] = smem[q * 256 + t];
      }
      __syncthreads();
    }
  }
}

// Single-vector form (bs == 1, n % 4 == 0): block blk owns rows [blk * chunk, (blk + 1) * chunk) with
// chunk a multiple of 128.  w's chunk is staged once in shared memory; warp q takes slots j = 1 + q,
// 1 + q + nwarps, ...: its lanes stream the slot's chunk with 128-bit loads (all of a slot's loads in
// flight at once), multiply by w from shared memory and finish with one shuffle reduction per slot.
// One pass reads each filled slot once, with no block-wide barrier per slot.
__global__ void __launch_bounds__(256) k_lz_project1(const float* __restrict__ basis, const float* __restrict__ w,
                                                     int64_t n, int64_t chunk, int64_t slots, LzState<float> s) {
  if (*s.done) return;
  extern __shared__ float4 wsm[];
  const int i = *s.step;
  const int64_t r0 = (int64_t)blockIdx.x * chunk;
  const int64_t r1 = r0 + chunk < n ? r0 + chunk : n;
  const int64_t n4 = (r1 - r0) / 4;  // float4 groups in this chunk (n and chunk are multiples of 4)
  const float4* w4 = reinterpret_cast<const float4*>(w + r0);
  for (int64_t u = threadIdx.x; u < n4; u += blockDim.x) wsm[u] = w4[u];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float* out = s.hpart + (int64_t)blockIdx.x * slots;
  for (int j = 1 + warp; j <= i; j += nw) {
    const float4* v4 = reinterpret_cast<const float4*>(basis + (int64_t)j * n + r0);
    float acc0 = 0.f, acc1 = 0.f;
    int64_t u = lane;
#pragma unroll 4
    for (; u + 32 < n4; u += 64) {
      const float4 a = __ldg(v4 + u), b = __ldg(v4 + u + 32);
      const float4 x = wsm[u], y = wsm[u + 32];
      acc0 += a.x * x.x + a.y * x.y + a.z * x.z + a.w * x.w;
      acc1 += b.x * y.x + b.y * y.y + b.z * y.z + b.w * y.w;
    }
    for (; u < n4; u += 32) {
      const float4 a = __ldg(v4 + u);
      const float4 x = wsm[u];
      acc0 += a.x * x.x + a.y * x.y + a.z * x.z + a.w * x.w;
    }
    const float t = warp_sum(acc0 + acc1);
    if (lane == 0) out[j] = t;
  }
}

// Block form (bs in {4, 8, 16, 32, 64, 128}, FP32): block blk owns rows [blk * chunk, ...), i.e. one
// contiguous run of chunk * bs floats per slot.  w's run is staged in shared memory; warp q takes
// slots j = 1 + q, 1 + q + nwarps, ...; a warp step covers 128 consecutive floats, so lane l always
// holds column quad l % (bs / 4) and accumulates it in a float4; a shuffle tree over the lanes of
// the same quad finishes the slot.  128-bit streams, no block-wide barrier per slot.
__global__ void __launch_bounds__(512) k_lz_projectq(const float* __restrict__ basis, const float* __restrict__ w,
                                                     int64_t n, int64_t bs, int64_t chunk, int64_t slots,
                                                     LzState<float> s) {
  if (*s.done) return;
  extern __shared__ float4 wsm[];
  const int i = *s.step;
  const int64_t r0 = (int64_t)blockIdx.x * chunk;
  const int64_t r1 = r0 + chunk < n ? r0 + chunk : n;
  const int64_t n4 = (r1 - r0) * bs / 4;  // float4 units of this block's run
  const float4* w4 = reinterpret_cast<const float4*>(w + r0 * bs);
  for (int64_t u = threadIdx.x; u < n4; u += blockDim.x) wsm[u] = w4[u];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int qd = (int)(bs / 4);  // column quads per row: a power of two in [1, 32]
  float* out = s.hpart + (int64_t)blockIdx.x * slots * bs;
  for (int j = 1 + warp; j <= i; j += nw) {
    const float4* v4 = reinterpret_cast<const float4*>(basis + (int64_t)j * n * bs + r0 * bs);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f), acc2 = make_float4(0.f, 0.f, 0.f, 0.f);
    int64_t u = lane;
#pragma unroll 4
    for (; u + 32 < n4; u += 64) {
      const float4 a = __ldg(v4 + u), b = __ldg(v4 + u + 32);
      const float4 x = wsm[u], y = wsm[u + 32];
      acc.x += a.x * x.x; acc.y += a.y * x.y; acc.z += a.z * x.z; acc.w += a.w * x.w;
      acc2.x += b.x * y.x; acc2.y += b.y * y.y; acc2.z += b.z * y.z; acc2.w += b.w * y.w;
    }
    for (; u < n4; u += 32) {
      const float4 a = __ldg(v4 + u);
      const float4 x = wsm[u];
      acc.x += a.x * x.x; acc.y += a.y * x.y; acc.z += a.z * x.z; acc.w += a.w * x.w;
    }
    acc.x += acc2.x; acc.y += acc2.y; acc.z += acc2.z; acc.w += acc2.w;
    for (int o = 16; o >= qd; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
      acc.w += __shfl_xor_sync(0xffffffffu, acc.w, o);
    }
    if (lane < qd) reinterpret_cast<float4*>(out + (int64_t)j * bs)[lane] = acc;
  }
}

// h[j][b] = sum over blocks of hpart  (one warp per (j, b): lanes take strided blocks, then a
// shuffle tree; a thread per (j, b) would wait on nblk dependent loads)
template <class T>
__global__ void k_lz_reduce_h(int nblk, int64_t bs, int64_t slots, LzState<T> s) {
  if (*s.done) return;
  const int i = *s.step;
  const int64_t total = (int64_t)(i + 1) * bs;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = warp0; u < total; u += nwarps) {
    T acc = T(0);
    if (u >= bs)  // slot 0 is the zero vector
      for (int q = lane; q < nblk; q += 32) acc += s.hpart[(int64_t)q * slots * bs + u];
    acc = warp_sum(acc);
    if (lane == 0) s.hbuf[u] = acc;
  }
}

// w -= sum_j V[j] h[j]  (128-bit accesses for FP32 when bs is a multiple of 4)
template <class T>
__global__ void k_lz_subtract(const T* basis, T* w, int64_t n, int64_t bs, LzState<T> s) {
  if (*s.done) return;
  const int i = *s.step;
  if constexpr (std::is_same<T, float>::value) {
    if (bs == 1 && n % 4 == 0) {  // one coefficient per slot, four rows per 128-bit access
      const int64_t n4 = n / 4;
      float4* w4 = reinterpret_cast<float4*>(w);
      for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n4; u += (int64_t)gridDim.x * blockDim.x) {
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
        for (int j = 1; j <= i; ++j) {
          const float4 v = __ldg(reinterpret_cast<const float4*>(basis + (int64_t)j * n) + u);
          const float h = s.hbuf[j];
          acc.x += v.x * h;
          acc.y += v.y * h;
          acc.z += v.z * h;
          acc.w += v.w * h;
        }
        float4 wv = w4[u];
        wv.x -= acc.x;
        wv.y -= acc.y;
        wv.z -= acc.z;
        wv.w -= acc.w;
        w4[u] = wv;
      }
      return;
    }
    if (bs % 4 == 0) {
      const int64_t n4 = n * bs / 4;
      float4* w4 = reinterpret_cast<float4*>(w);
      for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n4; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = (4 * u) % bs;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int j = 1; j <= i; ++j) {
          const float4 v = reinterpret_cast<const float4*>(basis + (int64_t)j * n * bs)[u];
          const float* h = s.hbuf + (int64_t)j * bs + b;
          acc.x += v.x * h[0];
          acc.y += v.y * h[1];
          acc.z += v.z * h[2];
          acc.w += v.w * h[3];
        }
        float4 wv = w4[u];
        wv.x -= acc.x;
        wv.y -= acc.y;
        wv.z -= acc.z;
        wv.w -= acc.w;
        w4[u] = wv;
      }
      return;
    }
  }
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * bs; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = u % bs;
    T acc = T(0);
    for (int j = 1; j <= i; ++j) acc += basis[(int64_t)j * n * bs + u] * s.hbuf[(int64_t)j * bs + b];
    w[u] -= acc;
  }
}

// subdiag[b][i] = |w| ; i += 1 ; stop test of lanczos_fact.cond_fun
template <class T>
__global__ void __launch_bounds__(256) k_lz_finish(const T* w, int64_t n, int64_t bs, T* subdiag, int max_iters,
                                                   double tol, LzState<T> s) {
  if (*s.done) return;
  __shared__ T smem[256];
  lz_colsum<T>(n, bs, w, w, s.npart + (int64_t)blockIdx.x * bs, smem);
  if (lz_last_block(s.counters + 2)) {
    __shared__ int s_any;
    __shared__ T tot[kLzStage], red[32];
    lz_stage(s.npart, gridDim.x, bs, tot, red, smem);
    const int i = *s.step;
    if (threadIdx.x == 0) s_any = 0;
    __syncthreads();
    for (int64_t b = threadIdx.x; b < bs; b += blockDim.x) {
      const T nv = sqrt(lz_total(s.npart, gridDim.x, bs, b, tot));
      subdiag[b * (max_iters + 1) + i] = nv;
      const T first = subdiag[b * (max_iters + 1) + 1];
      if (nv > (T)tol * first) atomicOr(&s_any, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int ni = i + 1;
      *s.step = ni;
      *s.done = !(ni <= max_iters && (s_any || ni <= 1));
      s.counters[2] = 0;
    }
  }
}

// V[1] = V0 / |V0| (init_lanczos) -- norm partials then scale
template <class T>
__global__ void k_lz_init_copy(const T* v0, int64_t ldv0, T* v1, int64_t n, int64_t bs) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * bs; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = u / bs, b = u % bs;
    v1[u] = v0[r * ldv0 + b];
  }
}

template <class T>
__global__ void k_lz_set_state(LzState<T> s, int max_iters) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *s.step = 1;
    *s.done = !(1 <= max_iters);
  }
}

// out[r][b] = sum_{j<m} basis[j+1][r][b] * coef[b * ldc + j]
template <class T>
__global__ void k_basis_combine(const T* basis, int64_t n, int64_t bs, int m, const T* coef, int64_t ldc, T* out) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * bs; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = u % bs;
    T acc = T(0);
    for (int j = 0; j < m; ++j) acc += basis[(int64_t)(j + 1) * n * bs + u] * coef[b * ldc + j];
    out[u] = acc;
  }
}

// ---------------------------------------------------------------------------------------------
// Symmetric tridiagonal eigensolver (batched): implicit QL with Wilkinson shifts, one CTA per
// matrix, in R = double or float.  The matrix is first scaled by a power of two (exact) so that its
// largest entry lies in [0.5, 1): the sweep below forms squares without overflow checks in either
// precision.  Thread 0 runs the scalar recurrence; each QL sweep's Givens rotations are recorded in
// shared memory and then applied by all threads to their own rows of the eigenvector matrix (rows are
// independent under column rotations).  Row 0 alone (Gauss weights) is tracked by thread 0.
// `rec` (optional, with evecs == nullptr): every Givens rotation (c, s) on columns (i, i+1) is
// appended in generation order to rec[sys * cap ...] / rec_i, the count to rec_n[sys] (-1 when cap
// was exceeded), and the sorting permutation to rec_perm[sys * m ...]; k_tridiag_apply replays them.
template <class R> struct TriTraits;
template <> struct TriTraits<double> {
  using R2 = double2;
  static constexpr double eps = 2.220446049250313e-16;
  __device__ static double rsq(double x) { return rsqrt(x); }
  __device__ static double hyp(double a, double b) { return hypot(a, b); }
  __device__ static double2 pack(double c, double s) { return make_double2(c, s); }
  __device__ static double ab(double x) { return fabs(x); }
  __device__ static double mx(double x, double y) { return fmax(x, y); }
  __device__ static double fm(double x, double y, double z) { return fma(x, y, z); }
  __device__ static double fr(double x, int* ex) { return frexp(x, ex); }
  __device__ static double ld(double x, int ex) { return ldexp(x, ex); }
};
template <> struct TriTraits<float> {
  using R2 = float2;
  static constexpr float eps = 1.1920928955078125e-7f;
  __device__ static float rsq(float x) { return rsqrtf(x); }
  __device__ static float hyp(float a, float b) { return hypotf(a, b); }
  __device__ static float2 pack(float c, float s) { return make_float2(c, s); }
  __device__ static float ab(float x) { return fabsf(x); }
  __device__ static float mx(float x, float y) { return fmaxf(x, y); }
  __device__ static float fm(float x, float y, float z) { return fmaf(x, y, z); }
  __device__ static float fr(float x, int* ex) { return frexpf(x, ex); }
  __device__ static float ld(float x, int ex) { return ldexpf(x, ex); }
};

// Strict total order for the eigenvalue sort: ascending, NaN last, ties by index.
template <class R>
__device__ inline bool tri_before(R x, int64_t i, R y, int64_t j) {
  const bool nx = isnan(x), ny = isnan(y);
  if (nx != ny) return ny;
  if (!nx && x != y) return x < y;
  return i < j;
}

template <class R>
__global__ void k_tridiag_ql(const R* A, const R* Bv, int64_t m, R* evals, R* first_row, R* evecs,
                             int32_t* status, typename TriTraits<R>::R2* rec = nullptr, int32_t* rec_i = nullptr,
                             int32_t* rec_n = nullptr, int32_t* rec_perm = nullptr, int64_t cap = 0) {
  using TT = TriTraits<R>;
  extern __shared__ __align__(16) unsigned char tri_smem[];
  R* d = reinterpret_cast<R*>(tri_smem);  // m
  R* e = d + m;                           // m
  R* z0 = e + m;                          // m (row 0 of Z)
  R* rc = z0 + m;                         // m rotation cosines
  R* rs = rc + m;                         // m rotation sines
  int* perm = reinterpret_cast<int*>(rs + m);  // m
  __shared__ int s_cmd, s_lo, s_hi, s_fail;
  __shared__ R s_amax[32];
  const int64_t sys = blockIdx.x;
  const R* a = A + sys * m;
  const R* b = Bv + sys * m;
  R* Z = evecs ? evecs + sys * m * m : nullptr;
  R amax = R(0);
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const R ai = a[i], bi = (i + 1 < m) ? b[i] : R(0);
    amax = TT::mx(amax, TT::mx(TT::ab(ai), TT::ab(bi)));
  }
  for (int o = 16; o > 0; o >>= 1) amax = TT::mx(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((threadIdx.x & 31) == 0) s_amax[threadIdx.x >> 5] = amax;
  __syncthreads();
  if (threadIdx.x == 0) {
    R t = R(0);
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = TT::mx(t, s_amax[w]);
    s_amax[0] = t;
    s_fail = 0;
  }
  __syncthreads();
  // 2^-e with amax = f * 2^e, f in [0.5, 1): exact scaling, undone on the eigenvalues
  int ex = 0;
  const R amx = s_amax[0];
  if (amx > R(0) && isfinite(amx)) TT::fr(amx, &ex);
  const R scale = TT::ld(R(1), -ex), unscale = TT::ld(R(1), ex);
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    d[i] = a[i] * scale;
    e[i] = (i + 1 < m) ? b[i] * scale : R(0);
    z0[i] = (i == 0) ? R(1) : R(0);
  }
  if (Z)
    for (int64_t u = threadIdx.x; u < m * m; u += blockDim.x) Z[u] = (u / m == u % m) ? R(1) : R(0);
  __syncthreads();
  int l = 0, iter = 0;
  int64_t nrec = 0;
  typename TT::R2* my_rec = rec ? rec + sys * cap : nullptr;
  int32_t* my_rec_i = rec ? rec_i + sys * cap : nullptr;
  while (true) {
    // thread 0: one QL sweep (or decide to move on)
    if (threadIdx.x == 0) {
      s_cmd = 0;  // 0 = nothing to apply, 1 = apply rotations [s_lo, s_hi), 2 = finished
      while (l < m) {
        int mm = l;
        for (; mm < m - 1; ++mm) {
          const R dd = TT::ab(d[mm]) + TT::ab(d[mm + 1]);
          if (TT::ab(e[mm]) <= TT::eps * dd) break;
        }
        if (mm == l) { ++l; iter = 0; continue; }
        if (iter++ >= 60) { s_fail = 1; ++l; iter = 0; continue; }
        R g = (d[l + 1] - d[l]) / (R(2) * e[l]);
        R r = TT::hyp(g, R(1));
        g = d[mm] - d[l] + e[l] / (g + (g >= R(0) ? TT::ab(r) : -TT::ab(r)));
        R s = R(1), c = R(1), p = R(0);
        int i = mm - 1;
        bool underflow = false;
        // The sweep is one dependent chain on this thread: the operands of step i - 1 (e[i-1], d[i-1],
        // z0[i-1]), which step i does not modify, are loaded ahead, d[i] / z0[i] are carried in
        // registers, and each rotation takes one reciprocal square root instead of a hypot and two
        // divisions (|f|, |g| are bounded by a small multiple of the scaled matrix's norm).
        R ei = e[i], di1 = d[i + 1], di = d[i], zi1 = z0[i + 1];
        for (; i >= l; --i) {
          const R e_nx = i > l ? e[i - 1] : R(0);
          const R d_nx = i > l ? d[i - 1] : R(0);
          const R zi = z0[i];
          const R f = s * ei, bb = c * ei;
          const R q = TT::fm(f, f, g * g);
          if (q == R(0)) {
            e[i + 1] = R(0);
            d[i + 1] = di1 - p;
            e[mm] = R(0);
            underflow = true;
            break;
          }
          const R ri = TT::rsq(q);
          e[i + 1] = q * ri;
          s = f * ri;
          c = g * ri;
          g = di1 - p;
          r = (di - g) * s + R(2) * c * bb;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - bb;
          rc[i] = c;
          rs[i] = s;
          if (my_rec) {
            if (nrec < cap) {
              my_rec[nrec] = TT::pack(c, s);
              my_rec_i[nrec] = i;
            }
            ++nrec;
          }
          z0[i + 1] = s * zi + c * zi1;
          const R zi_new = c * zi - s * zi1;
          z0[i] = zi_new;
          ei = e_nx;
          di1 = di;
          di = d_nx;
          zi1 = zi_new;
        }
        if (underflow) {
          s_lo = i + 1;
          s_hi = mm;
        } else {
          d[l] -= p;
          e[l] = g;
          e[mm] = R(0);
          s_lo = l;
          s_hi = mm;
        }
        s_cmd = 1;
        break;
      }
      if (l >= m) s_cmd = (s_cmd == 1) ? 1 : 2;
    }
    __syncthreads();
    const int cmd = s_cmd;
    if (cmd == 1 && Z) {
      // rotations were generated for i = hi-1 down to lo, apply in that order
      const int lo = s_lo, hi = s_hi;
      for (int64_t row = threadIdx.x; row < m; row += blockDim.x) {
        R* zr = Z + row * m;
        for (int i = hi - 1; i >= lo; --i) {
          const R c = rc[i], s = rs[i];
          const R f = zr[i + 1];
          zr[i + 1] = s * zr[i] + c * f;
          zr[i] = c * zr[i] - s * f;
        }
      }
    }
    __syncthreads();
    if (cmd == 2) break;
    if (cmd == 0) break;
  }
  // ascending order by rank (ties by index): every thread ranks its own entries, O(m) each
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    const R dj = d[j];
    int rank = 0;
    for (int64_t i = 0; i < m; ++i) rank += tri_before(d[i], i, dj, j);
    perm[rank] = (int)j;
  }
  __syncthreads();
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    evals[sys * m + j] = d[perm[j]] * unscale;
    if (first_row) first_row[sys * m + j] = Z ? Z[perm[j]] : z0[perm[j]];
    if (rec_perm) rec_perm[sys * m + j] = perm[j];
  }
  if (rec && threadIdx.x == 0) rec_n[sys] = nrec <= cap ? (int32_t)nrec : -1;
  __syncthreads();
  if (Z) {
    R* tmp = rc;  // reuse as a row buffer
    for (int64_t row = 0; row < m; ++row) {
      for (int64_t j = threadIdx.x; j < m; j += blockDim.x) tmp[j] = Z[row * m + perm[j]];
      __syncthreads();
      for (int64_t j = threadIdx.x; j < m; j += blockDim.x) Z[row * m + j] = tmp[j];
      __syncthreads();
    }
  }
  if (threadIdx.x == 0 && status) status[sys] = s_fail;
}

// Replays the recorded rotations on the eigenvector matrix: Z starts as the identity, each thread
// owns one row (rows are independent), held in shared memory as zs[col][lane] (conflict-free);
// every rotation acts on columns (i, i+1).  Output columns follow the sorted eigenvalues.
constexpr int kRotRows = 32;
template <class R>
__global__ void __launch_bounds__(kRotRows) k_tridiag_apply(const typename TriTraits<R>::R2* rec,
                                                            const int32_t* rec_i, const int32_t* rec_n,
                                                            const int32_t* rec_perm, int64_t m, int64_t cap,
                                                            R* evecs) {
  extern __shared__ __align__(16) unsigned char rot_smem[];
  R* zs = reinterpret_cast<R*>(rot_smem);  // m x kRotRows
  const int64_t sys = blockIdx.y;
  const int t = threadIdx.x;
  const int64_t row = (int64_t)blockIdx.x * kRotRows + t;
  const int32_t nr = rec_n[sys];
  if (nr < 0) return;  // the recording overflowed: the in-kernel path produced Z
  for (int64_t i = 0; i < m; ++i) zs[i * kRotRows + t] = (row == i) ? R(1) : R(0);
  const typename TriTraits<R>::R2* r = rec + sys * cap;
  const int32_t* ri = rec_i + sys * cap;
  for (int32_t q = 0; q < nr; ++q) {
    const auto cs = r[q];
    const int i = ri[q];
    const R zi = zs[i * kRotRows + t], f = zs[(i + 1) * kRotRows + t];
    zs[(i + 1) * kRotRows + t] = cs.y * zi + cs.x * f;
    zs[i * kRotRows + t] = cs.x * zi - cs.y * f;
  }
  if (row < m) {
    R* out = evecs + sys * m * m + row * m;
    const int32_t* perm = rec_perm + sys * m;
    for (int64_t j = 0; j < m; ++j) out[j] = zs[perm[j] * kRotRows + t];
  }
}

// ---------------------------------------------------------------------------------------------
// host

static int lz_blocks(int64_t n, int64_t bs) {
  const int64_t want = ceil_div(n * bs, 1024);
  const int64_t cap = (int64_t)num_sms() * 4;
  return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

template <class T>
static LzState<T> lz_carve(Bump& ws, int64_t bs, int32_t max_iters, int nb) {
  LzState<T> s;
  const int64_t slots = (int64_t)max_iters + 2;
  s.nrm = ws.take<T>(bs);
  s.hbuf = ws.take<T>(slots * bs);
  s.hpart = ws.take<T>((size_t)nb * slots * bs);
  s.npart = ws.take<T>((size_t)nb * bs);
  s.done = ws.take<int>(4);
  s.step = ws.take<int>(4);
  s.counters = ws.take<unsigned int>(8);
  return s;
}

template <class T>
static int lanczos_t(const colagb_op* A, const T* V0, int64_t ldv0, int64_t bs, const colagb_lanczos_params& prm,
                     T* basis, T* diag, T* subdiag, int32_t* steps, void* workspace, size_t ws_bytes,
                     cudaStream_t st) {
  const int64_t n = A->nodes[A->root].rows;
  const int m = prm.max_iters;
  const int64_t slots = (int64_t)m + 2;
  const int nb = lz_blocks(n, bs);
  Bump ws(workspace, ws_bytes);
  LzState<T> s = lz_carve<T>(ws, bs, m, nb);
  size_t opb = 0;
  COLAGB_TRY(colagb_matmat_workspace_bytes(A, bs, &opb));
  void* opws = ws.take<char>(opb > 0 ? opb : 1);
  if (workspace == nullptr || ws.overflow())
    return fail(COLAGB_ERR_WORKSPACE, "colagb_lanczos: workspace too small (need " + std::to_string(ws.peak) + ")");
  const int eg = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n * bs, 256), 1), (int64_t)num_sms() * 8);
  const size_t blk = (size_t)n * bs;
  COLAGB_CUDA(cudaMemsetAsync(basis, 0, sizeof(T) * blk * slots, st));
  COLAGB_CUDA(cudaMemsetAsync(diag, 0, sizeof(T) * bs * m, st));
  COLAGB_CUDA(cudaMemsetAsync(subdiag, 0, sizeof(T) * bs * (m + 1), st));
  COLAGB_CUDA(cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned int), st));
  k_lz_set_state<T><<<1, 32, 0, st>>>(s, m);
  // V[1] = V0 / |V0|
  T* v1 = basis + blk;
  k_lz_init_copy<T><<<eg, 256, 0, st>>>(V0, ldv0, v1, n, bs);
  k_lz_norm<T><<<nb, 256, 0, st>>>(v1, n, bs, s);
  k_lz_scale<T><<<eg, 256, 0, st>>>(v1, n, bs, s);
  COLAGB_CUDA(cudaGetLastError());
  const int every = prm.check_every > 0 ? prm.check_every : 8;
  // single-vector FP32 runs project with k_lz_project1 (w's chunk in shared memory, a warp per slot)
  bool p1 = false;
  int64_t chunk = 0;
  int nb1 = nb;
  bool pq = false;  // bs in {4, ..., 128}: k_lz_projectq
  if constexpr (std::is_same<T, float>::value) {
    if (bs == 1 && n % 4 == 0 && (uintptr_t)basis % 16 == 0) {
      chunk = ceil_div(ceil_div(n, nb), 128) * 128;
      if (chunk * (int64_t)sizeof(float) <= 160 * 1024) {
        p1 = true;
        nb1 = (int)ceil_div(n, chunk);
        COLAGB_CUDA(cudaFuncSetAttribute(k_lz_project1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(chunk * sizeof(float))));
      }
    } else if (bs >= 4 && bs <= 128 && (bs & (bs - 1)) == 0 && (uintptr_t)basis % 16 == 0) {
      // rows per block so that a block's run is a whole number of 128-float warp steps
      const int64_t rstep = 128 / bs;
      chunk = ceil_div(ceil_div(n, nb), rstep) * rstep;
      if (chunk * bs * (int64_t)sizeof(float) <= 160 * 1024) {
        pq = true;
        nb1 = (int)ceil_div(n, chunk);
        COLAGB_CUDA(cudaFuncSetAttribute(k_lz_projectq, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(chunk * bs * sizeof(float))));
      }
    }
  }
  int host_step = 1;  // the step index the next launch group starts at (upper bound)
  int hdone = 0;
  while (true) {
    for (int q = 0; q < every && host_step <= m; ++q, ++host_step) {
      const int i = host_step;  // kernels read the device step; host_step picks the basis slots
      T* vi = basis + (size_t)i * blk;
      T* vim1 = basis + (size_t)(i - 1) * blk;
      T* w = basis + (size_t)(i + 1) * blk;
      k_lz_norm<T><<<nb, 256, 0, st>>>(vi, n, bs, s);
      k_lz_scale<T><<<eg, 256, 0, st>>>(vi, n, bs, s);
      Bump ow(opws, opb > 0 ? opb : 1);
      COLAGB_TRY(op_apply<T>(A, A->root, vi, bs, 0, w, bs, 0, bs, 1, T(1), T(0), ow, s.done, st));
      k_lz_alpha<T><<<nb, 256, 0, st>>>(w, vi, n, bs, diag, m, s);
      k_lz_three_term<T><<<eg, 256, 0, st>>>(w, vi, vim1, n, bs, diag, subdiag, m, s);
      for (int pass = 0; pass < 2; ++pass) {
        if constexpr (std::is_same<T, float>::value) {
          if (p1)
            k_lz_project1<<<nb1, 256, chunk * sizeof(float), st>>>(basis, w, n, chunk, slots, s);
          else if (pq)
            k_lz_projectq<<<nb1, 512, chunk * bs * sizeof(float), st>>>(basis, w, n, bs, chunk, slots, s);
          else
            k_lz_project<T><<<nb, 256, 0, st>>>(basis, w, n, bs, slots, s);
        } else {
          k_lz_project<T><<<nb, 256, 0, st>>>(basis, w, n, bs, slots, s);
        }
        k_lz_reduce_h<T><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div((int64_t)(i + 1) * bs, 8), 4096)),
                           256, 0, st>>>((p1 || pq) ? nb1 : nb, bs, slots, s);
        k_lz_subtract<T><<<eg, 256, 0, st>>>(basis, w, n, bs, s);
      }
      k_lz_finish<T><<<nb, 256, 0, st>>>(w, n, bs, subdiag, m, prm.tol, s);
      COLAGB_CUDA(cudaGetLastError());
    }
    COLAGB_CUDA(cudaMemcpyAsync(&hdone, s.done, sizeof(int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaStreamSynchronize(st));
    if (hdone || host_step > m) break;
  }
  int dstep = 0;
  COLAGB_CUDA(cudaMemcpyAsync(&dstep, s.step, sizeof(int), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaStreamSynchronize(st));
  *steps = dstep;
  return COLAGB_OK;
}


// ---- Arnoldi (arnoldi.py:303-334) on the same basis slots: Q[j] lives in slot j + 1 ----------
// H is (bs, max_iters + 1, max_iters) row-major; column idx = step - 1 collects the projection
// coefficients of both Gram-Schmidt passes and, below them, |w|.
template <class T>
__global__ void k_ar_accum_h(T* H, int64_t bs, int max_iters, int first_pass, LzState<T> s) {
  if (*s.done) return;
  const int i = *s.step;  // slots 1..i were projected out: rows 0..i-1 of column i-1
  const int idx = i - 1;
  const int64_t total = (int64_t)i * bs;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = u / bs, b = u % bs;
    T* h = H + (b * (max_iters + 1) + j) * max_iters + idx;
    const T c = s.hbuf[(j + 1) * bs + b];
    *h = first_pass ? c : *h + c;
  }
}

// w /= max(|w|, tol / 2)  (the new basis vector; |w| from k_lz_norm)
template <class T>
__global__ void k_ar_scale_clip(T* w, int64_t n, int64_t bs, double tol, LzState<T> s) {
  if (*s.done) return;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n * bs; u += (int64_t)gridDim.x * blockDim.x) {
    const T nv = s.nrm[u % bs];
    w[u] = w[u] / (nv > (T)(tol / 2) ? nv : (T)(tol / 2));
  }
}

// H[b][idx + 1][idx] = |w| ; idx += 1 ; stop test of arnoldi_fact.cond_fun:
// continue while idx < max_iters and (any |w| > tol * H[b][1][0] or idx <= 0)
template <class T>
__global__ void k_ar_finish(T* H, int64_t bs, int max_iters, double tol, LzState<T> s) {
  if (*s.done) return;
  __shared__ int s_any;
  const int i = *s.step;
  const int idx = i - 1;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  for (int64_t b = threadIdx.x; b < bs; b += blockDim.x) {
    const T nv = s.nrm[b];
    H[(b * (max_iters + 1) + idx + 1) * max_iters + idx] = nv;
    const T h10 = H[(b * (max_iters + 1) + 1) * max_iters + 0];
    if (nv > (T)tol * h10) atomicOr(&s_any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nidx = idx + 1;
    *s.step = nidx + 1;
    *s.done = !(nidx < max_iters && (s_any || nidx <= 0));
  }
}

template <class T>
static int arnoldi_t(const colagb_op* A, const T* V0, int64_t ldv0, int64_t bs, const colagb_lanczos_params& prm,
                     T* basis, T* H, int32_t* steps, void* workspace, size_t ws_bytes, cudaStream_t st) {
  const int64_t n = A->nodes[A->root].rows;
  const int m = prm.max_iters;
  const int64_t slots = (int64_t)m + 2;
  const int nb = lz_blocks(n, bs);
  Bump ws(workspace, ws_bytes);
  LzState<T> s = lz_carve<T>(ws, bs, m, nb);
  size_t opb = 0;
  COLAGB_TRY(colagb_matmat_workspace_bytes(A, bs, &opb));
  void* opws = ws.take<char>(opb > 0 ? opb : 1);
  if (workspace == nullptr || ws.overflow())
    return fail(COLAGB_ERR_WORKSPACE, "colagb_arnoldi: workspace too small (need " + std::to_string(ws.peak) + ")");
  const int eg = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n * bs, 256), 1), (int64_t)num_sms() * 8);
  const size_t blk = (size_t)n * bs;
  COLAGB_CUDA(cudaMemsetAsync(basis, 0, sizeof(T) * blk * slots, st));
  COLAGB_CUDA(cudaMemsetAsync(H, 0, sizeof(T) * bs * (m + 1) * (m > 0 ? m : 1), st));
  COLAGB_CUDA(cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned int), st));
  k_lz_set_state<T><<<1, 32, 0, st>>>(s, m);
  T* q0 = basis + blk;  // Q[0] = V0 / |V0|
  k_lz_init_copy<T><<<eg, 256, 0, st>>>(V0, ldv0, q0, n, bs);
  k_lz_norm<T><<<nb, 256, 0, st>>>(q0, n, bs, s);
  k_lz_scale<T><<<eg, 256, 0, st>>>(q0, n, bs, s);
  COLAGB_CUDA(cudaGetLastError());
  const int every = prm.check_every > 0 ? prm.check_every : 8;
  int host_step = 1;  // slot of Q[idx] for the next step (idx = host_step - 1)
  int hdone = 0;
  while (true) {
    for (int q = 0; q < every && host_step <= m; ++q, ++host_step) {
      const int i = host_step;
      T* qi = basis + (size_t)i * blk;
      T* w = basis + (size_t)(i + 1) * blk;
      Bump ow(opws, opb > 0 ? opb : 1);
      COLAGB_TRY(op_apply<T>(A, A->root, qi, bs, 0, w, bs, 0, bs, 1, T(1), T(0), ow, s.done, st));
      for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, twice
        k_lz_project<T><<<nb, 256, 0, st>>>(basis, w, n, bs, slots, s);
        k_lz_reduce_h<T><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div((int64_t)(i + 1) * bs, 8), 4096)),
                           256, 0, st>>>(nb, bs, slots, s);
        k_ar_accum_h<T><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div((int64_t)i * bs, 256), 4096)), 256,
                          0, st>>>(H, bs, m, pass == 0, s);
        k_lz_subtract<T><<<eg, 256, 0, st>>>(basis, w, n, bs, s);
      }
      k_lz_norm<T><<<nb, 256, 0, st>>>(w, n, bs, s);
      k_ar_scale_clip<T><<<eg, 256, 0, st>>>(w, n, bs, prm.tol, s);
      k_ar_finish<T><<<1, 256, 0, st>>>(H, bs, m, prm.tol, s);
      COLAGB_CUDA(cudaGetLastError());
    }
    COLAGB_CUDA(cudaMemcpyAsync(&hdone, s.done, sizeof(int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaStreamSynchronize(st));
    if (hdone || host_step > m) break;
  }
  int dstep = 0;
  COLAGB_CUDA(cudaMemcpyAsync(&dstep, s.step, sizeof(int), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaStreamSynchronize(st));
  *steps = dstep - 1;  // Arnoldi steps taken (idx)
  return COLAGB_OK;
}
}  // namespace colagb

using namespace colagb;

extern "C" int colagb_lanczos_workspace_bytes(const colagb_op* A, int64_t bs, int32_t max_iters, size_t* bytes) {
  if (!A || !bytes || bs < 1 || max_iters < 0) return fail(COLAGB_ERR_INVALID, "colagb_lanczos_workspace_bytes: bad arguments");
  const int64_t n = A->nodes[A->root].rows;
  Bump ws = Bump::measuring();
  if (A->compute_dtype == COLAGB_F64) lz_carve<double>(ws, bs, max_iters, lz_blocks(n, bs));
  else lz_carve<float>(ws, bs, max_iters, lz_blocks(n, bs));
  size_t opb = 0;
  COLAGB_TRY(colagb_matmat_workspace_bytes(A, bs, &opb));
  ws.take<char>(opb > 0 ? opb : 1);
  *bytes = ws.peak;
  return COLAGB_OK;
}

extern "C" int colagb_lanczos(const colagb_op* A, const void* V0, int64_t ldv0, int64_t bs,
                              const colagb_lanczos_params* params, void* basis, void* diag, void* subdiag,
                              int32_t* steps, void* workspace, size_t workspace_bytes, void* stream) {
  if (!A || !params || !V0 || !basis || !diag || !subdiag || !steps)
    return fail(COLAGB_ERR_INVALID, "colagb_lanczos: null argument");
  const colagb_op_node& r = A->nodes[A->root];
  if (r.rows != r.cols) return fail(COLAGB_ERR_INVALID, "colagb_lanczos: operator must be square");
  if (bs < 1 || ldv0 < bs || params->max_iters < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_lanczos: bad bs / ldv0 / max_iters");
  cudaStream_t st = as_stream(stream);
  if (A->compute_dtype == COLAGB_F64)
    return lanczos_t<double>(A, static_cast<const double*>(V0), ldv0, bs, *params, static_cast<double*>(basis),
                             static_cast<double*>(diag), static_cast<double*>(subdiag), steps, workspace,
                             workspace_bytes, st);
  return lanczos_t<float>(A, static_cast<const float*>(V0), ldv0, bs, *params, static_cast<float*>(basis),
                          static_cast<float*>(diag), static_cast<float*>(subdiag), steps, workspace, workspace_bytes,
                          st);
}

extern "C" int colagb_basis_combine(const void* basis, int64_t n, int64_t bs, int32_t m, const void* coef,
                                    int64_t ldc, void* out, int32_t dtype, void* stream) {
  if (!basis || !coef || !out || n < 0 || bs < 1 || m < 0 || ldc < m)
    return fail(COLAGB_ERR_INVALID, "colagb_basis_combine: bad arguments");
  cudaStream_t st = as_stream(stream);
  const int eg = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(n * bs, 256), 1), (int64_t)num_sms() * 8);
  if (n * bs == 0) return COLAGB_OK;
  if (dtype == COLAGB_F64)
    k_basis_combine<double><<<eg, 256, 0, st>>>(static_cast<const double*>(basis), n, bs, m,
                                                 static_cast<const double*>(coef), ldc, static_cast<double*>(out));
  else if (dtype == COLAGB_F32)
    k_basis_combine<float><<<eg, 256, 0, st>>>(static_cast<const float*>(basis), n, bs, m,
                                                static_cast<const float*>(coef), ldc, static_cast<float*>(out));
  else
    return fail(COLAGB_ERR_UNSUPPORTED, "colagb_basis_combine: dtype must be F32 or F64");
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

// Rayleigh quotients of the computed eigenvectors in FP64: evals[j] = s_j^T T s_j / s_j^T s_j.  After an
// FP32 QL the eigenvalues carry the sweeps' accumulated rounding (a few FP32 ulps of |T|); the quotient
// of the FP32 eigenvector is off by the square of the vector's error, so this returns each eigenvalue
// to within FP32 rounding.  One thread per eigenvector; consecutive threads read consecutive columns.
template <class R>
__global__ void k_tridiag_rq(const R* A, const R* Bv, int64_t m, const R* evecs, R* evals) {
  const int64_t sys = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const R* a = A + sys * m;
  const R* b = Bv + sys * m;
  const R* Z = evecs + sys * m * m;
  double num = 0.0, den = 0.0, sp = 0.0, si = (double)Z[j];
  for (int64_t i = 0; i < m; ++i) {
    const double sn = i + 1 < m ? (double)Z[(i + 1) * m + j] : 0.0;
    double t = (double)a[i] * si + (i > 0 ? (double)b[i - 1] * sp : 0.0);
    if (i + 1 < m) t += (double)b[i] * sn;
    num += si * t;
    den += si * si;
    sp = si;
    si = sn;
  }
  if (den > 0.0) evals[sys * m + j] = (R)(num / den);
}

template <class R>
static int tridiag_eig(const R* a, const R* b, int64_t m, int64_t batch, R* evals, R* first_row, R* evecs,
                       int32_t* status, cudaStream_t st, const char* name) {
  using R2 = typename TriTraits<R>::R2;
  if (m < 0 || batch < 0 || (m * batch > 0 && (!a || !b || !evals))) return fail(COLAGB_ERR_INVALID, name);
  if (m * batch == 0) return COLAGB_OK;
  const size_t smem = (size_t)m * (5 * sizeof(R) + sizeof(int));
  if (smem > 200 * 1024) return fail(COLAGB_ERR_INVALID, "tridiagonal eigensolver: m too large");
  if (smem > 48 * 1024)
    COLAGB_CUDA(cudaFuncSetAttribute(k_tridiag_ql<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const size_t smem_rot = (size_t)m * kRotRows * sizeof(R);
  if (evecs && smem_rot <= 200 * 1024) {
    // eigenvectors: QL records its rotations (one thread generates them serially), then many CTAs
    // replay them on the rows of Z in shared memory; applying them to Z in global memory from the
    // same CTA, row per thread, cost ~95 % of the solve
    const int64_t cap = 6 * m * m + 64;
    void* buf = nullptr;
    const size_t bytes = (size_t)batch * cap * (sizeof(R2) + sizeof(int32_t)) +
                         (size_t)batch * (m + 1) * sizeof(int32_t);
    COLAGB_CUDA(cudaMallocAsync(&buf, bytes, st));
    R2* rec = static_cast<R2*>(buf);
    int32_t* rec_i = reinterpret_cast<int32_t*>(rec + batch * cap);
    int32_t* rec_n = rec_i + batch * cap;
    int32_t* rec_perm = rec_n + batch;
    k_tridiag_ql<R><<<(unsigned)batch, 128, smem, st>>>(a, b, m, evals, first_row, nullptr, status, rec, rec_i,
                                                        rec_n, rec_perm, cap);
    COLAGB_CUDA(cudaGetLastError());
    if (smem_rot > 48 * 1024)
      COLAGB_CUDA(cudaFuncSetAttribute(k_tridiag_apply<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rot));
    k_tridiag_apply<R><<<dim3((unsigned)ceil_div(m, (int64_t)kRotRows), (unsigned)batch), kRotRows, smem_rot, st>>>(
        rec, rec_i, rec_n, rec_perm, m, cap, evecs);
    COLAGB_CUDA(cudaGetLastError());
    std::vector<int32_t> hn(batch);
    COLAGB_CUDA(cudaMemcpyAsync(hn.data(), rec_n, batch * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaStreamSynchronize(st));
    bool overflow = false;
    for (int64_t q = 0; q < batch; ++q) overflow |= hn[q] < 0;
    COLAGB_CUDA(cudaFreeAsync(buf, st));
    if (!overflow) {
      if (std::is_same<R, float>::value) {
        k_tridiag_rq<R><<<dim3((unsigned)ceil_div(m, (int64_t)128), (unsigned)batch), 128, 0, st>>>(a, b, m, evecs, evals);
        COLAGB_CUDA(cudaGetLastError());
      }
      return COLAGB_OK;
    }
    // rare: more rotations than recorded -- recompute with Z updated inside the QL kernel
  }
  k_tridiag_ql<R><<<(unsigned)batch, 128, smem, st>>>(a, b, m, evals, first_row, evecs, status);
  COLAGB_CUDA(cudaGetLastError());
  if (evecs && std::is_same<R, float>::value) {
    k_tridiag_rq<R><<<dim3((unsigned)ceil_div(m, (int64_t)128), (unsigned)batch), 128, 0, st>>>(a, b, m, evecs, evals);
    COLAGB_CUDA(cudaGetLastError());
  }
  return COLAGB_OK;
}

extern "C" int colagb_tridiag_eig_f64(const double* a, const double* b, int64_t m, int64_t batch, double* evals,
                                      double* first_row, double* evecs, int32_t* status, void* stream) {
  return tridiag_eig<double>(a, b, m, batch, evals, first_row, evecs, status, as_stream(stream),
                             "colagb_tridiag_eig_f64: bad arguments");
}

extern "C" int colagb_tridiag_eig_f32(const float* a, const float* b, int64_t m, int64_t batch, float* evals,
                                      float* first_row, float* evecs, int32_t* status, void* stream) {
  return tridiag_eig<float>(a, b, m, batch, evals, first_row, evecs, status, as_stream(stream),
                            "colagb_tridiag_eig_f32: bad arguments");
}

extern "C" int colagb_arnoldi_workspace_bytes(const colagb_op* A, int64_t bs, int32_t max_iters, size_t* bytes) {
  return colagb_lanczos_workspace_bytes(A, bs, max_iters, bytes);
}

extern "C" int colagb_arnoldi(const colagb_op* A, const void* V0, int64_t ldv0, int64_t bs,
                              const colagb_lanczos_params* params, void* basis, void* H, int32_t* steps, void* workspace,
                              size_t workspace_bytes, void* stream) {
  if (!A || !params || !V0 || !basis || !H || !steps) return fail(COLAGB_ERR_INVALID, "colagb_arnoldi: null argument");
  const colagb_op_node& r = A->nodes[A->root];
  if (r.rows != r.cols) return fail(COLAGB_ERR_INVALID, "colagb_arnoldi: operator must be square");
  if (bs < 1 || ldv0 < bs || params->max_iters < 1)
    return fail(COLAGB_ERR_INVALID, "colagb_arnoldi: bad bs / ldv0 / max_iters");
  cudaStream_t st = as_stream(stream);
  if (A->compute_dtype == COLAGB_F64)
    return arnoldi_t<double>(A, static_cast<const double*>(V0), ldv0, bs, *params, static_cast<double*>(basis),
                             static_cast<double*>(H), steps, workspace, workspace_bytes, st);
  return arnoldi_t<float>(A, static_cast<const float*>(V0), ldv0, bs, *params, static_cast<float*>(basis),
                          static_cast<float*>(H), steps, workspace, workspace_bytes, st);
}
