// Tensor-core contraction for the Kronecker matvec on sm_103a: tcgen05.mma with the accumulator in
// tensor memory, operands brought into shared memory by TMA (cp.async.bulk.tensor), BF16 inputs and
// FP32 accumulation, and an optional three-product split that recovers FP32-level accuracy.
//
// Reference behaviour (cola/ops/operators.py:216-223): Kronecker._matmat contracts one factor M_i
// (r_i x c_i) at a time along its own axis of X viewed as (pre, c_i, post * k):
//     out[p, r, q] = sum_c M_i[r, c] * in[p, c, q].
// Here that is a batched GEMM  D_b (M x N) = A_b (M x K) . B (N x K)^T  with N = r_i, K = c_i and
//   * q = post * k > 1:  batch b = p, M = q, A_b[m][c] = in[p, c, m]   (the operand is transposed into
//     K-major BF16 by the split pass), out address  p * r * q + n * q + m;
//   * q == 1:           batch = 1, M = pre, A[m][c] = in[m, c] (already K-major), out  m * r + n.
// B = M_i as stored (row-major r x c is K-major).  Both operands are K-major with the 128-byte swizzle,
// the canonical UMMA layout.
//
// Precision: "bf16" runs one product per K step (BF16 inputs, FP32 accumulation); "bf16x3" splits every
// FP32 input into hi = bf16(v) and lo = bf16(v - hi) and accumulates hi.hi + hi.lo + lo.hi into the same
// tensor-memory accumulator (the dropped lo.lo term is ~2^-16 of each product).
//
// Kernel structure (one 128 x BN output tile per CTA, 128 threads):
//   warp 0 lane 0: TMA producer over a ring of kStages shared-memory stages (full / empty mbarriers);
//   warp 1: allocates BN tensor-memory columns; lane 0 issues the tcgen05.mma of each stage and commits
//           the stage's empty barrier, then the accumulator barrier;
//   warps 0-3: epilogue, tcgen05.ld of their 32 accumulator lanes, alpha * D + beta * out, global stores.
// Every mbarrier wait is bounded; a wait that gives up records an error word, marks its tile's output
// NaN, drains its own TMA copies (bounded), frees the tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "ops.cuh"

namespace colagb {

constexpr int kTcBM = 128;     // rows of a tile (tensor-memory lanes)
constexpr int kTcBK = 64;      // K per stage: one 128-byte swizzle row of BF16
constexpr int kTcThreads = 128;
constexpr long long kTcSpinLimit = 1LL << 22;  // try_wait rounds before a wait gives up (~seconds)

// ---------------------------------------------------------------------------------------------
// PTX wrappers

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of `parity` to complete; false if it did not within the limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kTcSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(bar)), "r"(c0), "r"(c1)
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with the 128-byte swizzle: rows of
// 128 bytes, 8-row groups 1024 bytes apart (SBO), leading offset unused for this layout, version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulator, both operands K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------------------------
// the GEMM kernel

struct TcArgs {
  int64_t M, N, K, batch;
  float* out;
  int64_t s_b, s_m, s_n;
  float alpha, beta;
  int a_batched;  // 1: A map is 3-D (K, M, batch); 0: 2-D (K, M)
  int* err;
  const int* skip;  // device flag: when set, the launch does nothing (finished CG iterations)
};

template <int BN, bool SPLIT>
struct TcCfg {
  static constexpr int kABytes = kTcBM * kTcBK * 2;  // 16 KB
  static constexpr int kBBytes = BN * kTcBK * 2;
  static constexpr int kStageBytes = (SPLIT ? 2 : 1) * (kABytes + kBBytes);
  static constexpr int kStages = (200 * 1024) / kStageBytes > 6 ? 6 : (200 * 1024) / kStageBytes;
  static constexpr int kSmem = kStages * kStageBytes + 1024 /* alignment */ + 256 /* barriers */;
  static constexpr uint32_t kTmemCols = BN < 32 ? 32 : BN;
};

template <int BN, bool SPLIT>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap map_a_hi, const __grid_constant__ CUtensorMap map_a_lo,
              const __grid_constant__ CUtensorMap map_b_hi, const __grid_constant__ CUtensorMap map_b_lo,
              const TcArgs args) {
  using Cfg = TcCfg<BN, SPLIT>;
  constexpr int S = Cfg::kStages;
  if (args.skip && *args.skip) return;  // uniform across the CTA: before any barrier or allocation
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + S * Cfg::kStageBytes);
  uint64_t* empty = full + S;
  uint64_t* accum = empty + S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
  int* s_fail = reinterpret_cast<int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t m0 = (int64_t)blockIdx.x * kTcBM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  const int64_t b = blockIdx.z;
  const int nkb = (int)((args.K + kTcBK - 1) / kTcBK);

  auto a_hi_s = [&](int s) { return base + s * Cfg::kStageBytes; };
  auto b_hi_s = [&](int s) { return base + s * Cfg::kStageBytes + Cfg::kABytes; };
  auto a_lo_s = [&](int s) { return base + s * Cfg::kStageBytes + Cfg::kABytes + Cfg::kBBytes; };
  auto b_lo_s = [&](int s) { return base + s * Cfg::kStageBytes + 2 * Cfg::kABytes + Cfg::kBBytes; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    *s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // whole warp: allocate the accumulator columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(Cfg::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- producer ----
    const uint32_t bytes = Cfg::kStageBytes;
    int issued = 0;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % S;
      if (kb >= S && !mbar_wait(&empty[s], ((kb / S) - 1) & 1)) {
        *s_fail = 1;
        break;
      }
      mbar_expect_tx(&full[s], bytes);
      const int k0 = kb * kTcBK;
      if (args.a_batched) {
        tma_load_3d(a_hi_s(s), &map_a_hi, &full[s], k0, (int)m0, (int)b);
        if (SPLIT) tma_load_3d(a_lo_s(s), &map_a_lo, &full[s], k0, (int)m0, (int)b);
      } else {
        tma_load_2d(a_hi_s(s), &map_a_hi, &full[s], k0, (int)m0);
        if (SPLIT) tma_load_2d(a_lo_s(s), &map_a_lo, &full[s], k0, (int)m0);
      }
      tma_load_2d(b_hi_s(s), &map_b_hi, &full[s], k0, (int)n0);
      if (SPLIT) tma_load_2d(b_lo_s(s), &map_b_lo, &full[s], k0, (int)n0);
      issued = kb + 1;
    }
    // drain: the last copy issued into each stage has landed before this CTA can leave
    for (int kb = issued - S > 0 ? issued - S : 0; kb < issued; ++kb)
      if (!mbar_wait(&full[kb % S], (kb / S) & 1)) *s_fail = 1;
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer ----
    constexpr uint32_t idesc = idesc_bf16(kTcBM, BN);
    bool ok = true;
    for (int kb = 0; kb < nkb && ok; ++kb) {
      const int s = kb % S;
      if (!mbar_wait(&full[s], (kb / S) & 1)) {
        *s_fail = 1;
        ok = false;
        break;
      }
      tc_fence_after();
      const uint64_t ah = sw128_desc(smem_addr(a_hi_s(s))), bh = sw128_desc(smem_addr(b_hi_s(s)));
      const uint64_t al = sw128_desc(smem_addr(a_lo_s(s))), bl = sw128_desc(smem_addr(b_lo_s(s)));
#pragma unroll
      for (int kk = 0; kk < kTcBK / 16; ++kk) {
        const uint64_t adv = (uint64_t)((kk * 32) >> 4);  // 16 BF16 = 32 bytes along the swizzled row
        umma_bf16(tmem, ah + adv, bh + adv, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
        if (SPLIT) {
          umma_bf16(tmem, ah + adv, bl + adv, idesc, 1u);
          umma_bf16(tmem, al + adv, bh + adv, idesc, 1u);
        }
      }
      umma_commit(&empty[s]);
    }
    umma_commit(accum);  // arrives once every MMA issued above has completed
  }
  __syncwarp();

  // ---- epilogue: all four warps, one accumulator lane (= tile row) per thread ----
  const bool got = mbar_wait(accum, 0);
  tc_fence_after();
  __syncthreads();
  const bool failed = !got || *s_fail != 0;
  const int64_t row = m0 + warp * 32 + lane;
  const bool row_ok = row < args.M;
  float* outb = args.out + b * args.s_b + row * args.s_m;
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 16) {
    float v[16];
    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    if (!row_ok) continue;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int64_t n = n0 + c0 + j;
      if (n < args.N) {
        float* p = outb + n * args.s_n;
        float y = failed ? __int_as_float(0x7fc00000) : args.alpha * v[j];
        if (!failed && args.beta != 0.f) y += args.beta * *p;
        *p = y;
      }
    }
  }
  if (failed && threadIdx.x == 0) atomicExch(args.err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols) : "memory");
  }
}

// ---------------------------------------------------------------------------------------------
// FP32 -> BF16 (hi, lo) operand passes

// Non-transposed: rows x cols of a row-major source (row stride ld) -> dst rows x K_pad.
__global__ void k_split_rows(const float* __restrict__ src, int64_t rows, int64_t cols, int64_t ld,
                             __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t kpad,
                             const int* skip) {
  if (skip && *skip) return;
  const int64_t total = rows * kpad;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = u / kpad, c = u - r * kpad;
    const float v = c < cols ? src[r * ld + c] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi[u] = h;
    if (lo) lo[u] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}
__global__ void k_split_rows_bf16(const __nv_bfloat16* __restrict__ src, int64_t rows, int64_t cols, int64_t ld,
                                  __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t kpad,
                                  const int* skip) {
  if (skip && *skip) return;
  const int64_t total = rows * kpad;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = u / kpad, c = u - r * kpad;
    hi[u] = c < cols ? src[r * ld + c] : __float2bfloat16_rn(0.f);
    if (lo) lo[u] = __float2bfloat16_rn(0.f);
  }
}

// Transposed per batch: src[b][k][m] (k stride M, batch stride K*M) -> dst[b][m][k] (row stride K_pad),
// 32 x 32 tiles through shared memory.
__global__ void __launch_bounds__(256) k_split_transpose(const float* __restrict__ src, int64_t M, int64_t K,
                                                         __nv_bfloat16* __restrict__ hi,
                                                         __nv_bfloat16* __restrict__ lo, int64_t kpad,
                                                         const int* skip) {
  if (skip && *skip) return;
  __shared__ float t[32][33];
  const int64_t b = blockIdx.z;
  const int64_t m0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 32;
  const float* s = src + b * K * M;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int64_t k = k0 + ty + j, m = m0 + tx;
    t[ty + j][tx] = (k < K && m < M) ? s[k * M + m] : 0.f;
  }
  __syncthreads();
  __nv_bfloat16* h = hi + b * M * kpad;
  __nv_bfloat16* l = lo ? lo + b * M * kpad : nullptr;
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int64_t m = m0 + ty + j, k = k0 + tx;
    if (m < M && k < kpad) {
      const float v = t[tx][ty + j];
      const __nv_bfloat16 hv = __float2bfloat16_rn(v);
      h[m * kpad + k] = hv;
      if (l) l[m * kpad + k] = __float2bfloat16_rn(v - __bfloat162float(hv));
    }
  }
}

// ---------------------------------------------------------------------------------------------
// host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    cudaGetLastError();
  });
  return fn;
}

// BF16 K-major operand map: dims (K_pad, rows[, batch]) with the 128-byte swizzle, box (64, box_rows[, 1]).
static int make_map(CUtensorMap* map, const void* ptr, int64_t kpad, int64_t rows, int64_t batch, int box_rows) {
  auto enc = encode_fn();
  if (!enc) return fail(COLAGB_ERR_UNSUPPORTED, "tensor-core contraction: cuTensorMapEncodeTiled unavailable");
  if (((uintptr_t)ptr % 16) != 0 || (kpad * 2) % 16 != 0)
    return fail(COLAGB_ERR_INVALID, "tensor-core contraction: operand not 16-byte aligned");
  const cuuint32_t rank = batch > 1 ? 3 : 2;
  cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rows, (cuuint64_t)(batch > 1 ? batch : 1)};
  cuuint64_t strides[2] = {(cuuint64_t)(kpad * 2), (cuuint64_t)(kpad * 2 * rows)};
  cuuint32_t box[3] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, const_cast<void*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(COLAGB_ERR_CUDA, "tensor-core contraction: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return COLAGB_OK;
}

template <int BN, bool SPLIT>
static int launch_tc(const CUtensorMap* maps, const TcArgs& a, cudaStream_t st) {
  using Cfg = TcCfg<BN, SPLIT>;
  static_assert(Cfg::kStages >= 2, "at least two pipeline stages");
  COLAGB_CUDA(cudaFuncSetAttribute(k_tc_gemm<BN, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem));
  dim3 grid((unsigned)ceil_div(a.M, kTcBM), (unsigned)ceil_div(a.N, BN), (unsigned)a.batch);
  k_tc_gemm<BN, SPLIT><<<grid, kTcThreads, Cfg::kSmem, st>>>(maps[0], maps[1], maps[2], maps[3], a);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

bool tc_contract_supported(int64_t batch, int64_t M, int64_t N, int64_t K) {
  return batch >= 1 && batch <= 65535 && M >= 1 && N >= 1 && K >= 8 && M <= (int64_t)1 << 31 && N <= 65535 * 64 &&
         ceil_div(M, kTcBM) <= 2147483647LL;
}

// out[b * s_b + m * s_m + n * s_n] = alpha * sum_k A_b[m, k] B[n, k] + beta * out[...], where
//   transposed_a: A_b[m, k] = a_src[b * K * M + k * M + m]   (the Kronecker operand with q = M > 1)
//   otherwise:    A[m, k]   = a_src[m * K + k]               (batch must be 1)
// and B[n, k] = b_src[n * ldb + k] (FP32 or BF16 storage).  Scratch comes from `ws`.
int tc_contract(const float* a_src, bool transposed_a, int64_t batch, int64_t M, int64_t K, const void* b_src,
                int32_t b_dtype, int64_t ldb, int64_t N, float* out, int64_t s_b, int64_t s_m, int64_t s_n,
                float alpha, float beta, bool split, Bump& ws, const int* skip, cudaStream_t st) {
  const int64_t kpad = (K + 7) / 8 * 8;
  __nv_bfloat16* a_hi = ws.take<__nv_bfloat16>((size_t)(batch * M * kpad));
  __nv_bfloat16* b_hi = ws.take<__nv_bfloat16>((size_t)(N * kpad));
  __nv_bfloat16* a_lo = split ? ws.take<__nv_bfloat16>((size_t)(batch * M * kpad)) : nullptr;
  __nv_bfloat16* b_lo = split ? ws.take<__nv_bfloat16>((size_t)(N * kpad)) : nullptr;
  int* err = ws.take<int>(1);
  if (ws.measure) return COLAGB_OK;
  if (!transposed_a && batch != 1) return fail(COLAGB_ERR_INVALID, "tensor-core contraction: batch with row operand");
  // operand passes
  {
    const int64_t tot = N * kpad;
    const int g = (int)std::min<int64_t>(ceil_div(tot, 256), (int64_t)num_sms() * 8);
    if (b_dtype == COLAGB_BF16)
      k_split_rows_bf16<<<g, 256, 0, st>>>(static_cast<const __nv_bfloat16*>(b_src), N, K, ldb, b_hi, b_lo, kpad,
                                           skip);
    else
      k_split_rows<<<g, 256, 0, st>>>(static_cast<const float*>(b_src), N, K, ldb, b_hi, b_lo, kpad, skip);
    COLAGB_CUDA(cudaGetLastError());
  }
  if (transposed_a) {
    dim3 grid((unsigned)ceil_div(M, 32), (unsigned)ceil_div(kpad, 32), (unsigned)batch);
    k_split_transpose<<<grid, 256, 0, st>>>(a_src, M, K, a_hi, a_lo, kpad, skip);
  } else {
    const int64_t tot = M * kpad;
    const int g = (int)std::min<int64_t>(ceil_div(tot, 256), (int64_t)num_sms() * 8);
    k_split_rows<<<g, 256, 0, st>>>(a_src, M, K, K, a_hi, a_lo, kpad, skip);
  }
  COLAGB_CUDA(cudaGetLastError());
  COLAGB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  // tile width: the widest of 256 / 128 / 64 columns that still gives every SM a tile
  int bn = 64;
  const int64_t mt = ceil_div(M, kTcBM) * batch;
  if (N >= 256 && mt * ceil_div(N, 256) >= num_sms()) bn = 256;
  else if (N >= 128 && mt * ceil_div(N, 128) >= num_sms()) bn = 128;
  if (split && bn == 256) bn = 128;
  CUtensorMap maps[4];
  COLAGB_TRY(make_map(&maps[0], a_hi, kpad, M, batch, kTcBM));
  COLAGB_TRY(make_map(&maps[1], split ? a_lo : a_hi, kpad, M, batch, kTcBM));
  COLAGB_TRY(make_map(&maps[2], b_hi, kpad, N, 1, bn));
  COLAGB_TRY(make_map(&maps[3], split ? b_lo : b_hi, kpad, N, 1, bn));
  TcArgs a;
  a.M = M;
  a.N = N;
  a.K = kpad;
  a.batch = batch;
  a.out = out;
  a.s_b = s_b;
  a.s_m = s_m;
  a.s_n = s_n;
  a.alpha = alpha;
  a.beta = beta;
  a.a_batched = batch > 1 ? 1 : 0;
  a.err = err;
  a.skip = skip;
  if (split) {
    if (bn == 64) return launch_tc<64, true>(maps, a, st);
    return launch_tc<128, true>(maps, a, st);
  }
  if (bn == 64) return launch_tc<64, false>(maps, a, st);
  if (bn == 128) return launch_tc<128, false>(maps, a, st);
  return launch_tc<256, false>(maps, a, st);
}

}  // namespace colagb
